"""Generate the mean-field TEMPO fixture by running the unmodified OQuPy
reference (``oqupy.MeanFieldTempo``) on the cases of
``tests/mean_field_cases.py``.

Run from the repository root, where the reference sources are present:

    python tests/golden/make_mean_field.py <OQuPy source tree>

``tensornetwork`` comes from the stand-in in ``oracle/tnshim``.  The systems
are built with ``TempoParameters(subdiv_limit=None)``, so the reference's
propagators are the sampled-Liouvillian ones that ``mean_field_cases``
restates.  Recorded per case: the influence matrices and coupling eigenbasis
of every system (the inputs the backends consume), every system's density
matrix and the field after every step, and the trace-distance envelope of
the reference rerun with its initial states and field perturbed by 1e-15
relative (two seeds).  As a check of the stand-in, case G is also run with
the reference's default parameters and compared with the known answer stored
in the reference's tests/physics/mean_field_tempo_test.py (4 decimals).
The reference wraps field-dependent Hamiltonians in ``np.vectorize``, which
numpy 2.5 no longer allows for matrix-valued functions of scalars;
``mean_field_cases.patch_field_hamiltonian_check`` replaces that wrapper by
a direct call (the numbers the Hamiltonian returns are unchanged).
"""

import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests import mean_field_cases as mfc  # noqa: E402

sys.path.insert(0, HERE)
from make_golden import _perturbed  # noqa: E402


def _import_reference(ref_root):
    sys.path[:0] = [os.path.join(ROOT, "oracle", "tnshim"), ref_root]
    warnings.simplefilter("ignore")
    import oqupy  # noqa: E402
    oqupy.config.PROGRESS_TYPE = "silent"
    mfc.patch_field_hamiltonian_check(oqupy)
    return oqupy


def build(oqupy, case, subdiv_limit=None, rho_pert=None, field_pert=0.0):
    systems, baths, rho0 = [], [], []
    for k, s in enumerate(case["systems"]):
        gam = [(lambda t, g=g: g) for g in s["gammas"]]
        lops = [(lambda t, a=a: a) for a in s["lops"]]
        systems.append(oqupy.TimeDependentSystemWithField(s["h"], gammas=gam, lindblad_operators=lops))
        corr = oqupy.PowerLawSD(alpha=s["alpha"], zeta=s["zeta"], cutoff=s["wc"],
                                cutoff_type=s["cutoff_type"], temperature=s["T"])
        baths.append(oqupy.Bath(s["coupling"], corr))
        r = np.array(s["rho0"], dtype=np.complex128)
        if rho_pert is not None:
            r = r * (1.0 + rho_pert[k])
        rho0.append(r)
    mfs = oqupy.MeanFieldSystem(systems, field_eom=case["field_eom"])
    kw = {} if subdiv_limit == "default" else {"subdiv_limit": subdiv_limit}
    params = oqupy.TempoParameters(dt=case["dt"], tcut=case["tcut"], epsrel=case["epsrel"], **kw)
    mft = oqupy.MeanFieldTempo(mfs, baths, params, rho0, case["field0"] * (1.0 + field_pert),
                               start_time=0.0)
    return mft, baths, params


def run(oqupy, case, **kw):
    mft, baths, params = build(oqupy, case, **kw)
    dyn = mft.compute(end_time=(case["nsteps"] + 0.5) * case["dt"])
    states = np.array([[np.asarray(m).reshape(-1) for m in sd.states] for sd in dyn.system_dynamics])
    return states, np.array(dyn.fields, dtype=np.complex128), mft, baths, params


def trace_distance(a, b):
    d = int(round(np.sqrt(a.size)))
    return 0.5 * np.abs(np.linalg.eigvalsh((a - b).reshape(d, d))).sum()


def main(ref_root):
    oqupy = _import_reference(ref_root)
    out = {}
    for name, case in mfc.CASES.items():
        states, fields, mft, baths, params = run(oqupy, case)
        n_sys = len(case["systems"])
        nsteps = case["nsteps"]
        assert states.shape[1] == nsteps + 1, states.shape
        be = mft._backend_instance
        dkmax = params.dkmax
        ninfl = nsteps + 1 if dkmax is None else dkmax + 1
        for i in range(n_sys):
            infl = be._backend_list[i]._influence
            out[f"{name}/influences{i}"] = np.array([infl(dk) for dk in range(ninfl)])
            out[f"{name}/unitary{i}"] = np.asarray(baths[i].unitary_transform, dtype=np.complex128)
        out[f"{name}/dkmax"] = np.int64(-1 if dkmax is None else dkmax)
        out[f"{name}/states"] = states
        out[f"{name}/fields"] = fields
        env = np.zeros((n_sys, nsteps + 1))
        fenv = np.zeros(nsteps + 1)
        for seed in (1, 2):
            rng = np.random.default_rng(seed)
            st2, f2, *_ = run(oqupy, case, rho_pert=1e-15 * rng.standard_normal(n_sys),
                              field_pert=1e-15 * rng.standard_normal())
            for i in range(n_sys):
                env[i] = np.maximum(env[i], [trace_distance(a, b) for a, b in zip(states[i], st2[i])])
            fenv = np.maximum(fenv, np.abs(fields - f2))
        out[f"{name}/envelope"] = env
        out[f"{name}/field_envelope"] = fenv
        print(f"{name}: {n_sys} systems, {nsteps} steps, dkmax {dkmax}, final field {fields[-1]:.6f}, "
              f"envelope {env.max():.1e} (field {fenv.max():.1e})")
    # the same models on process tensors: compute_dynamics_with_field
    # (system_dynamics.py:184-476), one process tensor per system's bath
    for name, case in mfc.CASES.items():
        mft, baths, params = build(oqupy, case)
        mfs = oqupy.MeanFieldSystem(
            [oqupy.TimeDependentSystemWithField(
                s["h"], gammas=[(lambda t, g=g: g) for g in s["gammas"]],
                lindblad_operators=[(lambda t, a=a: a) for a in s["lops"]]) for s in case["systems"]],
            field_eom=case["field_eom"])
        end_time = case["nsteps"] * case["dt"]
        pts = []
        for i, bath in enumerate(baths):
            ptt = oqupy.PtTempo(bath, 0.0, end_time, params)
            pt = ptt.get_process_tensor(progress_type="silent")
            pts.append(pt)
            kmax = ptt._backend_instance._num_infl
            out[f"{name}/pt_influences{i}"] = np.array([ptt._influence(dk) for dk in range(kmax)])
            out[f"{name}/pt_dkmax{i}"] = np.int64(ptt._backend_instance._dkmax
                                                   if ptt._backend_instance._dkmax is not None else -1)
            if pt.transform_in is not None:
                out[f"{name}/pt_transform_in{i}"] = np.asarray(pt.transform_in)
                out[f"{name}/pt_transform_out{i}"] = np.asarray(pt.transform_out)
        def run_pt(pts):
            dyn = oqupy.compute_dynamics_with_field(
                mfs, initial_field=case["field0"], process_tensor_list=pts,
                initial_state_list=[np.asarray(s["rho0"]) for s in case["systems"]],
                start_time=0.0, subdiv_limit=None, progress_type="silent")
            st = np.array([[np.asarray(m).reshape(-1) for m in sd.states] for sd in dyn.system_dynamics])
            return st, np.array(dyn.fields, dtype=np.complex128)
        st, fl = run_pt(pts)
        out[f"{name}/pt_states"] = st
        out[f"{name}/pt_fields"] = fl
        # spread: the process tensors rebuilt with influences perturbed by
        # 1e-15 relative (two seeds)
        env = np.zeros(st.shape[:2])
        fenv = np.zeros(len(fl))
        for seed in (1, 2):
            pts2 = []
            for bath in baths:
                p2 = oqupy.PtTempo(bath, 0.0, end_time, params)
                p2._backend_instance._influence = _perturbed(p2._backend_instance._influence, seed)
                pts2.append(p2.get_process_tensor(progress_type="silent"))
            st2, fl2 = run_pt(pts2)
            for i in range(st.shape[0]):
                env[i] = np.maximum(env[i], [trace_distance(a, b) for a, b in zip(st[i], st2[i])])
            fenv = np.maximum(fenv, np.abs(fl - fl2))
        out[f"{name}/pt_envelope"] = env
        out[f"{name}/pt_field_envelope"] = fenv
        print(f"{name} on process tensors: {st.shape[1] - 1} steps, final field {fl[-1]:.6f}, "
              f"vs TEMPO {out[name + '/fields'][-1]:.6f}, envelope {env.max():.1e}")
    # the reference's own known answer for case G (default parameters)
    st, f, *_ = run(oqupy, mfc.CASES["dicke_G"], subdiv_limit="default")
    rho_g = np.array([[0.6245009 + 3.19373236e-15j, 0.14243496 - 2.19523032e-01j],
                      [0.14243496 + 2.19523032e-01j, 0.3754991 - 2.26692588e-15j]])
    field_g = 0.10602369935009 - 0.46986388684474406j
    np.testing.assert_almost_equal(f[-1], field_g, decimal=4)
    np.testing.assert_almost_equal(st[0, -1].reshape(2, 2), rho_g, decimal=4)
    print("case G with default parameters reproduces the reference test's known answer")
    np.savez_compressed(os.path.join(HERE, "mean_field.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit(__doc__)
    main(sys.argv[1])
