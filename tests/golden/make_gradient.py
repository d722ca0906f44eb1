"""Generate the gradient fixture by running the unmodified OQuPy reference's
``compute_gradient_and_dynamics`` (oqupy/gradient.py:169-437) on process
tensors it builds itself.

Run from the repository root, where the reference sources are present:

    python tests/golden/make_gradient.py <OQuPy source tree>

``tensornetwork`` comes from the stand-in in ``oracle/tnshim``.  The system
is a ``ParameterizedSystem`` (H = hx sigma_x + hz sigma_z, a decay channel)
with seeded parameters for every half step; its propagators are recorded as
the inputs the backends consume.  Two runs per case: without and with a
control (a pre-measurement operation at one step and a post-measurement one
at another).  Recorded: the process tensor's inputs (influences, memory,
epsrel, transforms), the per-step propagators, the target, the control
operations, the reference's derivative tensors (one D x D x D x D tensor per
step) and states, and the largest change of each under a rebuild of the
process tensor with its influences perturbed by 1e-15 relative (two seeds)
or with LAPACK gesvd in the SVDs.  The reference keeps the Hamiltonian
wrapped in ``np.vectorize`` (system.py:530), which numpy 2.5 no longer
allows for matrix-valued functions: the script replaces the wrapper by the
callable itself (no number changes).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden import _import_reference, _perturbed  # noqa: E402
from tests.reference_compat import patch_vectorize_checks  # noqa: E402


def cases(oqupy):
    sx, sz, sm = oqupy.operators.sigma("x"), oqupy.operators.sigma("z"), oqupy.operators.sigma("-")
    yield "grad_nondiag", dict(
        coupling=0.5 * sx, alpha=0.15, wc=3.0, cutoff_type="exponential", T=0.5,
        dt=0.1, dkmax=6, epsrel=1e-7, nsteps=14, d=2,
        h=lambda hx, hz: hx * sx + hz * sz, gammas=[lambda hx, hz: 0.1], lops=[lambda hx, hz: sm],
        rho0=oqupy.operators.spin_dm("up"), target=oqupy.operators.spin_dm("down").T,
        control=[(4, oqupy.operators.left_super(sz), False),
                 (9, oqupy.operators.right_super(sx), True)])
    yield "grad_diag", dict(
        coupling=0.5 * sz, alpha=0.3, wc=5.0, cutoff_type="exponential", T=0.2,
        dt=0.05, dkmax=8, epsrel=1e-7, nsteps=16, d=2,
        h=lambda hx, hz: hx * sx + hz * sz, gammas=[], lops=[],
        rho0=np.array([[0.7, 0.2 - 0.1j], [0.2 + 0.1j, 0.3]]), target=sx.T,
        control=[(6, oqupy.operators.left_super(sx), False)])


def run(oqupy, c, pt, params, with_control):
    ps = oqupy.ParameterizedSystem(c["h"], gammas=c["gammas"], lindblad_operators=c["lops"])
    ps._hamiltonian = c["h"]          # see the module docstring
    ctrl = None
    if with_control:
        ctrl = oqupy.Control(c["d"])
        for step, op, post in c["control"]:
            ctrl.add_single(step, op, post=post)
    derivs, dyn = oqupy.gradient.compute_gradient_and_dynamics(
        system=ps, initial_state=c["rho0"], target_derivative=c["target"],
        process_tensors=[pt], parameters=params, dt=c["dt"], num_steps=c["nsteps"],
        control=ctrl, progress_type="silent")
    props = ps.get_propagators(c["dt"], params)
    # the reference returns the last step's tensor as a node (gradient.py:382)
    return (np.array([np.asarray(getattr(x, "tensor", x)) for x in derivs]),
            np.array(dyn.states).reshape(len(dyn.states), -1), props)


def main(ref_root):
    oqupy = _import_reference(ref_root)
    patch_vectorize_checks(oqupy)
    import oqupy.gradient  # noqa: F401
    res = {}
    for name, c in cases(oqupy):
        corr = oqupy.PowerLawSD(alpha=c["alpha"], zeta=1.0, cutoff=c["wc"],
                                cutoff_type=c["cutoff_type"], temperature=c["T"])
        bath = oqupy.Bath(c["coupling"], corr)
        params_t = oqupy.TempoParameters(dt=c["dt"], dkmax=c["dkmax"], epsrel=c["epsrel"])
        end_time = c["nsteps"] * c["dt"]
        ptt = oqupy.PtTempo(bath, 0.0, end_time, params_t)
        pt = ptt.get_process_tensor(progress_type="silent")
        assert len(pt) == c["nsteps"]
        kmax = ptt._backend_instance._num_infl
        res[f"{name}/influences"] = np.array([ptt._influence(dk) for dk in range(kmax)])
        for key in ("dkmax", "nsteps", "d"):
            res[f"{name}/{key}"] = np.int64(c[key])
        res[f"{name}/epsrel"] = np.float64(c["epsrel"])
        res[f"{name}/rho0"] = np.asarray(c["rho0"], dtype=np.complex128).reshape(-1)
        res[f"{name}/target"] = np.asarray(c["target"], dtype=np.complex128).reshape(-1)
        if pt.transform_in is not None:
            res[f"{name}/transform_in"] = np.asarray(pt.transform_in)
            res[f"{name}/transform_out"] = np.asarray(pt.transform_out)
        rng = np.random.default_rng(42)
        params = rng.uniform(-1.0, 1.0, size=(2 * c["nsteps"], 2))
        res[f"{name}/control_steps"] = np.array([s for s, _, _ in c["control"]])
        res[f"{name}/control_ops"] = np.array([op for _, op, _ in c["control"]], dtype=np.complex128)
        res[f"{name}/control_post"] = np.array([p for _, _, p in c["control"]])
        for tag, wc in (("plain", False), ("control", True)):
            derivs, states, props = run(oqupy, c, pt, params, wc)
            res[f"{name}/{tag}_derivs"] = derivs
            res[f"{name}/{tag}_states"] = states
            pp = [props(k) for k in range(c["nsteps"])]
            res[f"{name}/prop1"] = np.array([p[0] for p in pp])
            res[f"{name}/prop2"] = np.array([p[1] for p in pp])
            env_d = np.zeros(len(derivs))
            env_s = np.zeros(len(states))
            for seed in (1, 2, "gesvd"):
                p2t = oqupy.PtTempo(bath, 0.0, end_time, params_t)
                if seed == "gesvd":
                    os.environ["OQUPY_TNSHIM_SVD"] = "gesvd"
                else:
                    p2t._backend_instance._influence = _perturbed(p2t._backend_instance._influence, seed)
                try:
                    pt2 = p2t.get_process_tensor(progress_type="silent")
                finally:
                    os.environ.pop("OQUPY_TNSHIM_SVD", None)
                d2, s2, _ = run(oqupy, c, pt2, params, wc)
                env_d = np.maximum(env_d, np.abs(d2 - derivs).reshape(len(derivs), -1).max(axis=1))
                env_s = np.maximum(env_s, np.abs(s2 - states).max(axis=1))
            res[f"{name}/{tag}_derivs_envelope"] = env_d
            res[f"{name}/{tag}_states_envelope"] = env_s
            print(name, tag, "derivs", derivs.shape, "max |deriv|", float(np.abs(derivs).max()),
                  "envelope", float(env_d.max()), float(env_s.max()))
    np.savez_compressed(os.path.join(HERE, "gradient.npz"), **res)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit(__doc__)
    main(sys.argv[1])
