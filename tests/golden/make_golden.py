"""Generate golden fixtures by running the unmodified OQuPy reference.

Run from the repository root, in a container where the reference sources are
present (it cannot run on a machine without them):

    python tests/golden/make_golden.py <OQuPy source tree> [case ...]

The reference imports the third-party ``tensornetwork`` package, which is not
installed here; ``oracle/tnshim`` provides a from-scratch stand-in for the few
calls on this path.  For every case the script records the exact inputs the
reference backend consumed (influence matrices per ``dk``, half-step
propagators, coupling unitary, initial state) and the reference's outputs
(density matrix per step, bond dimensions), so the oracle and the CUDA path
can be run on bit-identical inputs.  Each case also records a per-step
rounding envelope: how far the unmodified reference itself moves when its
inputs are perturbed by 1e-15 relative (two seeds) or when its SVD calls use
LAPACK gesvd instead of gesdd.  Process tensors are gauge dependent and
are not stored; their bond dimensions and the dynamics computed from them are.
"""

import os
import sys
import time
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _import_reference(ref_root):
    sys.path[:0] = [os.path.join(ROOT, "oracle", "tnshim"), ref_root]
    warnings.simplefilter("ignore")
    import oqupy  # noqa: E402
    oqupy.config.PROGRESS_TYPE = "silent"
    return oqupy


def _gue(d, rng):
    a = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    h = 0.5 * (a + a.conj().T)
    return h / np.linalg.norm(h, 2)


def cases(oqupy):
    """Yield ``(name, dict)`` case descriptions."""
    sx = oqupy.operators.sigma("x")
    sz = oqupy.operators.sigma("z")
    sm = oqupy.operators.sigma("-")
    up = oqupy.operators.spin_dm("up")
    rng = np.random.default_rng(1234)
    # plain TEMPO spin-boson (alpha 0.08, wc 4, T 0, dkmax 20, 100 steps)
    yield "config1_spin_boson", dict(
        h=0.5 * 1.0 * sx, gammas=[], lops=[], coupling=0.5 * sz,
        alpha=0.08, zeta=1.0, wc=4.0, cutoff_type="exponential", T=0.0,
        dt=0.05, dkmax=20, epsrel=1e-6, nsteps=100, rho0=up,
        add_corr=None, tempo=True, pt=False)
    # reference tests/physics/tempo_spin_boson_test.py case A (full memory)
    yield "ref_spin_boson_A", dict(
        h=np.array([[0.0, 0.5], [0.5, 0.0]]), gammas=[0.1, 0.2],
        lops=[sm, sz], coupling=np.array([[0.5, 0.0], [0.0, -0.5]]),
        alpha=0.3, zeta=1.0, wc=5.0, cutoff_type="exponential", T=0.2,
        dt=0.05, dkmax=None, epsrel=1e-7, nsteps=20,
        rho0=np.array([[1.0, 0.0], [0.0, 0.0]]), add_corr=None,
        tempo=True, pt=True)
    # reference tests/physics/tempo_qutrit_test.py case C
    hC = np.array([[1.0, 0.0, 0.0], [0.0, 0.5, 0.0], [0.0, 0.0, 0.0]]) \
        + np.array([[0.0, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.0]])
    yield "ref_qutrit_C", dict(
        h=hC, gammas=[0.1, 0.2],
        lops=[np.array([[0.0, 0, 0], [0, 0, 0], [0, 1.0, 0]]),
              np.array([[0.5, 0, 0], [0, -0.5, 0], [0, 0, 0]])],
        coupling=np.array([[0.5, 0, 0], [0, -0.5, 0], [0, 0, 0.0]]),
        alpha=0.3, zeta=1.0, wc=5.0, cutoff_type="exponential", T=0.0,
        dt=0.05, dkmax=10, epsrel=1e-7, nsteps=20,
        rho0=np.array([[0.0, 0, 0], [0, 1.0, 0], [0, 0, 0]]),
        add_corr=None, tempo=True, pt=True)
    # non-diagonal coupling: exercises the eigenbasis transforms
    yield "nondiag_coupling", dict(
        h=0.5 * sz + 0.3 * sx, gammas=[], lops=[], coupling=0.5 * sx,
        alpha=0.15, zeta=1.0, wc=3.0, cutoff_type="exponential", T=0.5,
        dt=0.1, dkmax=6, epsrel=1e-7, nsteps=18, rho0=up, add_corr=None,
        tempo=True, pt=True)
    # add_correlation_time (negative-dk rectangle influences)
    yield "add_corr_time", dict(
        h=0.5 * sx, gammas=[], lops=[], coupling=0.5 * sz,
        alpha=0.2, zeta=1.0, wc=4.0, cutoff_type="gaussian", T=0.3,
        dt=0.1, dkmax=4, epsrel=1e-7, nsteps=14, rho0=up, add_corr=0.25,
        tempo=True, pt=True)
    # strongly coupled, hot instance of the batched spin-boson distribution
    yield "batched_like_hot", dict(
        h=0.5 * 1.5 * sx, gammas=[], lops=[], coupling=0.5 * sz,
        alpha=0.4, zeta=1.0, wc=8.0, cutoff_type="exponential", T=3.0,
        dt=0.05, dkmax=30, epsrel=1e-6, nsteps=60, rho0=up, add_corr=None,
        tempo=True, pt=False)
    # qutrit, super-ohmic bath, GUE Hamiltonian (batched-qutrit distribution)
    yield "qutrit_superohmic", dict(
        h=_gue(3, rng), gammas=[], lops=[],
        coupling=np.diag([1.0, 0.0, -1.0]), alpha=0.12, zeta=3.0, wc=3.0,
        cutoff_type="exponential", T=1.0, dt=0.05, dkmax=10, epsrel=1e-7,
        nsteps=30, rho0=np.diag([1.0, 0.0, 0.0]).astype(complex),
        add_corr=None, tempo=True, pt=True)
    # PT build of the alpha 0.3 / epsrel 1e-7 model (reduced memory and length) + dynamics
    hs = []
    for _ in range(3):
        a, b = rng.uniform(-2, 2, size=2)
        hs.append(a * sx + b * sz)
    yield "pt_config2_small", dict(
        h=hs[0], h_list=hs, gammas=[], lops=[], coupling=0.5 * sz,
        alpha=0.3, zeta=1.0, wc=5.0, cutoff_type="exponential", T=1.0,
        dt=0.02, dkmax=20, epsrel=1e-7, nsteps=50, rho0=up, add_corr=None,
        tempo=False, pt=True)


def _perturbed(influence, seed, rel=1e-15):
    """Wrap ``influence(dk)`` so each matrix is multiplied element-wise by
    ``1 + rel * N(0, 1)`` (a few ulp): used to measure how far the reference's
    own result moves under rounding-level changes of its inputs."""
    rng = np.random.default_rng(seed)
    cache = {}

    def f(dk):
        m = influence(dk)
        if m is None:
            return None
        if dk not in cache:
            cache[dk] = 1.0 + rel * rng.normal(size=m.shape)
        return m * cache[dk]
    return f


def _trace_dist(a, b):
    d = int(round(np.sqrt(a.size)))
    diff = (a - b).reshape(d, d)
    herm = 0.5 * (diff + diff.conj().T)
    return 0.5 * np.sum(np.abs(np.linalg.eigvalsh(herm)))


def run_case(oqupy, name, c):
    corr = oqupy.PowerLawSD(alpha=c["alpha"], zeta=c["zeta"], cutoff=c["wc"],
                            cutoff_type=c["cutoff_type"], temperature=c["T"])
    bath = oqupy.Bath(c["coupling"], corr)
    params = oqupy.TempoParameters(dt=c["dt"], dkmax=c["dkmax"],
                                   epsrel=c["epsrel"],
                                   add_correlation_time=c["add_corr"])
    out = {}
    d = c["rho0"].shape[0]
    nsteps = c["nsteps"]
    end_time = nsteps * c["dt"]
    for key in ("alpha", "zeta", "wc", "T", "dt", "epsrel", "nsteps"):
        out[key] = np.array(c[key])
    out["dkmax"] = np.array(-1 if c["dkmax"] is None else c["dkmax"])
    out["add_corr"] = np.array(-1.0 if c["add_corr"] is None
                               else c["add_corr"])
    out["cutoff_type"] = np.array(c["cutoff_type"])
    out["rho0"] = np.asarray(c["rho0"], dtype=complex)
    out["coupling"] = np.asarray(c["coupling"], dtype=complex)
    out["unitary"] = bath.unitary_transform.astype(complex)
    out["comm"] = bath.coupling_comm
    out["acomm"] = bath.coupling_acomm
    systems = [c["h"]] + list(c.get("h_list", [])[1:])
    sys_objs = [oqupy.System(h, gammas=c["gammas"],
                             lindblad_operators=c["lops"]) for h in systems]
    props = [s.get_propagators(c["dt"], 0.0, None, None)(0) for s in sys_objs]
    out["prop1"] = np.array([p[0] for p in props])
    out["prop2"] = np.array([p[1] for p in props])
    if c["tempo"]:
        t0 = time.time()
        tempo = oqupy.Tempo(sys_objs[0], bath, params, c["rho0"], 0.0)
        be = tempo._backend_instance
        bonds = []
        orig = be.compute_step

        def hooked():
            r = orig()
            bonds.append(list(be._mps.bond_dimensions))
            return r
        be.compute_step = hooked
        dyn = tempo.compute(end_time, progress_type="silent")
        out["tempo_time_s"] = np.array(time.time() - t0)
        out["tempo_states"] = np.array(dyn.states).reshape(-1, d * d)
        out["tempo_times"] = np.array(dyn.times)
        out["tempo_max_bond"] = np.array([max(b) if b else 1 for b in bonds])
        out["tempo_final_bonds"] = np.array(bonds[-1])
        kmax = nsteps if c["dkmax"] is None else c["dkmax"]
        infl = [tempo._influence(dk) for dk in range(kmax + 1)]
        out["tempo_infl"] = np.array(infl)
        if c["dkmax"] is not None and c["add_corr"] is not None:
            neg = [tempo._influence(c["dkmax"] - s)
                   for s in range(c["dkmax"] + 1, nsteps + 1)]
            out["tempo_infl_neg"] = np.array(neg)
        env = np.zeros(nsteps + 1)
        for seed in (1, 2, "gesvd"):
            t2 = oqupy.Tempo(sys_objs[0], bath, params, c["rho0"], 0.0)
            if seed == "gesvd":
                os.environ["OQUPY_TNSHIM_SVD"] = "gesvd"
            else:
                t2._backend_instance._influence = _perturbed(
                    t2._backend_instance._influence, seed)
            try:
                dyn2 = t2.compute(end_time, progress_type="silent")
            finally:
                os.environ.pop("OQUPY_TNSHIM_SVD", None)
            st2 = np.array(dyn2.states).reshape(-1, d * d)
            env = np.maximum(env, [_trace_dist(a, b) for a, b in
                                   zip(out["tempo_states"], st2)])
        out["tempo_envelope"] = env
    if c["pt"]:
        t0 = time.time()
        ptt = oqupy.PtTempo(bath, 0.0, end_time, params)
        pt = ptt.get_process_tensor(progress_type="silent")
        out["pt_time_s"] = np.array(time.time() - t0)
        out["pt_bonds"] = np.array(pt.get_bond_dimensions())
        kmax = ptt._backend_instance._num_infl
        out["pt_infl"] = np.array([ptt._influence(dk) for dk in range(kmax)])
        if c["add_corr"] is not None:
            neg = [ptt._influence(-s) for s in range(2, nsteps + 1)]
            out["pt_infl_neg"] = np.array(neg)
        states = []
        for s in sys_objs:
            dyn = oqupy.compute_dynamics(system=s, process_tensor=pt,
                                         initial_state=c["rho0"],
                                         progress_type="silent")
            states.append(np.array(dyn.states).reshape(-1, d * d))
        out["pt_states"] = np.array(states)
        if pt.transform_in is not None:
            out["pt_transform_in"] = pt.transform_in
            out["pt_transform_out"] = pt.transform_out
        env = np.zeros(out["pt_states"].shape[:2])
        for seed in (1, 2, "gesvd"):
            p2 = oqupy.PtTempo(bath, 0.0, end_time, params)
            if seed == "gesvd":
                os.environ["OQUPY_TNSHIM_SVD"] = "gesvd"
            else:
                p2._backend_instance._influence = _perturbed(
                    p2._backend_instance._influence, seed)
            try:
                pt2 = p2.get_process_tensor(progress_type="silent")
            finally:
                os.environ.pop("OQUPY_TNSHIM_SVD", None)
            for i, s in enumerate(sys_objs):
                dyn = oqupy.compute_dynamics(system=s, process_tensor=pt2,
                                             initial_state=c["rho0"],
                                             progress_type="silent")
                st2 = np.array(dyn.states).reshape(-1, d * d)
                env[i] = np.maximum(env[i], [_trace_dist(a, b) for a, b in
                                             zip(out["pt_states"][i], st2)])
        out["pt_envelope"] = env
    return out


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_golden.py <OQuPy source tree> [case ...]")
    ref_root = sys.argv[1]
    oqupy = _import_reference(ref_root)
    only = sys.argv[2:] if len(sys.argv) > 2 else None
    for name, c in cases(oqupy):
        if only and name not in only:
            continue
        t0 = time.time()
        out = run_case(oqupy, name, c)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name}: {time.time() - t0:.1f}s", flush=True)


if __name__ == "__main__":
    main()
