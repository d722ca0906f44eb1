"""Generate the correlation / controlled-dynamics fixture by running the
unmodified OQuPy reference on process tensors it builds itself.

Run from the repository root, where the reference sources are present:

    python tests/golden/make_correlations.py <OQuPy source tree>

``tensornetwork`` comes from the stand-in in ``oracle/tnshim``.  Per case the
script records the process tensor's inputs (influence matrices, memory,
epsrel, transforms) and the reference's outputs on it:

* ``compute_correlations`` (system_dynamics.py:1011-1093), time-ordered and
  anti-time-ordered, and ``compute_correlations_nt`` with three operators
  (:791-990), together with the integer operator steps the reference parsed;
* ``compute_dynamics`` with a ``Control`` holding a pre- and a
  post-measurement operation (:131-160);
* ``compute_dynamics`` of a ``TimeDependentSystem`` (its per-step half-step
  propagators are stored as the inputs they are);

and each output's spread when the process tensor is rebuilt with its
influences perturbed by 1e-15 relative (two seeds) or with LAPACK gesvd in
the SVDs.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden import _import_reference, _perturbed, _trace_dist  # noqa: E402
from tests.reference_compat import patch_vectorize_checks  # noqa: E402


def cases(oqupy):
    sx, sy, sz = (oqupy.operators.sigma(c) for c in "xyz")
    sm, sp = oqupy.operators.sigma("-"), oqupy.operators.sigma("+")
    up = oqupy.operators.spin_dm("up")
    yield "corr_nondiag", dict(
        d=2, h=0.5 * sz + 0.3 * sx, coupling=0.5 * sx, alpha=0.15, wc=3.0,
        cutoff_type="exponential", T=0.5, dt=0.1, dkmax=6, epsrel=1e-7,
        nsteps=18, rho0=up, op_a=sm, op_b=sp,
        times_a=slice(0, 10, 3), times_b=slice(0, None), anti_a=(0.0, 0.6),
        nt_ops=[sx, sz, sy], nt_times=[[1, 4], slice(2, 8, 2), slice(0, None)],
        nt_order=["left", "right", "left"],
        control=[(3, oqupy.operators.left_super(sx), False),
                 (5, "rotation", True), (5, oqupy.operators.right_super(sz), True)],
        h_t=lambda t: 0.5 * sz + 0.3 * np.cos(2.0 * t) * sx)
    lower = np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [0.0, 0.0, 0.0]])
    yield "corr_qutrit", dict(
        d=3, h=np.diag([1.0, 0.5, 0.0]) + 0.5 * (lower + lower.T),
        coupling=np.diag([0.5, -0.5, 0.0]), alpha=0.3, wc=5.0,
        cutoff_type="exponential", T=0.0, dt=0.05, dkmax=10, epsrel=1e-7,
        nsteps=20, rho0=np.diag([0.0, 1.0, 0.0]).astype(complex),
        op_a=lower, op_b=lower.T, times_a=slice(0, 12, 4), times_b=slice(0, None),
        anti_a=(0.0, 0.4), nt_ops=[lower.T, np.diag([1.0, 0.0, -1.0]), lower],
        nt_times=[[2, 5], [5, 9], slice(0, None)], nt_order=["left", "left", "right"],
        control=[(4, oqupy.operators.left_super(np.diag([1.0, 0.0, 0.0])), False)],
        h_t=lambda t: np.diag([1.0, 0.5, 0.0]) + 0.5 * np.sin(t) * (lower + lower.T))


def control_ops(oqupy, c):
    """``(step, superoperator, post)`` of a case's control operations (the
    "rotation" entry: exp(-0.4 i sigma_y) acting as U rho U^+)."""
    ops = []
    for step, op, post in c["control"]:
        if isinstance(op, str):
            u = np.cos(0.4) * np.identity(2) - 1j * np.sin(0.4) * oqupy.operators.sigma("y")
            op = oqupy.operators.left_right_super(u, u.conj().T)
        ops.append((step, op, post))
    return ops


def outputs(oqupy, c, pt):
    """Every reference output of one case on process tensor ``pt``."""
    sd = oqupy.system_dynamics
    system = oqupy.System(c["h"])
    out = {}
    t, corr = oqupy.compute_correlations(system, pt, c["op_a"], c["op_b"], c["times_a"],
                                         c["times_b"], initial_state=c["rho0"],
                                         progress_type="silent")
    out["ordered"] = corr
    t, corr = oqupy.compute_correlations(system, pt, c["op_a"], c["op_b"], c["anti_a"],
                                         c["times_b"], time_order="anti",
                                         initial_state=c["rho0"], progress_type="silent")
    out["anti"] = corr
    t, corr = oqupy.compute_correlations_nt(system, pt, c["nt_ops"], c["nt_times"],
                                            c["nt_order"], initial_state=c["rho0"],
                                            progress_type="silent")
    out["nt"] = corr
    ctrl = oqupy.Control(c["d"])
    for step, op, post in control_ops(oqupy, c):
        ctrl.add_single(step, op, post=post)
    dyn = oqupy.compute_dynamics(system, process_tensor=pt, control=ctrl,
                                 initial_state=c["rho0"], progress_type="silent")
    out["control_states"] = np.array(dyn.states).reshape(len(dyn.states), -1)
    tds = oqupy.TimeDependentSystem(c["h_t"])
    dyn = oqupy.compute_dynamics(tds, process_tensor=pt, initial_state=c["rho0"],
                                 progress_type="silent")
    out["td_states"] = np.array(dyn.states).reshape(len(dyn.states), -1)
    return out


def main(ref_root):
    oqupy = _import_reference(ref_root)
    patch_vectorize_checks(oqupy)
    sd = oqupy.system_dynamics
    res = {}
    for name, c in cases(oqupy):
        corr = oqupy.PowerLawSD(alpha=c["alpha"], zeta=1.0, cutoff=c["wc"],
                                cutoff_type=c["cutoff_type"], temperature=c["T"])
        bath = oqupy.Bath(c["coupling"], corr)
        params = oqupy.TempoParameters(dt=c["dt"], dkmax=c["dkmax"], epsrel=c["epsrel"])
        end_time = c["nsteps"] * c["dt"]
        ptt = oqupy.PtTempo(bath, 0.0, end_time, params)
        pt = ptt.get_process_tensor(progress_type="silent")
        assert len(pt) == c["nsteps"]
        kmax = ptt._backend_instance._num_infl
        res[f"{name}/influences"] = np.array([ptt._influence(dk) for dk in range(kmax)])
        res[f"{name}/dkmax"] = np.int64(c["dkmax"])
        res[f"{name}/epsrel"] = np.float64(c["epsrel"])
        res[f"{name}/nsteps"] = np.int64(c["nsteps"])
        res[f"{name}/d"] = np.int64(c["d"])
        res[f"{name}/rho0"] = np.asarray(c["rho0"], dtype=np.complex128).reshape(-1)
        for tname, tr in (("transform_in", pt.transform_in), ("transform_out", pt.transform_out)):
            if tr is not None:
                res[f"{name}/{tname}"] = np.asarray(tr)
        system = oqupy.System(c["h"])
        p1, p2 = system.get_propagators(c["dt"], 0.0, None, None)(0)
        res[f"{name}/prop1"], res[f"{name}/prop2"] = p1, p2
        tds = oqupy.TimeDependentSystem(c["h_t"])
        fprops = tds.get_propagators(c["dt"], 0.0, sd.SUBDIV_LIMIT, sd.INTEGRATE_EPSREL)
        tdp = [fprops(k) for k in range(c["nsteps"])]
        res[f"{name}/td_prop1"] = np.array([p[0] for p in tdp])
        res[f"{name}/td_prop2"] = np.array([p[1] for p in tdp])
        max_step = len(pt)
        res[f"{name}/ordered_steps_a"] = sd._parse_times(c["times_a"], max_step, c["dt"], 0.0)
        res[f"{name}/steps_b"] = sd._parse_times(c["times_b"], max_step, c["dt"], 0.0)
        res[f"{name}/anti_steps_a"] = sd._parse_times(c["anti_a"], max_step, c["dt"], 0.0)
        for j, t in enumerate(c["nt_times"]):
            res[f"{name}/nt_steps{j}"] = sd._parse_times(t, max_step, c["dt"], 0.0)
        res[f"{name}/nt_ops"] = np.array(c["nt_ops"], dtype=np.complex128)
        res[f"{name}/nt_order"] = np.array(c["nt_order"])
        res[f"{name}/op_a"] = np.asarray(c["op_a"], dtype=np.complex128)
        res[f"{name}/op_b"] = np.asarray(c["op_b"], dtype=np.complex128)
        ctrl_steps, ctrl_ops, ctrl_post = [], [], []
        for step, op, post in control_ops(oqupy, c):
            ctrl_steps.append(step)
            ctrl_ops.append(op)
            ctrl_post.append(post)
        res[f"{name}/control_steps"] = np.array(ctrl_steps)
        res[f"{name}/control_ops"] = np.array(ctrl_ops, dtype=np.complex128)
        res[f"{name}/control_post"] = np.array(ctrl_post)
        out = outputs(oqupy, c, pt)
        for k, v in out.items():
            res[f"{name}/{k}"] = v
        env = {k: np.zeros(len(v) if k.endswith("states") else np.shape(v)) for k, v in out.items()}
        for seed in (1, 2, "gesvd"):
            p2t = oqupy.PtTempo(bath, 0.0, end_time, params)
            if seed == "gesvd":
                os.environ["OQUPY_TNSHIM_SVD"] = "gesvd"
            else:
                p2t._backend_instance._influence = _perturbed(p2t._backend_instance._influence, seed)
            try:
                pt2 = p2t.get_process_tensor(progress_type="silent")
            finally:
                os.environ.pop("OQUPY_TNSHIM_SVD", None)
            out2 = outputs(oqupy, c, pt2)
            for k in out:
                if k.endswith("states"):
                    env[k] = np.maximum(env[k], [_trace_dist(a, b) for a, b in zip(out[k], out2[k])])
                else:
                    a, b = np.nan_to_num(out[k]), np.nan_to_num(out2[k])
                    env[k] = np.maximum(env[k], np.abs(a - b))
        for k, v in env.items():
            res[f"{name}/{k}_envelope"] = v
        print(name, {k: float(np.max(v)) for k, v in env.items()})
    np.savez_compressed(os.path.join(HERE, "correlations.npz"), **res)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit(__doc__)
    main(sys.argv[1])
