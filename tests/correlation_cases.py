"""The correlation / controlled-dynamics fixture (``tests/golden/
correlations.npz``, made by ``tests/golden/make_correlations.py`` from the
unmodified reference) and the checks shared by the CPU and GPU tests.

Every case runs five computations on one process tensor: time-ordered and
anti-time-ordered two-time correlations (``compute_correlations``,
system_dynamics.py:1011-1093), a three-operator ``compute_correlations_nt``
(:791-990), ``compute_dynamics`` with pre- and post-measurement controls
(:131-160) and ``compute_dynamics`` of a time-dependent system.  ``run``
evaluates them through two callables -- a controlled sweep and an n-time
correlation function -- so that the oracle and the GPU path are checked the
same way.
"""

import os

import numpy as np

from tests import golden_cases as gc

FIXTURE = os.path.join(gc.GOLDEN, "correlations.npz")
CASES = ("corr_nondiag", "corr_qutrit")


def load():
    return np.load(FIXTURE)


def get(g, name, key, default=None):
    k = f"{name}/{key}"
    return g[k] if k in g.files else default


def influence(g, name):
    infl = g[f"{name}/influences"]

    def f(dk):
        return infl[dk] if dk >= 0 else None
    return f


def controls(g, name):
    """``{"pre": {step: C}, "post": {step: C}}`` of the case's ``Control``
    (several operations at one step compose in insertion order,
    control.py:90-96)."""
    out = {"pre": {}, "post": {}}
    for step, op, post in zip(g[f"{name}/control_steps"], g[f"{name}/control_ops"],
                              g[f"{name}/control_post"]):
        side = out["post" if post else "pre"]
        step = int(step)
        side[step] = op if step not in side else op @ side[step]
    return out


def run(g, name, sweep, correlations):
    """The case's five outputs.

    ``sweep(propagators, rho0, num_steps, controls) -> states[num_steps+1, D]``;
    ``correlations(propagators, rho0, operators, op_steps, ops_order) -> array``.
    """
    p1, p2 = g[f"{name}/prop1"], g[f"{name}/prop2"]

    def props(step):
        return p1, p2
    tp1, tp2 = g[f"{name}/td_prop1"], g[f"{name}/td_prop2"]

    def td_props(step):
        return tp1[step], tp2[step]
    rho0 = g[f"{name}/rho0"]
    n = int(g[f"{name}/nsteps"])
    a, b = g[f"{name}/op_a"], g[f"{name}/op_b"]
    sb = g[f"{name}/steps_b"]
    out = {}
    out["ordered"] = correlations(props, rho0, [a, b], [g[f"{name}/ordered_steps_a"], sb],
                                  ["left", "left"])
    # time_order "anti": operators (B, A) at steps (b, a), orders right / left,
    # result transposed (system_dynamics.py:1076-1093)
    out["anti"] = correlations(props, rho0, [b, a], [sb, g[f"{name}/anti_steps_a"]],
                               ["right", "left"]).T
    steps = [g[f"{name}/nt_steps{j}"] for j in range(3)]
    out["nt"] = correlations(props, rho0, list(g[f"{name}/nt_ops"]), steps,
                             [str(x) for x in g[f"{name}/nt_order"]])
    out["control_states"] = sweep(props, rho0, n, controls(g, name))
    out["td_states"] = sweep(td_props, rho0, n, None)
    return out


def check(g, name, out, abs_tol=gc.PARITY_ABS):
    """Violations of ``max(abs_tol, 10 x the reference's own spread)``: trace
    distance for states, absolute error for correlations (NaN where the
    reference leaves NaN)."""
    from oracle import tempo_oracle as to
    bad = []
    worst = {}
    for k, got in out.items():
        ref = g[f"{name}/{k}"]
        env = g[f"{name}/{k}_envelope"]
        if k.endswith("states"):
            err = np.array([to.trace_distance(x, y) for x, y in zip(got, ref)])
        else:
            if not np.array_equal(np.isnan(got), np.isnan(ref)):
                bad.append((k, "NaN pattern"))
                continue
            err = np.abs(np.nan_to_num(got) - np.nan_to_num(ref))
        tol = np.maximum(abs_tol, gc.ENVELOPE_FACTOR * env)
        worst[k] = float(err.max())
        if (err > tol).any():
            bad.append((k, float(err.max()), float(tol.min())))
    return bad, worst
