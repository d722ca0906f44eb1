"""Process-tensor sweeps with step-dependent propagators and control
operations, and n-time correlations, on the GPU.

Reference: ``compute_dynamics`` with a ``Control`` and a time-dependent
system (oqupy/system_dynamics.py:41-182; controls applied at :131-160 as
``Control.get_controls`` returns them, control.py:119-180) and
``compute_correlations_nt`` / ``compute_correlations``
(system_dynamics.py:791-1093), which run one ``compute_dynamics`` per
combination of the earlier operators' times.  Here every such run is one
system slot of a single batched sweep over the device process tensor
(``otb_dyn_run_steps``): the slots share the process tensor and differ only
in the propagator pairs of the steps that carry a control operation, which
are folded in on the host (a post-measurement control C of step k:
P1 <- P1 C at step k; a pre-measurement control of step k + 1:
P2 <- C P2 at step k; a pre-measurement control of step 0 acts on rho0).
"""

from itertools import product
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

MAX_SLOTS = 1024   # systems per sweep launch (otb_dyn_run_steps)


def _pt_handle(process_tensor):
    if isinstance(process_tensor, tuple):
        batch, idx = process_tensor
        return batch, idx, None, None
    batch, idx = process_tensor.device
    return batch, idx, process_tensor.transform_in, process_tensor.transform_out


class PropagatorTable:
    """Distinct (P1, P2) pairs of a sweep; ``add`` returns a pair's index."""

    def __init__(self):
        self._rows: List[np.ndarray] = []
        self._index: Dict[bytes, int] = {}

    def add(self, p1: np.ndarray, p2: np.ndarray) -> int:
        pair = np.stack([p1, p2]).astype(np.complex128)
        key = pair.tobytes()
        j = self._index.get(key)
        if j is None:
            j = len(self._rows)
            self._rows.append(pair)
            self._index[key] = j
        return j

    def array(self) -> np.ndarray:
        return np.array(self._rows)

    def __len__(self):
        return len(self._rows)


def propagator_table(process_tensor, propagators, initial_states, num_steps, controls=None):
    """The sweep inputs of several systems: ``(batch, index in the batch,
    pair table [n_props, 2, D, D], pair index [H, num_steps], rho0 [H, D])``
    with the process tensor's transforms and the control operations folded
    in (see the module docstring)."""
    batch, i, tin, tout = _pt_handle(process_tensor)
    H = len(initial_states)
    n = int(num_steps)
    table = PropagatorTable()
    base: Dict[int, Tuple[list, np.ndarray]] = {}
    index = np.zeros((H, n), dtype=np.int32)
    rho0 = []
    for h in range(H):
        f = propagators[h]
        if id(f) not in base:
            pairs = []
            for k in range(n):
                p1, p2 = f(k)
                p1 = np.asarray(p1, dtype=np.complex128)
                p2 = np.asarray(p2, dtype=np.complex128)
                if tin is not None:
                    p1 = np.asarray(tin).T @ p1
                if tout is not None:
                    p2 = p2 @ np.asarray(tout).T
                pairs.append((p1, p2))
            base[id(f)] = (pairs, np.array([table.add(a, b) for a, b in pairs], dtype=np.int32))
        pairs, bidx = base[id(f)]
        index[h] = bidx
        rho = np.asarray(initial_states[h], dtype=np.complex128).reshape(-1)
        ctl = controls[h] if controls is not None else None
        if ctl:
            pre, post = ctl.get("pre", {}), ctl.get("post", {})
            if 0 in pre:
                rho = np.asarray(pre[0]) @ rho
            for k in sorted(set(post) | {s - 1 for s in pre if s >= 1}):
                if k < 0 or k >= n:
                    continue
                p1, p2 = pairs[k]
                if k in post:
                    p1 = p1 @ np.asarray(post[k])
                if k + 1 in pre:
                    p2 = np.asarray(pre[k + 1]) @ p2
                index[h, k] = table.add(p1, p2)
        rho0.append(rho)
    return batch, i, table.array(), index, np.array(rho0)


def device_dynamics(process_tensor, propagators: Sequence[Callable[[int], Tuple]],
                    initial_states: Sequence[np.ndarray], num_steps: int,
                    controls: Optional[Sequence[Optional[Dict]]] = None) -> np.ndarray:
    """``compute_dynamics`` of several systems on one device process tensor
    in one batched sweep.

    ``propagators[h](step) -> (P1, P2)`` (``BaseSystem.get_propagators``'s
    function; slots that share one function object share its pairs);
    ``controls[h]``: ``None`` or ``{"pre": {step: C}, "post": {step: C}}``
    superoperators.  Returns states ``[num_steps+1, H, D]`` (the state of
    every step, read after that step's pre-measurement control).
    """
    batch, i, table, index, rho0 = propagator_table(process_tensor, propagators, initial_states,
                                                    num_steps, controls)
    H = len(rho0)
    out = []
    for s in range(0, H, MAX_SLOTS):
        out.append(batch.dynamics_steps(i, table, index[s:s + MAX_SLOTS], rho0[s:s + MAX_SLOTS],
                                        int(num_steps)))
    return np.concatenate(out, axis=1)


def device_gradient(process_tensor, propagators: Callable[[int], Tuple], initial_state: np.ndarray,
                    target: np.ndarray, num_steps: int, controls: Optional[Dict] = None):
    """``compute_gradient_and_dynamics`` (gradient.py:169-437) on one device
    process tensor: the forward sweep keeps the state with its bond leg at
    every step, the adjoint sweep carries the target back through the
    transposed steps, and a kernel contracts both with every step's
    process-tensor tensor (``otb_dyn_gradient``).  The controls and
    transforms act on the outer legs of each step's tensor and are applied
    here.  Returns ``(derivs[num_steps, D, D, D, D], states[num_steps+1, D])``
    in the reference's leg order: [0] the state leg before the first
    half-step propagator of step n, [1] / [2] the MPO's input / output legs,
    [3] the leg after the second half-step propagator."""
    batch, i, tin, tout = _pt_handle(process_tensor)
    _, _, table, index, rho0 = propagator_table(process_tensor, [propagators], [initial_state],
                                                num_steps, [controls])
    n = int(num_steps)
    D = rho0.shape[1]
    states, cores = batch.gradient_cores(i, table, index, rho0, np.asarray(target).reshape(1, D), n)
    core = cores[0]                                   # [n, a', m, e']
    pre = (controls or {}).get("pre", {})
    post = (controls or {}).get("post", {})
    eye = np.identity(D, dtype=np.complex128)
    Tin = eye if tin is None else np.asarray(tin, dtype=np.complex128)
    Tout = eye if tout is None else np.asarray(tout, dtype=np.complex128)
    derivs = np.empty((n, D, D, D, D), dtype=np.complex128)
    for k in range(n):
        Pa = np.asarray(post.get(k, eye))             # F_k = post_k v_k on leg a
        Pe = np.asarray(pre.get(k + 1, eye))          # B_{k+1} = pre_{k+1}^T Y_{k+1} on leg e
        derivs[k] = np.einsum("ax,bm,mc,ye,xmy->abce", Pa, Tin, Tout, Pe, core[k])
    return derivs, states[:, 0]


def superoperator(operator: np.ndarray, side: str) -> np.ndarray:
    """``left_super`` (A rho) or ``right_super`` (rho A) of operators.py:139-147."""
    op = np.asarray(operator)
    eye = np.identity(op.shape[0])
    if side == "left":
        return np.kron(op, eye)
    if side == "right":
        return np.kron(eye, op.T)
    raise ValueError("ops_order entries must be 'left' or 'right'")


def device_correlations_nt(process_tensor, propagators: Callable[[int], Tuple],
                           initial_state: np.ndarray, operators: Sequence[np.ndarray],
                           op_steps: Sequence[Sequence[int]], ops_order: Sequence[str]) -> np.ndarray:
    """The correlation array of ``compute_correlations_nt``
    (system_dynamics.py:791-990) for operator time steps already parsed to
    integers: one sweep slot per time-ordered combination of the first n-1
    operators' steps, each applied as a pre-measurement control at its step
    (several at one step compose in order, control.py:90-96); the
    expectation ``Tr(O rho)`` of the last operator is read at every
    last-operator step not before the combination's latest step.  Entries
    the reference leaves unset are NaN."""
    sups = [superoperator(op, o) for op, o in zip(operators, ops_order)]
    shape = [len(t) for t in op_steps]
    out = np.full(shape, np.nan + 1j * np.nan, dtype=np.complex128)
    last = np.asarray(op_steps[-1], dtype=int)
    slots, ctls, keeps = [], [], []
    for idx in product(*[range(len(t)) for t in op_steps[:-1]]):
        first = [int(op_steps[j][i]) for j, i in enumerate(idx)]
        if first != sorted(first):
            continue
        keep = np.flatnonzero(last >= (max(first) if first else 0))
        if keep.size == 0:
            continue
        pre: Dict[int, np.ndarray] = {}
        for j, st in enumerate(first):
            pre[st] = sups[j] if st not in pre else sups[j] @ pre[st]
        slots.append(idx)
        ctls.append({"pre": pre})
        keeps.append(keep)
    if not slots:
        return out
    nsteps = int(max(last[k].max() for k in keeps))
    states = device_dynamics(process_tensor, [propagators] * len(slots),
                             [initial_state] * len(slots), nsteps, ctls)
    D = states.shape[-1]
    d = int(round(np.sqrt(D)))
    op = np.asarray(operators[-1], dtype=np.complex128)
    for h, (idx, keep) in enumerate(zip(slots, keeps)):
        rhos = states[last[keep], h].reshape(-1, d, d)
        out[tuple(np.array(idx)[:, None]) + (keep,)] = np.einsum("ab,kba->k", op, rhos)
    return out
