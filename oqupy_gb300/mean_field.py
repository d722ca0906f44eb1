"""Mean-field TEMPO on the batched GPU engine: the drop-in for
``oqupy.backends.tempo_backend.MeanFieldTempoBackend``
(tempo_backend.py:629-773).

The systems of a mean-field model are the instances of one ``TempoBatch``:
one launch advances all of them by a TEMPO step.  The coherent field stays on
the host, as in the reference: every step evaluates the field derivative and
each system's propagators from the current states and field (the user's
callables), uploads the propagators of all systems in one copy, advances the
batch, reads the next states back and evaluates the next field
(tempo_backend.py:747-773).

``device_dynamics_with_field`` is the process-tensor form
(``compute_dynamics_with_field``, system_dynamics.py:184-476): the systems'
sweeps over their device process tensors advance one step per call, with
the field evaluated on the host in between.
"""

from copy import deepcopy
from typing import Callable, Dict, List, Optional

import numpy as np

from . import _native as nat
from .tempo import DEFAULT_CHI_CAP, TempoBatch


class GpuMeanFieldTempoBackend:
    """Same constructor, ``step`` property, ``initialize() -> (0, states,
    field)`` and ``compute_step() -> (step, states, field)`` as the
    reference's ``MeanFieldTempoBackend``.

    ``config`` keys used: ``precision`` ("complex128" | "mixed"), ``chi_cap``
    (initial bond capacity; a step whose bonds outgrow it is redone with
    twice the capacity, up to 1152 / D, after replaying the earlier steps
    with the propagators recorded for them), ``block`` / ``smem_kb`` (launch
    shape, default 512 threads and 200 KiB: mean-field models have few
    systems, so each gets a wide CTA), ``qr_cut``.  Degeneracy maps are not
    supported by the GPU engine (``oqupy_gb300.install`` routes such runs to
    the reference backend).
    """

    def __init__(self, initial_state_list, initial_field, influence_list,
                 unitary_transform_list, propagators_list, compute_field,
                 compute_field_derivative, sum_north_list, sum_west_list,
                 dkmax, epsrel, config: Optional[Dict] = None,
                 degeneracy_maps_list=None, dim_list=None):
        if degeneracy_maps_list is not None and any(m is not None for m in degeneracy_maps_list):
            raise NotImplementedError("the GPU TEMPO engine needs unique=False")
        for sn, sw in zip(sum_north_list, sum_west_list):
            if not (np.allclose(sn, 1.0) and np.allclose(sw, 1.0)):
                raise NotImplementedError("the GPU TEMPO engine needs all-ones sums")
        self._initial_state_list = initial_state_list   # as given (returned by initialize)
        self._initial_states = [np.array(s, dtype=np.complex128).reshape(-1)
                                for s in initial_state_list]
        self._initial_field = complex(initial_field)
        self._influences = list(influence_list)
        self._unitaries = [np.asarray(u, dtype=np.complex128) for u in unitary_transform_list]
        self._propagators = list(propagators_list)
        self._compute_field = compute_field
        self._compute_field_derivative = compute_field_derivative
        self._dkmax = dkmax
        self._epsrel = epsrel
        self._config = {} if config is None else config
        self._step = None
        self._batch: Optional[TempoBatch] = None
        self._field = self._initial_field
        self._states: List[np.ndarray] = []
        self._history: List[tuple] = []   # propagators of every step, for a replay
        self._ninfl = 0
        self._slots = 16

    @property
    def step(self):
        """The current step of the computation."""
        return self._step

    @property
    def chi_cap(self) -> int:
        """Current bond capacity of the device handle."""
        return self._cap

    def bond_dimensions(self, system: int) -> List[int]:
        """Bond dimensions of one system's current MPS."""
        return self._batch.bond_dims(system)

    def initialize(self):
        """tempo_backend.py:740-745: every system at rho0, field at its
        initial value."""
        Ds = [s.size for s in self._initial_states]
        n = 1 if self._dkmax is None else self._dkmax + 1
        self._insts = []
        for s, infl, u in zip(self._initial_states, self._influences, self._unitaries):
            D = s.size
            d = int(round(np.sqrt(D)))
            self._insts.append(dict(
                hs_dim=d, dkmax=self._dkmax, epsrel=self._epsrel,
                influences=np.array([infl(dk) for dk in range(n)], dtype=np.complex128),
                prop1=np.identity(D, dtype=np.complex128), prop2=np.identity(D, dtype=np.complex128),
                rho0=s, unitary=u))
        self._cap = max(int(self._config.get("chi_cap", DEFAULT_CHI_CAP)), max(Ds))
        self._cap_max = min(nat.MAX_COLUMNS // D for D in Ds)
        self._new_batch()
        self._history = []
        self._step = 0
        self._field = self._initial_field
        # the step-0 states are the initial states as given, as in the
        # reference (tempo_backend.py:740-745); later ones are vectors
        self._states = deepcopy(list(self._initial_state_list))
        return self._step, deepcopy(self._states), self._field

    def _new_batch(self):
        if self._batch is not None:
            self._batch.close()
        self._batch = TempoBatch(
            self._insts, precision=self._config.get("precision", "complex128"),
            chi_cap=self._cap, out_cap=4, max_sites=16 if self._dkmax is None else 0,
            block=int(self._config.get("block", 512)), smem_kb=int(self._config.get("smem_kb", 200)),
            qr_cut=float(self._config.get("qr_cut", 0.0)))
        self._ninfl = len(self._insts[0]["influences"])
        self._slots = 16

    def _advance(self, step: int) -> int:
        """One engine step of every system with the propagators recorded for
        ``step``; returns the first nonzero instance status (0 if none)."""
        b = self._batch
        p1s, p2s = self._history[step - 1]
        b.set_all_propagators(p1s, p2s, self._unitaries)
        if self._dkmax is None:
            # the window of step s holds dk = 0 .. s-1 (tempo_backend.py:487-497)
            while self._ninfl < step:
                for i, infl in enumerate(self._influences):
                    b.set_influence(i, self._ninfl, infl(self._ninfl))
                self._ninfl += 1
            if max(b.info(i)["nsites"] for i in range(b.n)) + 2 > self._slots:
                self._slots = max(2 * self._slots, step + 2)
                b.reserve_sites(self._slots)
        elif step > self._dkmax:
            for i, infl in enumerate(self._influences):
                neg = infl(self._dkmax - step)
                if neg is not None:
                    b.set_first_influence(i, neg)
        b.advance(1)
        for i in range(b.n):
            st = b.info(i)["status"]
            if st != 0:
                return st
        return 0

    def compute_step(self):
        """tempo_backend.py:747-773."""
        cur = self._step
        nxt_step = cur + 1
        states = deepcopy(self._states)
        field = self._field
        deriv = self._compute_field_derivative(cur, states, field)
        props = [p(cur, field, deriv) for p in self._propagators]
        self._history.append(([np.asarray(p[0]) for p in props], [np.asarray(p[1]) for p in props]))
        st = self._advance(nxt_step)
        while st == nat.OTB_ERR_CHI_OVERFLOW and self._cap < self._cap_max:
            self._cap = min(2 * self._cap, self._cap_max)
            self._new_batch()
            for s in range(1, nxt_step + 1):
                st = self._advance(s)
                if st != 0:
                    break
        if st != 0:
            raise nat.DeviceError(st, f"mean-field TEMPO step {nxt_step}")
        got = self._batch.states(nxt_step, 1)
        nxt = [np.array(x[0]) for x in got]
        self._field = complex(self._compute_field(cur, states, field, nxt))
        self._states = nxt
        self._step = nxt_step
        return self._step, deepcopy(self._states), self._field

    def close(self):
        if self._batch is not None:
            self._batch.close()
            self._batch = None


def device_dynamics_with_field(propagators_list, field_eom, initial_field, process_tensors,
                               initial_states, num_steps: int, dt: float, start_time: float = 0.0,
                               controls=None):
    """``compute_dynamics_with_field`` (system_dynamics.py:184-476) with one
    device process tensor per system: every step reads the systems' states,
    advances the field by the reference's second-order Runge-Kutta rule,
    evaluates each system's propagators from the field and its derivative
    and advances all systems that share a process tensor in one sweep step
    (``otb_dyn_session_step``).

    ``propagators_list[i](step, field, field_derivative) -> (P1, P2)``;
    ``field_eom(t, states, field)`` with ``d x d`` states;
    ``process_tensors[i]``: a ``DeviceProcessTensor`` (or ``(PtBatch, i)``);
    ``controls[i]``: ``None`` or ``{"pre": {step: C}, "post": {step: C}}``.
    Returns ``(times, states[num_steps+1][system] (d x d), fields)``."""
    from .correlations import _pt_handle
    n_sys = len(propagators_list)
    controls = [None] * n_sys if controls is None else list(controls)
    D = [np.asarray(s).size for s in initial_states]
    dims = [int(round(np.sqrt(x))) for x in D]
    # systems that share a process tensor share one session
    groups = {}
    for i, pt in enumerate(process_tensors):
        groups.setdefault(id(pt), []).append(i)
    sessions = []
    for key, members in groups.items():
        batch, idx, tin, tout = _pt_handle(process_tensors[members[0]])
        rho0 = []
        for i in members:
            r = np.asarray(initial_states[i], dtype=np.complex128).reshape(-1)
            pre0 = (controls[i] or {}).get("pre", {}).get(0)
            rho0.append(r if pre0 is None else np.asarray(pre0) @ r)
        sessions.append((members, batch.session(idx, np.array(rho0)), tin, tout))

    def mats(vecs):
        return [np.asarray(v).reshape(d, d) for v, d in zip(vecs, dims)]

    def rk2(t, prev, field, cur):
        rk1 = field_eom(t, mats(prev), field)
        rk2_ = field_eom(t + dt, mats(cur), field + rk1 * dt)
        return field + dt * (rk1 + rk2_) / 2

    current = [None] * n_sys
    for members, sess, _, _ in sessions:
        st = sess.state(0)
        for j, i in enumerate(members):
            current[i] = st[j]
    states, fields = [], []
    field = complex(initial_field)
    previous = None
    try:
        for step in range(num_steps):
            t = start_time + step * dt
            if step > 0:
                field = rk2(t, previous, field, current)
            previous = list(current)
            states.append(mats(current))
            fields.append(field)
            deriv = field_eom(t, mats(current), field)
            nxt = [None] * n_sys
            for members, sess, tin, tout in sessions:
                pairs = []
                for i in members:
                    p1, p2 = propagators_list[i](step, field, deriv)
                    p1 = np.asarray(p1, dtype=np.complex128)
                    p2 = np.asarray(p2, dtype=np.complex128)
                    if tin is not None:
                        p1 = np.asarray(tin).T @ p1
                    if tout is not None:
                        p2 = p2 @ np.asarray(tout).T
                    ctl = controls[i] or {}
                    post = ctl.get("post", {}).get(step)
                    pre_next = ctl.get("pre", {}).get(step + 1)
                    if post is not None:
                        p1 = p1 @ np.asarray(post)
                    if pre_next is not None:
                        p2 = np.asarray(pre_next) @ p2
                    pairs.append(np.stack([p1, p2]))
                out = sess.step(np.array(pairs))
                for j, i in enumerate(members):
                    nxt[i] = out[j]
            current = nxt
        t = start_time + num_steps * dt
        states.append(mats(current))
        fields.append(rk2(t, previous, field, current) if num_steps > 0 else field)
    finally:
        for _, sess, _, _ in sessions:
            sess.close()
    times = start_time + np.arange(len(states)) * dt
    return list(times), states, fields
