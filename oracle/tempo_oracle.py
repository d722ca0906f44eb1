"""Plain-numpy restatement of OQuPy's TEMPO / PT-TEMPO / PT-sweep hot path.

TEST INFRASTRUCTURE ONLY -- the oracle the CUDA path is checked against.  It
is never imported by the product package ``oqupy_gb300``.

Every MPS / MPO site is held in one uniform layout so that the algebra is
explicit (no edge bookkeeping):

* MPS site  ``A[l, a, r]``        left bond, array (Liouville) leg, right bond
* MPO site  ``B[ml, ain, aout, mr]``  left bond, input leg, output leg, right
  bond

A missing leg of the reference's ``NodeArray`` (``left=False`` etc.) is a leg
of dimension one here, which does not change any number.

Reference being restated (OQuPy 0.5.0, paths relative to the project root):

* ``oqupy/backends/node_array.py:226-299``  ``NodeArray.svd_sweep``
* ``oqupy/backends/node_array.py:413-554``  ``NodeArray.zip_up``
* ``oqupy/backends/node_array.py:301-411``  ``NodeArray.contract`` (trace-out)
* ``oqupy/backends/tempo_backend.py:379-575`` ``BaseTempoBackend``
* ``oqupy/backends/tempo_backend.py:610-626`` ``TempoBackend.initialize/compute_step``
* ``oqupy/backends/tempo_backend.py:629-773`` ``MeanFieldTempoBackend``
* ``oqupy/backends/pt_tempo_backend.py:105-316`` ``PtTempoBackend``
* ``oqupy/process_tensor.py:326-406``  ``get_mpo_tensor`` / ``compute_caps``
* ``oqupy/system_dynamics.py:41-182, 631-700``  ``compute_dynamics``
* ``oqupy/system_dynamics.py:184-476``  ``compute_dynamics_with_field``
* ``oqupy/system_dynamics.py:791-990``  ``compute_correlations_nt``
* ``oqupy/gradient.py:169-437``  ``compute_gradient_and_dynamics``
* truncation rule of ``tensornetwork.split_node_full_svd(relative=True)``,
  also stated in-tree at ``oqupy/mps_mpo.py:452-457``.
"""

from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np

CDT = np.complex128


# ---------------------------------------------------------------------------
# truncated SVD
# ---------------------------------------------------------------------------

def truncation_rank(s: np.ndarray, epsrel: float) -> int:
    """Number of singular values kept: discard the longest tail whose 2-norm
    is ``<= epsrel * s[0]`` (``oqupy/mps_mpo.py:452-457``; the
    ``max_truncation_err``/``relative=True`` arguments at
    ``oqupy/backends/node_array.py:541-547``)."""
    if s.size == 0:
        return 0
    tail = np.sqrt(np.cumsum(np.square(s[::-1])))
    return int(np.count_nonzero(tail > epsrel * s[0]))


def truncated_svd(mat: np.ndarray, epsrel: float):
    """Thin SVD + relative truncation.  Returns ``(u, s, vh, discarded)``."""
    u, s, vh = np.linalg.svd(mat, full_matrices=False)
    k = truncation_rank(s, epsrel)
    return u[:, :k], s[:k], vh[:k, :], s[k:]


# ---------------------------------------------------------------------------
# NodeArray operations on uniform site lists
# ---------------------------------------------------------------------------

def zip_up_right(mps: List[np.ndarray], mpo: List[np.ndarray], left_index: int,
                 epsrel: float, stats: Optional[list] = None) -> None:
    """``NodeArray.zip_up(direction="right")`` (node_array.py:503-552).

    Zips ``mpo`` onto ``mps[left_index : left_index+len(mpo)]``; every site
    but the last is split by a truncated SVD with rows (outer bond, output
    leg) and columns (MPS bond, MPO bond); ``S @ Vh`` is carried right.
    The last site keeps the merged (MPS right bond, MPO right bond) as its
    right bond."""
    n = len(mpo)
    first = mps[left_index]
    l0 = first.shape[0]
    ml0 = mpo[0].shape[0]
    assert ml0 == 1, "first MPO site must have a closed left bond"
    carry = np.eye(l0, dtype=CDT).reshape(l0, l0, 1)
    for j in range(n):
        ia = left_index + j
        A = mps[ia]
        B = mpo[j]
        # theta[x, aout, r, mr] = sum_{l, ml, a} carry[x,l,ml] A[l,a,r] B[ml,a,aout,mr]
        tmp = np.tensordot(carry, A, axes=([1], [0]))          # x, ml, a, r
        theta = np.tensordot(tmp, B, axes=([1, 2], [0, 1]))    # x, r, aout, mr
        theta = theta.transpose(0, 2, 1, 3)                    # x, aout, r, mr
        x, ao, r, mr = theta.shape
        if j == n - 1:
            mps[ia] = theta.reshape(x, ao, r * mr)
        else:
            u, s, vh, disc = truncated_svd(theta.reshape(x * ao, r * mr), epsrel)
            k = s.size
            if stats is not None:
                stats.append((x * ao, r * mr, k))
            mps[ia] = u.reshape(x, ao, k)
            carry = (s[:, None] * vh).reshape(k, r, mr)


def zip_up_left(mps: List[np.ndarray], mpo: List[np.ndarray], right_index: int,
                epsrel: float, stats: Optional[list] = None) -> None:
    """``NodeArray.zip_up(direction="left")`` (node_array.py:503-552 with the
    left-direction variables of :456-467).

    Zips ``mpo`` onto ``mps[right_index-len(mpo)+1 : right_index+1]`` going
    right-to-left.  Rows of each split are (outer right bond, output leg),
    columns are (MPS left bond, MPO left bond)."""
    n = len(mpo)
    last = mps[right_index]
    r0 = last.shape[2]
    mr0 = mpo[-1].shape[3]
    assert mr0 == 1, "last MPO site must have a closed right bond"
    carry = np.eye(r0, dtype=CDT).reshape(r0, r0, 1)          # x, r, mr
    for j in range(n):
        ia = right_index - j
        ib = n - 1 - j
        A = mps[ia]
        B = mpo[ib]
        # theta[l, ml, aout, x] = sum_{r, mr, a} A[l,a,r] B[ml,a,aout,mr] carry[x,r,mr]
        tmp = np.tensordot(A, carry, axes=([2], [1]))          # l, a, x, mr
        theta = np.tensordot(tmp, B, axes=([1, 3], [1, 3]))    # l, x, ml, aout
        l, x, ml, ao = theta.shape
        if j == n - 1:
            mps[ia] = theta.transpose(0, 2, 3, 1).reshape(l * ml, ao, x)
        else:
            mat = theta.transpose(1, 3, 0, 2).reshape(x * ao, l * ml)
            u, s, vh, disc = truncated_svd(mat, epsrel)
            k = s.size
            if stats is not None:
                stats.append((x * ao, l * ml, k))
            # U edges (right bond x, aout, new) -> site (new, aout, x)
            mps[ia] = u.reshape(x, ao, k).transpose(2, 1, 0)
            carry = (s[:, None] * vh).reshape(k, l, ml)


def svd_sweep_right_to_left(mps: List[np.ndarray], from_index: int,
                            to_index: int, epsrel: float,
                            stats: Optional[list] = None) -> None:
    """``NodeArray.svd_sweep`` with ``to < from`` (node_array.py:274-296)."""
    for i in range(from_index, to_index, -1):
        A = mps[i]
        l, a, r = A.shape
        mat = A.transpose(1, 2, 0).reshape(a * r, l)
        u, s, vh, disc = truncated_svd(mat, epsrel)
        k = s.size
        if stats is not None:
            stats.append((a * r, l, k))
        mps[i] = u.reshape(a, r, k).transpose(2, 0, 1)
        svh = s[:, None] * vh                                   # k, l
        mps[i - 1] = np.tensordot(mps[i - 1], svh, axes=([2], [1]))


def svd_sweep_left_to_right(mps: List[np.ndarray], from_index: int,
                            to_index: int, epsrel: float,
                            stats: Optional[list] = None) -> None:
    """``NodeArray.svd_sweep`` with ``from < to`` (node_array.py:251-273)."""
    for i in range(from_index, to_index):
        A = mps[i]
        l, a, r = A.shape
        u, s, vh, disc = truncated_svd(A.reshape(l * a, r), epsrel)
        k = s.size
        if stats is not None:
            stats.append((l * a, r, k))
        mps[i] = u.reshape(l, a, k)
        svh = s[:, None] * vh                                   # k, r
        mps[i + 1] = np.tensordot(svh, mps[i + 1], axes=([1], [0]))


def trace_out_first(mps: List[np.ndarray], sum_north: np.ndarray) -> None:
    """``NodeArray.contract`` of the first site with ``sum_north`` and merge
    into its neighbour (node_array.py:301-411; used at
    tempo_backend.py:531-537)."""
    A0 = mps.pop(0)
    v = np.tensordot(A0, sum_north, axes=([1], [0]))            # l, r
    mps[0] = np.tensordot(v, mps[0], axes=([1], [0]))          # l, a, r


# ---------------------------------------------------------------------------
# helpers restating oqupy.util / oqupy.operators
# ---------------------------------------------------------------------------

def left_right_super(left: np.ndarray, right: np.ndarray) -> np.ndarray:
    """``oqupy/operators.py:149-153``."""
    return np.kron(left, right.T)


def delta_1001(infl: np.ndarray) -> np.ndarray:
    """``create_delta(infl, [1, 0, 0, 1])`` (util.py:30-57):
    ``T[j, i, i, j] = infl[i, j]``."""
    n0, n1 = infl.shape
    T = np.zeros((n1, n0, n0, n1), dtype=CDT)
    for i in range(n0):
        for j in range(n1):
            T[j, i, i, j] = infl[i, j]
    return T


# ---------------------------------------------------------------------------
# TEMPO
# ---------------------------------------------------------------------------

class TempoOracle:
    """Restatement of ``TempoBackend`` (tempo_backend.py:315-626), same
    constructor arguments, ``unique=False`` (no degeneracy maps).

    ``initialize() -> (0, state)``; ``compute_step() -> (step, state)``.
    """

    def __init__(self, initial_state, influence, unitary_transform,
                 propagators, sum_north, sum_west, dkmax, epsrel,
                 config=None, degeneracy_maps=None, dim=None):
        if degeneracy_maps is not None:
            raise NotImplementedError("oracle covers unique=False only")
        self._initial_state = np.array(initial_state, dtype=CDT).reshape(-1)
        self._influence = influence
        self._unitary = np.array(unitary_transform, dtype=CDT)
        self._propagators = propagators
        self._sum_north = np.array(sum_north, dtype=CDT)
        self._sum_west = np.array(sum_west, dtype=CDT)
        self._dkmax = dkmax
        self._epsrel = epsrel
        self._step = None
        self.stats = []           # (rows, cols, kept) of every split
        self.bond_history = []    # max bond dimension after every step

    @property
    def step(self):
        return self._step

    def _initialize_mps_mpo(self):
        """tempo_backend.py:379-437."""
        U = self._unitary
        super_u = left_right_super(U, U.conjugate().T)
        super_u_dagg = left_right_super(U.conjugate().T, U)
        self._super_u, self._super_u_dagg = super_u, super_u_dagg
        npre = 1 if self._dkmax is None else self._dkmax + 1
        infls = []
        for i in range(npre):
            infl = self._influence(i)
            T = delta_1001(infl)
            if i == 0:
                # tempo_backend.py:419-424: rotate input leg and right bond
                T = np.einsum("lpor,px->lxor", T, super_u_dagg)
                T = np.einsum("lxor,yr->lxoy", T, super_u)
            infls.append(T)
        self._mpo = list(reversed(infls))
        self._mps = [self._initial_state.reshape(1, -1, 1)]

    def initialize(self):
        self._step = 0
        self._initialize_mps_mpo()
        return 0, self._initial_state.copy()

    def compute_step(self):
        """TempoBackend.compute_step (tempo_backend.py:619-626)."""
        self._step += 1
        p1, p2 = self._propagators(self._step - 1)
        state = self.compute_system_step(self._step, np.asarray(p1, CDT),
                                         np.asarray(p2, CDT))
        return self._step, state

    def compute_system_step(self, current_step, prop_1, prop_2):
        """tempo_backend.py:439-575."""
        D = prop_1.shape[0]
        # -- MPO window (tempo_backend.py:487-517)
        if self._dkmax is None:
            mpo = [b.copy() for b in self._mpo]
            infl = self._influence(len(mpo))
            self._mpo = [delta_1001(infl)] + self._mpo
        elif current_step <= self._dkmax:
            mpo = [b.copy() for b in self._mpo[-current_step:]]
        else:
            mpo = [b.copy() for b in self._mpo]
            infl = self._influence(self._dkmax - current_step)
            if infl is not None:
                mpo[0] = delta_1001(infl)
        # -- sum west (tempo_backend.py:519)
        b0 = mpo[0]
        mpo[0] = np.tensordot(self._sum_west, b0, axes=([0], [0]))[None]
        # -- first half-step propagator on the last site (:521-529)
        last = self._mps[-1]
        self._mps[-1] = np.einsum("ba,lar->lbr", prop_1, last)
        # -- trace out the oldest site (:531-537)
        if len(self._mps) != len(mpo):
            trace_out_first(self._mps, self._sum_north)
        # -- zip-up and sweep (:539-553)
        zip_up_right(self._mps, mpo, 0, self._epsrel, self.stats)
        svd_sweep_right_to_left(self._mps, len(self._mps) - 1, 0,
                                self._epsrel, self.stats)
        # -- second half-step propagator as a new site (:555-558)
        self._mps.append(prop_2.T.reshape(D, D, 1).copy())
        self.bond_history.append(max(A.shape[2] for A in self._mps))
        # -- read-out (:560-573)
        v = np.ones(1, dtype=CDT)
        for A in self._mps[:-1]:
            v = np.einsum("l,lar,a->r", v, A, self._sum_north)
        state = np.einsum("l,lb->b", v, self._mps[-1][:, :, 0])
        return state

    def bond_dimensions(self):
        return [A.shape[2] for A in self._mps[:-1]]


def tempo_dynamics(initial_state, influence, unitary_transform, propagators,
                   dkmax, epsrel, num_steps):
    """Run ``num_steps`` TEMPO steps; returns ``(states[num_steps+1, D],
    oracle)`` where ``states[0]`` is the initial state."""
    D = np.asarray(initial_state).size
    ones = np.ones(D)
    o = TempoOracle(initial_state, influence, unitary_transform, propagators,
                    ones, ones, dkmax, epsrel)
    out = [o.initialize()[1]]
    for _ in range(num_steps):
        out.append(o.compute_step()[1])
    return np.array(out), o


class MeanFieldOracle:
    """Restatement of ``MeanFieldTempoBackend`` (tempo_backend.py:629-773):
    one ``TempoOracle`` per system, a coherent field advanced on the host.

    ``propagators_list[i](step, field, field_derivative) -> (P1, P2)``;
    ``compute_field(step, states, field, next_states) -> next field``;
    ``compute_field_derivative(step, states, field) -> derivative``.
    ``initialize() -> (0, states, field)``; ``compute_step() -> (step,
    states, field)``.
    """

    def __init__(self, initial_state_list, initial_field, influence_list,
                 unitary_transform_list, propagators_list, compute_field,
                 compute_field_derivative, dkmax, epsrel):
        self._field = complex(initial_field)
        self._states = [np.array(s, dtype=CDT).reshape(-1) for s in initial_state_list]
        self._propagators = list(propagators_list)
        self._compute_field = compute_field
        self._compute_field_derivative = compute_field_derivative
        self._systems = []
        for s, infl, u in zip(self._states, influence_list, unitary_transform_list):
            ones = np.ones(s.size)
            self._systems.append(TempoOracle(s, infl, u, None, ones, ones, dkmax, epsrel))
        self._step = None

    @property
    def step(self):
        return self._step

    def initialize(self):
        """tempo_backend.py:740-745."""
        self._step = 0
        for o in self._systems:
            o.initialize()
        return 0, [s.copy() for s in self._states], self._field

    def compute_step(self):
        """tempo_backend.py:747-773: the field derivative and the propagators
        from the current states and field, one TEMPO step per system, then
        the next field from the current and next states."""
        cur = self._step
        states = [s.copy() for s in self._states]
        deriv = self._compute_field_derivative(cur, states, self._field)
        props = [p(cur, self._field, deriv) for p in self._propagators]
        nxt = [o.compute_system_step(cur + 1, np.asarray(p1, CDT), np.asarray(p2, CDT))
               for o, (p1, p2) in zip(self._systems, props)]
        self._field = complex(self._compute_field(cur, states, self._field, nxt))
        self._states = nxt
        self._step = cur + 1
        return self._step, [s.copy() for s in nxt], self._field


# ---------------------------------------------------------------------------
# PT-TEMPO
# ---------------------------------------------------------------------------

class PtTempoOracle:
    """Restatement of ``PtTempoBackend`` (pt_tempo_backend.py:28-316),
    ``unique=False``.  ``get_mpo_tensors()`` returns the rank-3 PT-MPO
    tensors ``(chi_k, chi_{k+1}, D)`` that ``update_process_tensor`` stores."""

    def __init__(self, dimension, influence, sum_north, sum_west, num_steps,
                 dkmax, epsrel, degeneracy_maps=None):
        if degeneracy_maps is not None:
            raise NotImplementedError("oracle covers unique=False only")
        self._d = dimension
        self._influence = influence
        self._sum_north = np.array(sum_north, dtype=CDT)
        self._sum_west = np.array(sum_west, dtype=CDT)
        self._num_steps = num_steps
        self._dkmax = dkmax
        self._epsrel = epsrel
        self._num_infl = min(num_steps, dkmax + 1)
        self._step = None
        self.stats = []

    @property
    def step(self):
        return self._step

    @property
    def num_steps(self):
        return self._num_steps

    def initialize(self):
        """pt_tempo_backend.py:105-190."""
        d = self._d
        self._sum_north_scaled = self._sum_north * d
        mpo, mps = [], []
        n = self._num_infl
        assert n >= 2, "num_infl >= 2 required"
        for i in range(n):
            infl = np.asarray(self._influence(i), dtype=CDT)
            D = infl.shape[1]
            if i == 0:
                infl = infl / d
                B = np.zeros((1, D, D, infl.shape[0]), dtype=CDT)
                for a in range(infl.shape[0]):
                    for j in range(D):
                        B[0, j, j, a] = infl[a, j]
                A = (infl.T / d).reshape(1, D, infl.shape[0])
            elif i == n - 1:
                B = infl.reshape(infl.shape[0], 1, D, 1).copy()
                A = infl.reshape(infl.shape[0], D, 1).copy()
            else:
                m = infl.shape[0]
                B = np.zeros((m, D, D, m), dtype=CDT)
                A = np.zeros((m, D, m), dtype=CDT)
                for a in range(m):
                    for j in range(D):
                        B[a, j, j, a] = infl[a, j]
                        A[a, j, a] = infl[a, j] / d
            mpo.append(B)
            mps.append(A)
        self._mpo, self._mps = mpo, mps
        svd_sweep_right_to_left(self._mps, len(mps) - 1, 0, self._epsrel,
                                self.stats)
        svd_sweep_left_to_right(self._mps, 0, len(mps) - 1, self._epsrel,
                                self.stats)
        self._step = 1

    def compute_step(self) -> bool:
        """pt_tempo_backend.py:192-282."""
        self._step += 1
        end_phase = self._step > self._num_steps - self._num_infl + 1
        if end_phase:
            self._mpo = self._mpo[:-1]
            B = self._mpo[-1]
            self._mpo[-1] = np.tensordot(B, self._sum_north_scaled,
                                         axes=([3], [0]))[..., None]
        else:
            if self._dkmax is not None:
                infl = self._influence(int(0 - self._step))
                if infl is not None:
                    infl = np.asarray(infl, dtype=CDT)
                    self._mpo[-1] = infl.reshape(infl.shape[0], 1,
                                                 infl.shape[1], 1).copy()
            self._mps.append(np.ones((1, 1, 1), dtype=CDT))
        mpo = [b.copy() for b in self._mpo]
        zip_up_left(self._mps, mpo, len(self._mps) - 1, self._epsrel,
                    self.stats)
        svd_sweep_left_to_right(self._mps, self._step - 2,
                                len(self._mps) - 1, self._epsrel, self.stats)
        return self._step < self._num_steps

    def get_mpo_tensors(self) -> List[np.ndarray]:
        """pt_tempo_backend.py:284-307: ``(l, r, a) * d`` per step."""
        assert len(self._mps) == self._num_steps
        return [A.transpose(0, 2, 1) * self._d for A in self._mps]


def compute_caps(mpo_tensors: Sequence[np.ndarray], d: int) -> List[np.ndarray]:
    """``SimpleProcessTensor.compute_caps`` (process_tensor.py:380-406) for
    rank-3 tensors without transforms."""
    trace = (np.identity(d, dtype=CDT) / np.sqrt(float(d))).flatten()
    trace_sq = trace ** 2
    caps = [np.array([1.0], dtype=CDT)]
    for T in reversed(mpo_tensors):
        new = np.einsum("lra,r,a->l", T, caps[0], trace_sq)
        caps.insert(0, new)
    return caps


def pt_tempo_build(dimension, influence, num_steps, dkmax, epsrel):
    """Full PT-TEMPO build; returns ``(mpo_tensors, caps, oracle)``."""
    D = dimension ** 2
    ones = np.ones(D)
    o = PtTempoOracle(dimension, influence, ones, ones, num_steps, dkmax,
                      epsrel)
    o.initialize()
    while o.compute_step():
        pass
    mpos = o.get_mpo_tensors()
    return mpos, compute_caps(mpos, dimension), o


def pt_mpo_rank4(T3: np.ndarray, transform_in=None, transform_out=None):
    """``SimpleProcessTensor.get_mpo_tensor`` (process_tensor.py:326-356):
    rank-3 -> rank-4 with a delta between input and output legs, then the
    optional basis transforms."""
    l, r, D = T3.shape
    T = np.zeros((l, r, D, D), dtype=CDT)
    for a in range(D):
        T[:, :, a, a] = T3[:, :, a]
    if transform_in is not None:
        T = np.dot(np.moveaxis(T, -2, -1), np.asarray(transform_in).T)
        T = np.moveaxis(T, -1, -2)
    if transform_out is not None:
        T = np.dot(T, np.asarray(transform_out))
    return T


def compute_dynamics_pt(initial_state, propagators, mpo_tensors, caps,
                        num_steps=None, transform_in=None, transform_out=None,
                        controls=None):
    """``compute_dynamics`` with one process tensor (system_dynamics.py:41-182,
    helpers :631-700).  ``controls(step) -> (pre, post)`` superoperators or
    ``None`` (``Control.get_controls``, control.py:119-160): ``pre`` acts
    before the state of the step is read, ``post`` after it, before the
    step's propagation (system_dynamics.py:131-160).  Returns
    ``states[num_steps+1, D]``."""
    rho = np.asarray(initial_state, dtype=CDT).reshape(-1)
    D = rho.size
    if num_steps is None:
        num_steps = len(mpo_tensors)
    v = rho.reshape(1, D)
    states = []
    for step in range(num_steps + 1):
        pre, post = controls(step) if controls is not None else (None, None)
        if pre is not None:
            v = v @ np.asarray(pre, CDT).T
        if step == num_steps:
            break
        states.append(np.einsum("ba,b->a", v, caps[step]))
        if post is not None:
            v = v @ np.asarray(post, CDT).T
        p1, p2 = propagators(step)
        v = v @ np.asarray(p1, CDT).T
        T = pt_mpo_rank4(mpo_tensors[step], transform_in, transform_out)
        v = np.einsum("la,lrab->rb", v, T)
        v = v @ np.asarray(p2, CDT).T
    states.append(np.einsum("ba,b->a", v, caps[num_steps]))
    return np.array(states)


def dynamics_with_field_pt(initial_states, propagators_list, field_eom, initial_field,
                           pts, num_steps, dt, start_time=0.0, controls_list=None):
    """``compute_dynamics_with_field`` (system_dynamics.py:184-476) with one
    process tensor per system: ``pts[i] = (mpo_tensors, caps, transform_in,
    transform_out)``, ``propagators_list[i](step, field, derivative)``,
    ``field_eom(t, states, field)`` on ``d x d`` states.  Per step: the
    pre-measurement controls, the states, the field (initial value at step 0,
    afterwards the second-order Runge-Kutta rule of :319-325 at time t from
    the previous states), the post-measurement controls, the propagators from
    the field and its derivative, one sweep step per system; at the end the
    last states and one more field update.  Returns ``(states[num_steps+1]
    [system], fields)``."""
    n_sys = len(initial_states)
    ctls = controls_list or [None] * n_sys
    dims = [int(round(np.sqrt(np.asarray(s).size))) for s in initial_states]
    vs = [np.asarray(s, dtype=CDT).reshape(1, -1) for s in initial_states]

    def read(i, step):
        return np.einsum("ba,b->a", vs[i], pts[i][1][step]).reshape(dims[i], dims[i])

    def compute_field(t, prev, field, cur):
        rk1 = field_eom(t, prev, field)
        rk2 = field_eom(t + dt, cur, field + rk1 * dt)
        return field + dt * (rk1 + rk2) / 2

    states, fields = [], []
    field = complex(initial_field)
    prev = None
    for step in range(num_steps + 1):
        t = start_time + step * dt
        for i in range(n_sys):
            pre = ctls[i](step)[0] if ctls[i] is not None else None
            if pre is not None:
                vs[i] = vs[i] @ np.asarray(pre, CDT).T
        if step == num_steps:
            break
        cur = [read(i, step) for i in range(n_sys)]
        field = field if step == 0 else compute_field(t, prev, field, cur)
        prev = cur
        states.append(cur)
        fields.append(field)
        for i in range(n_sys):
            post = ctls[i](step)[1] if ctls[i] is not None else None
            if post is not None:
                vs[i] = vs[i] @ np.asarray(post, CDT).T
        deriv = field_eom(t, cur, field)
        for i in range(n_sys):
            p1, p2 = propagators_list[i](step, field, deriv)
            mpos, caps, tin, tout = pts[i]
            v = vs[i] @ np.asarray(p1, CDT).T
            v = np.einsum("la,lrab->rb", v, pt_mpo_rank4(mpos[step], tin, tout))
            vs[i] = v @ np.asarray(p2, CDT).T
    final = [read(i, num_steps) for i in range(n_sys)]
    states.append(final)
    fields.append(compute_field(start_time + num_steps * dt, prev, field, final))
    return states, fields


def gradient_pt(initial_state, propagators, mpo_tensors, caps, num_steps, target,
                transform_in=None, transform_out=None, controls=None):
    """``compute_gradient_and_dynamics`` with one process tensor
    (gradient.py:169-437; helpers system_dynamics.py:631-790).  Forward: the
    sweep of ``compute_dynamics_pt``, keeping the node after every step's
    post-measurement control (the forward derivative tensor ``F_n[l, a]``).
    Backward: the target (a ``D`` vector, bond 1) through the step's
    pre-measurement control transposed, then per step N-1 .. 1 through
    ``P2^T``, the MPO with bond and system legs swapped, ``P1^T`` and the
    post- and pre-measurement controls transposed (``B_n[r, e]``).  Returns
    ``(derivs[num_steps, D, D, D, D], states[num_steps+1, D])`` with
    ``derivs[n][a, b, c, e] = sum_{l, r} F_n[l, a] MPO_n[l, r, b, c]
    B_{n+1}[r, e]``: the derivative of the target's overlap with respect to
    the half-step propagators around the MPO of step n."""
    rho = np.asarray(initial_state, dtype=CDT).reshape(-1)
    D = rho.size
    ctl = controls if controls is not None else (lambda s: (None, None))
    v = rho.reshape(1, D)
    states, fwd, mpos = [], [], []
    for step in range(num_steps + 1):
        pre, post = ctl(step)
        if pre is not None:
            v = v @ np.asarray(pre, CDT).T
        if step == num_steps:
            break
        states.append(np.einsum("ba,b->a", v, caps[step]))
        if post is not None:
            v = v @ np.asarray(post, CDT).T
        fwd.append(v.copy())
        p1, p2 = propagators(step)
        T = pt_mpo_rank4(mpo_tensors[step], transform_in, transform_out)
        mpos.append(T)
        v = v @ np.asarray(p1, CDT).T
        v = np.einsum("la,lrab->rb", v, T)
        v = v @ np.asarray(p2, CDT).T
    states.append(np.einsum("ba,b->a", v, caps[num_steps]))
    b = np.asarray(target, dtype=CDT).reshape(1, D)
    pre, _ = ctl(num_steps)
    if pre is not None:
        b = b @ np.asarray(pre, CDT)          # (pre^T b) as a row vector
    derivs = [None] * num_steps
    derivs[num_steps - 1] = np.einsum("la,lrbc,re->abce", fwd[num_steps - 1], mpos[num_steps - 1], b)
    for step in range(num_steps - 1, 0, -1):
        pre, post = ctl(step)
        p1, p2 = propagators(step)
        b = b @ np.asarray(p2, CDT)           # P2^T
        b = np.einsum("re,lrbe->lb", b, mpos[step])
        b = b @ np.asarray(p1, CDT)           # P1^T
        if post is not None:
            b = b @ np.asarray(post, CDT)
        if pre is not None:
            b = b @ np.asarray(pre, CDT)
        derivs[step - 1] = np.einsum("la,lrbc,re->abce", fwd[step - 1], mpos[step - 1], b)
    return np.array(derivs), np.array(states)


def correlations_nt_pt(initial_state, propagators, mpo_tensors, caps, operators,
                       op_steps, ops_order, transform_in=None, transform_out=None):
    """``compute_correlations_nt`` (system_dynamics.py:791-990) for operator
    time steps already parsed to integers: for every combination of the
    first n-1 operators' steps (time-ordered, else skipped), one
    ``compute_dynamics`` run with each of those operators as a
    pre-measurement control at its step (``left``: A rho, ``right``: rho A;
    operators.py:139-147), read out as the expectation of the last operator
    at every last-operator step not before the latest first step.  Returns
    the array ``[len(op_steps[0]), ..., len(op_steps[-1])]`` with NaN where
    the reference leaves NaN."""
    from itertools import product
    d = int(round(np.sqrt(np.asarray(initial_state).size)))
    eye = np.identity(d)
    sups = [np.kron(op, eye) if o == "left" else np.kron(eye, np.asarray(op).T)
            for op, o in zip(operators, ops_order)]
    out = np.full([len(t) for t in op_steps], np.nan + 1j * np.nan, dtype=CDT)
    last = np.asarray(op_steps[-1])
    for idx in product(*[range(len(t)) for t in op_steps[:-1]]):
        first = [int(op_steps[j][i]) for j, i in enumerate(idx)]
        if first != sorted(first):
            continue
        keep = np.flatnonzero(last >= max(first))
        if keep.size == 0:
            continue
        ctrl = {}
        for j, st in enumerate(first):
            ctrl[st] = sups[j] if st not in ctrl else sups[j] @ ctrl[st]
        nsteps = int(last[keep].max())
        states = compute_dynamics_pt(initial_state, propagators, mpo_tensors, caps, nsteps,
                                     transform_in, transform_out,
                                     controls=lambda s: (ctrl.get(s), None))
        op = np.asarray(operators[-1])
        for k in keep:
            rho = states[int(last[k])].reshape(d, d)
            out[idx + (k,)] = np.trace(op @ rho)
    return out


# ---------------------------------------------------------------------------
# observables
# ---------------------------------------------------------------------------

def trace_distance(rho_a: np.ndarray, rho_b: np.ndarray) -> float:
    """``0.5 * || rho_a - rho_b ||_1`` via the eigenvalues of the Hermitian
    part of the difference (the reference has no such function)."""
    d = int(round(np.sqrt(np.asarray(rho_a).size)))
    diff = np.asarray(rho_a).reshape(d, d) - np.asarray(rho_b).reshape(d, d)
    herm = 0.5 * (diff + diff.conj().T)
    return float(0.5 * np.sum(np.abs(np.linalg.eigvalsh(herm))))


def max_trace_distance(states_a, states_b) -> float:
    return max(trace_distance(a, b) for a, b in zip(states_a, states_b))
