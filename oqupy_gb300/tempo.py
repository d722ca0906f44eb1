"""Batched TEMPO on the GPU and the drop-in ``TempoBackend`` replacement.

``TempoBatch`` advances many independent TEMPO instances (different
couplings, temperatures, memory lengths and bond dimensions) in one CUDA
launch per call.  ``GpuTempoBackend`` has the constructor and methods of the
reference's ``TempoBackend`` (oqupy/backends/tempo_backend.py:577-626) and
runs one instance through the same C ABI, so ``oqupy.Tempo`` can use it
unchanged (see ``oqupy_gb300.install``).
"""

import ctypes
from copy import copy
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

from . import _native as nat

DEFAULT_CHI_CAP = 64


def super_unitaries(unitary: np.ndarray):
    """``(super_u, super_u_dagg)`` of tempo_backend.py:383-388:
    ``left_right_super(U, U^dag)`` and ``left_right_super(U^dag, U)``
    (operators.py:149-153, ``kron(left, right.T)``)."""
    u = np.asarray(unitary, dtype=np.complex128)
    ud = u.conjugate().T
    return np.kron(u, ud.T), np.kron(ud, u.T)


def identity_mask(unitaries, d: int) -> np.ndarray:
    """Per instance: is the coupling eigenbasis the identity (np.allclose
    semantics, as fold_propagators tests it)?  One vectorised test for a
    batch of d x d unitaries (None counts as the identity)."""
    n = len(unitaries)
    mask = np.array([u is None for u in unitaries], dtype=bool)
    rest = [i for i in range(n) if not mask[i]]
    if rest:
        U = np.stack([np.asarray(unitaries[i], dtype=np.complex128) for i in rest])
        eye = np.identity(d)
        mask[rest] = np.all(np.abs(U - eye) <= 1e-8 + 1e-5 * np.abs(eye), axis=(1, 2))
    return mask


def fold_propagators(prop1, prop2, unitary=None):
    """Fold the coupling-eigenbasis rotation that the reference attaches to
    the dk=0 influence tensor (tempo_backend.py:419-424) into the half-step
    propagators: ``P1 <- super_u_dagg P1`` and ``P2 <- P2 super_u``.  The
    engine then works with diagonal dk=0 influences only."""
    p1 = np.asarray(prop1, dtype=np.complex128)
    p2 = np.asarray(prop2, dtype=np.complex128)
    if unitary is None or np.allclose(unitary, np.identity(len(unitary))):
        return p1, p2
    su, sud = super_unitaries(unitary)
    return sud @ p1, p2 @ su


class TempoBatch:
    """Many TEMPO instances advanced together on the GPU.

    Parameters
    ----------
    instances: sequence of dicts with keys
        ``hs_dim`` (d), ``dkmax`` (int, or None for full memory),
        ``epsrel``, ``influences`` (array ``[n, D, D]``, dk = 0..n-1, in the
        coupling eigenbasis; ``influence_matrix`` output of the reference),
        ``prop1``, ``prop2`` (``D x D`` half-step propagators),
        ``rho0`` (``d x d`` or ``D``), optional ``unitary`` (coupling
        eigenvectors; folded into the propagators).
    precision: ``"complex128"`` or ``"mixed"``.
    chi_cap: bond-dimension capacity of every site slot.
    out_cap: number of recent states kept per instance on the device.
    qr_cut: relative cut of the rank-revealing QR in every bond split
        (0 = the precision form's default; ``otb_tempo_config.qr_cut``).
    """

    def __init__(self, instances: Sequence[Dict], precision: str = "complex128",
                 chi_cap: int = DEFAULT_CHI_CAP, out_cap: int = 2, grid: int = 0,
                 max_sites: int = 0, block: int = 0, smem_kb: int = 0, qr_cut: float = 0.0):
        L = nat.lib()
        if precision not in nat.PRECISION:
            raise ValueError(f"precision must be one of {list(nat.PRECISION)}")
        self.precision = precision
        self.n = len(instances)
        if self.n == 0:
            raise ValueError("need at least one instance")
        self._keep = []
        arr = (nat.TempoInstance * self.n)()
        self.D = []
        for i, inst in enumerate(instances):
            d = int(inst["hs_dim"])
            D = d * d
            infl = nat.cplx(np.asarray(inst["influences"]).reshape(-1, D, D))
            p1, p2 = fold_propagators(inst["prop1"], inst["prop2"],
                                      inst.get("unitary"))
            p1, p2 = nat.cplx(p1), nat.cplx(p2)
            rho0 = nat.cplx(np.asarray(inst["rho0"]).reshape(D))
            self._keep += [infl, p1, p2, rho0]
            dk = inst.get("dkmax")
            arr[i].hs_dim = d
            arr[i].dkmax = -1 if dk is None else int(dk)
            arr[i].epsrel = float(inst["epsrel"])
            arr[i].n_influences = infl.shape[0]
            arr[i].influences = nat.dptr(infl)
            arr[i].prop1 = nat.dptr(p1)
            arr[i].prop2 = nat.dptr(p2)
            arr[i].rho0 = nat.dptr(rho0)
            arr[i].max_sites = int(max_sites)
            self.D.append(D)
        cfg = nat.TempoConfig(nat.PRECISION[precision], int(chi_cap),
                              int(out_cap), int(grid), int(block), int(smem_kb),
                              float(qr_cut))
        self.out_cap = int(out_cap)
        self.chi_cap = int(chi_cap)
        h = ctypes.c_void_p()
        nat.check(L.otb_tempo_create(ctypes.byref(cfg), self.n, arr, ctypes.byref(h)))
        self._h = h
        self._keep = []

    # -- lifetime --------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            nat.lib().otb_tempo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- stepping --------------------------------------------------------
    def advance(self, nsteps: int = 1, stream: Optional[int] = None):
        """Advance every instance by ``nsteps`` TEMPO steps (asynchronous
        on ``stream``; status is checked when results are read)."""
        nat.check(nat.lib().otb_tempo_advance(self._h, int(nsteps),
                                               ctypes.c_void_p(stream or 0)))

    def info(self, i: int) -> Dict:
        inf = nat.TempoInfo()
        nat.check(nat.lib().otb_tempo_get_info(self._h, int(i), ctypes.byref(inf)))
        return {"step": inf.step, "status": inf.status, "nsites": inf.nsites,
                "max_bond": inf.max_bond, "log_scale": inf.log_scale,
                "splits": inf.splits, "sweeps64": inf.sweeps64,
                "sweeps32": inf.sweeps32, "flops_alg": inf.flops_alg,
                "t_begin_ns": inf.t_begin_ns, "t_end_ns": inf.t_end_ns}

    def timeline(self) -> np.ndarray:
        """(n, 2) device-clock ns at which the last launch's CTA took each
        instance and finished it: the launch's critical path is the instance
        that ends last, its load balance the spread of the end times."""
        out = np.zeros((self.n, 2), dtype=np.int64)
        for i in range(self.n):
            inf = self.info(i)
            out[i] = (inf["t_begin_ns"], inf["t_end_ns"])
        return out

    def check_status(self):
        for i in range(self.n):
            st = self.info(i)["status"]
            if st != 0:
                raise nat.DeviceError(st, f"instance {i}")

    def states(self, first: int = 0, count: Optional[int] = None) -> np.ndarray:
        """States of steps ``[first, first+count)`` for all instances as a
        complex array ``[n, count, D]`` (uniform D) or a list."""
        if count is None:
            count = self.info(0)["step"] + 1 - first
        if len(set(self.D)) == 1:
            out = np.zeros((self.n, count, self.D[0], 2))
            nat.check(nat.lib().otb_tempo_read_all_states(
                self._h, int(first), int(count), nat.dptr(out)))
            return out.view(np.complex128)[..., 0]
        res = []
        for i in range(self.n):
            res.append(self.instance_states(i, first, count))
        return res

    def instance_states(self, i: int, first: int, count: int) -> np.ndarray:
        out = np.zeros((count, self.D[i], 2))
        nat.check(nat.lib().otb_tempo_read_states(self._h, int(i), int(first),
                                                  int(count), nat.dptr(out)))
        return out.view(np.complex128)[..., 0]

    def bond_dims(self, i: int) -> List[int]:
        buf = (ctypes.c_int32 * 4096)()
        cnt = ctypes.c_int32()
        nat.check(nat.lib().otb_tempo_bond_dims(self._h, int(i), buf, 4096,
                                                ctypes.byref(cnt)))
        return list(buf[:cnt.value])

    # -- per-step inputs (drop-in backend) ---------------------------------
    def set_influence(self, i: int, dk: int, mat):
        m = nat.cplx(mat)
        nat.check(nat.lib().otb_tempo_set_influence(self._h, int(i), int(dk), nat.dptr(m)))

    def set_propagators(self, i: int, p1, p2, unitary=None):
        a, b = fold_propagators(p1, p2, unitary)
        a, b = nat.cplx(a), nat.cplx(b)
        nat.check(nat.lib().otb_tempo_set_propagators(self._h, int(i), nat.dptr(a), nat.dptr(b)))

    def set_all_propagators(self, p1s, p2s, unitaries=None, stream: Optional[int] = None):
        """Propagators of every instance for the next step in one call.
        ``p1s``, ``p2s``: ``[n, D, D]`` (uniform D) or sequences; optional
        coupling eigenbases ``unitaries`` are folded in as for
        ``set_propagators``."""
        if unitaries is None:
            unitaries = [None] * self.n
        uniform = len(set(self.D)) == 1
        if uniform and identity_mask(unitaries, int(round(np.sqrt(self.D[0])))).all():
            # identity eigenbases: the fold is the identity, the batch is packed as given
            a = nat.cplx(np.asarray(p1s).reshape(self.n, self.D[0], self.D[0]))
            b = nat.cplx(np.asarray(p2s).reshape(self.n, self.D[0], self.D[0]))
        else:
            folded = [fold_propagators(x, y, u) for x, y, u in zip(p1s, p2s, unitaries)]
            a = nat.cplx(np.concatenate([np.asarray(f[0]).reshape(-1) for f in folded]))
            b = nat.cplx(np.concatenate([np.asarray(f[1]).reshape(-1) for f in folded]))
        self._staged = (a, b)          # alive until the (possibly asynchronous) copy ran
        nat.check(nat.lib().otb_tempo_set_all_propagators(self._h, nat.dptr(a), nat.dptr(b),
                                                          ctypes.c_void_p(stream or 0)))

    def set_first_influence(self, i: int, mat=None):
        if mat is None:
            nat.check(nat.lib().otb_tempo_set_first_influence(self._h, int(i), None))
        else:
            m = nat.cplx(mat)
            nat.check(nat.lib().otb_tempo_set_first_influence(self._h, int(i), nat.dptr(m)))

    def set_launch(self, block: int = 0, smem_kb: int = 0, grid: int = 0):
        """Launch shape of the next ``advance`` calls (``otb_tempo_set_launch``)."""
        nat.check(nat.lib().otb_tempo_set_launch(self._h, int(block), int(smem_kb), int(grid)))

    def max_bond(self) -> int:
        """Largest bond dimension over the instances (synchronises)."""
        return max(self.info(i)["max_bond"] for i in range(self.n))

    def reserve_sites(self, nslots: int):
        nat.check(nat.lib().otb_tempo_reserve_sites(self._h, int(nslots)))


class GpuTempoBackend:
    """Drop-in for ``oqupy.backends.tempo_backend.TempoBackend``
    (tempo_backend.py:577-626): same constructor, ``step`` property,
    ``initialize() -> (0, state)`` and ``compute_step() -> (step, state)``.

    ``config`` keys used: ``precision`` ("complex128" | "mixed"), ``block`` /
    ``smem_kb`` (launch shape, default 512 threads and 200 KiB), ``chi_cap``
    (initial bond capacity; a step whose bonds outgrow it is redone with
    twice the capacity, up to 1152 / D, after replaying the earlier steps on
    a fresh handle -- the engine is deterministic, so the replay repeats
    them), ``qr_cut``.  Degeneracy maps (``unique=True``) are not supported by
    the GPU engine; ``oqupy_gb300.install`` routes such runs to the reference
    backend.
    """

    def __init__(self, initial_state, influence: Callable[[int], np.ndarray],
                 unitary_transform, propagators, sum_north, sum_west, dkmax,
                 epsrel, config: Optional[Dict] = None, degeneracy_maps=None,
                 dim=None):
        if degeneracy_maps is not None:
            raise NotImplementedError("the GPU TEMPO engine needs unique=False")
        if not (np.allclose(sum_north, 1.0) and np.allclose(sum_west, 1.0)):
            raise NotImplementedError("the GPU TEMPO engine needs all-ones sums")
        self._initial_state = np.array(initial_state, dtype=np.complex128).reshape(-1)
        self._influence = influence
        self._unitary = np.asarray(unitary_transform, dtype=np.complex128)
        self._propagators = propagators
        self._dkmax = dkmax
        self._epsrel = epsrel
        self._config = {} if config is None else config
        self._step = None
        self._batch: Optional[TempoBatch] = None
        self._last_props = None
        self._ninfl = 0
        self._slots = 16

    @property
    def step(self):
        return self._step

    def bond_dimensions(self) -> List[int]:
        """Bond dimensions of the current MPS (sites - 1 values)."""
        return self._batch.bond_dims(0)

    @property
    def chi_cap(self) -> int:
        """Current bond capacity of the device handle."""
        return self._cap

    def initialize(self):
        D = self._initial_state.size
        d = int(round(np.sqrt(D)))
        n = 1 if self._dkmax is None else self._dkmax + 1
        infl = np.array([self._influence(dk) for dk in range(n)],
                        dtype=np.complex128)
        p1, p2 = self._propagators(0)
        self._inst = dict(hs_dim=d, dkmax=self._dkmax, epsrel=self._epsrel,
                          influences=infl, prop1=np.array(p1), prop2=np.array(p2),
                          rho0=self._initial_state, unitary=self._unitary)
        self._cap = max(int(self._config.get("chi_cap", DEFAULT_CHI_CAP)), D)
        self._cap_max = nat.MAX_COLUMNS // D
        self._new_batch()
        self._step = 0
        return self._step, copy(self._initial_state)

    def _new_batch(self):
        if self._batch is not None:
            self._batch.close()
        inst = self._inst
        # one instance on one CTA: the widest CTA (512 threads) with the
        # largest shared-memory share
        self._batch = TempoBatch(
            [inst], precision=self._config.get("precision", "complex128"),
            chi_cap=self._cap, out_cap=4, grid=1,
            max_sites=16 if self._dkmax is None else 0,
            block=int(self._config.get("block", 512)), smem_kb=int(self._config.get("smem_kb", 200)),
            qr_cut=float(self._config.get("qr_cut", 0.0)))
        self._ninfl = len(inst["influences"])
        self._last_props = (inst["prop1"], inst["prop2"])
        self._slots = 16

    def _advance(self, step: int) -> int:
        """Inputs of ``step`` (propagators, influences of a growing memory,
        the first-site influence past dkmax), one engine step; returns the
        instance's status."""
        b = self._batch
        p1, p2 = self._propagators(step - 1)
        if not (np.array_equal(p1, self._last_props[0])
                and np.array_equal(p2, self._last_props[1])):
            b.set_propagators(0, p1, p2, self._unitary)
            self._last_props = (np.array(p1), np.array(p2))
        if self._dkmax is None:
            # the window of step s holds dk = 0 .. s-1 (tempo_backend.py:487-497)
            while self._ninfl < step:
                b.set_influence(0, self._ninfl, self._influence(self._ninfl))
                self._ninfl += 1
            need = step + 2
            if b.info(0)["nsites"] + 2 > self._slots:
                self._slots = max(2 * self._slots, need)
                b.reserve_sites(self._slots)
        elif step > self._dkmax:
            neg = self._influence(self._dkmax - step)
            if neg is not None:
                b.set_first_influence(0, neg)
        b.advance(1)
        return b.info(0)["status"]

    def compute_step(self):
        step = self._step + 1
        st = self._advance(step)
        while st == nat.OTB_ERR_CHI_OVERFLOW and self._cap < self._cap_max:
            self._cap = min(2 * self._cap, self._cap_max)
            self._new_batch()
            for s in range(1, step + 1):
                st = self._advance(s)
                if st != 0:
                    break
        if st != 0:
            raise nat.DeviceError(st, f"TEMPO step {step}")
        state = self._batch.instance_states(0, step, 1)[0]
        self._step = step
        return self._step, state
