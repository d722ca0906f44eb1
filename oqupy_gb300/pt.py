"""PT-TEMPO process tensors and the process-tensor sweep on the GPU.

``PtBatch`` builds many process tensors in one launch per call
(reference: PtTempoBackend, oqupy/backends/pt_tempo_backend.py:28-316).
``GpuPtTempoBackend`` is the drop-in for ``PtTempoBackend``.  Built tensors
stay on the device; ``compute_dynamics`` runs the sweep of
oqupy/system_dynamics.py:131-165 for many systems at once on one process
tensor (``PtBatch.dynamics``).
"""

import ctypes
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

from . import _native as nat

DEFAULT_CHI_CAP = 64


class PtBatch:
    """Process tensors built together on the GPU.

    ``instances``: dicts with ``hs_dim``, ``num_steps``, ``dkmax``,
    ``epsrel``, ``influences`` (``[num_infl, D, D]``, dk = 0..num_infl-1 with
    ``num_infl = min(num_steps, dkmax+1)``) and optionally
    ``neg_influences`` (``[num_steps+1, D, D]`` indexed by step: the
    grow-phase ``influence(-step)`` of ``add_correlation_time``).
    """

    def __init__(self, instances: Sequence[Dict], precision: str = "complex128",
                 chi_cap: int = DEFAULT_CHI_CAP, grid: int = 0, qr_cut: float = 0.0):
        L = nat.lib()
        if precision not in nat.PRECISION:
            raise ValueError(f"precision must be one of {list(nat.PRECISION)}")
        self.n = len(instances)
        if self.n == 0:
            raise ValueError("need at least one instance")
        arr = (nat.PtInstance * self.n)()
        keep = []
        self.meta = []
        for i, inst in enumerate(instances):
            d = int(inst["hs_dim"])
            D = d * d
            num_steps = int(inst["num_steps"])
            dkmax = int(inst["dkmax"])
            num_infl = min(num_steps, dkmax + 1)
            if num_infl < 2:
                raise ValueError("PT-TEMPO needs min(num_steps, dkmax+1) >= 2")
            infl = nat.cplx(np.asarray(inst["influences"])[:num_infl].reshape(num_infl, D, D))
            keep.append(infl)
            arr[i].hs_dim = d
            arr[i].num_steps = num_steps
            arr[i].dkmax = dkmax
            arr[i].epsrel = float(inst["epsrel"])
            arr[i].influences = nat.dptr(infl)
            neg = inst.get("neg_influences")
            if neg is not None:
                neg = nat.cplx(np.asarray(neg).reshape(num_steps + 1, D, D))
                keep.append(neg)
                arr[i].neg_influences = nat.dptr(neg)
            else:
                arr[i].neg_influences = None
            self.meta.append(dict(d=d, D=D, num_steps=num_steps))
        cfg = nat.PtConfig(nat.PRECISION[precision], int(chi_cap), int(grid), float(qr_cut))
        self.chi_cap = int(chi_cap)
        h = ctypes.c_void_p()
        nat.check(L.otb_pt_create(ctypes.byref(cfg), self.n, arr, ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            nat.lib().otb_pt_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def advance(self, nsteps: int, stream: Optional[int] = None):
        """Initialise (first call) and advance every build by ``nsteps``."""
        nat.check(nat.lib().otb_pt_advance(self._h, int(nsteps), ctypes.c_void_p(stream or 0)))

    def build(self):
        """Run every build to completion (computes the caps)."""
        n = max(m["num_steps"] for m in self.meta)
        self.advance(n)
        self.check_status()

    def info(self, i: int) -> Dict:
        inf = nat.PtInfo()
        nat.check(nat.lib().otb_pt_get_info(self._h, int(i), ctypes.byref(inf)))
        return {k: getattr(inf, k) for k, _ in nat.PtInfo._fields_}

    def check_status(self):
        for i in range(self.n):
            st = self.info(i)["status"]
            if st != 0:
                raise nat.DeviceError(st, f"process tensor {i}")

    def bond_dimensions(self, i: int) -> np.ndarray:
        N = self.meta[i]["num_steps"]
        buf = (ctypes.c_int32 * (N + 1))()
        nat.check(nat.lib().otb_pt_bond_dims(self._h, int(i), buf, N + 1))
        return np.array(buf[:], dtype=int)

    def mpo_tensor(self, i: int, step: int) -> np.ndarray:
        """Rank-3 tensor ``[past bond, future bond, D]`` of one step."""
        D = self.meta[i]["D"]
        capn = self.chi_cap * self.chi_cap * D
        out = np.zeros((capn, 2))
        dims = (ctypes.c_int32 * 2)()
        nat.check(nat.lib().otb_pt_get_tensor(self._h, int(i), int(step), nat.dptr(out),
                                              capn, dims))
        l, r = dims[0], dims[1]
        return out[: l * r * D].view(np.complex128)[:, 0].reshape(l, r, D).copy()

    def cap(self, i: int, step: int) -> np.ndarray:
        out = np.zeros((self.chi_cap, 2))
        cnt = ctypes.c_int32()
        nat.check(nat.lib().otb_pt_get_cap(self._h, int(i), int(step), nat.dptr(out),
                                           self.chi_cap, ctypes.byref(cnt)))
        return out[: cnt.value].view(np.complex128)[:, 0].copy()

    def dynamics(self, i: int, prop1, prop2, rho0, num_steps: Optional[int] = None,
                 transform_in=None, transform_out=None,
                 stream: Optional[int] = None) -> np.ndarray:
        """compute_dynamics for ``H`` systems on process tensor ``i``.

        ``prop1``, ``prop2``: ``[H, D, D]`` half-step propagators; ``rho0``:
        ``[H, d, d]`` or ``[H, D]``.  Returns states ``[num_steps+1, H, D]``."""
        D = self.meta[i]["D"]
        p1 = np.asarray(prop1, dtype=np.complex128).reshape(-1, D, D)
        p2 = np.asarray(prop2, dtype=np.complex128).reshape(-1, D, D)
        if transform_in is not None:
            p1 = np.einsum("xa,hxb->hab", np.asarray(transform_in), p1)
        if transform_out is not None:
            p2 = np.einsum("hab,yb->hay", p2, np.asarray(transform_out))
        H = p1.shape[0]
        r0 = np.asarray(rho0, dtype=np.complex128).reshape(H, D)
        n = self.meta[i]["num_steps"] if num_steps is None else int(num_steps)
        a1, a2, a3 = nat.cplx(p1), nat.cplx(p2), nat.cplx(r0)
        out = np.zeros((n + 1, H, D, 2))
        nat.check(nat.lib().otb_dyn_run(self._h, int(i), H, nat.dptr(a1), nat.dptr(a2),
                                        nat.dptr(a3), n, nat.dptr(out),
                                        ctypes.c_void_p(stream or 0)))
        return out.view(np.complex128)[..., 0]

    def dynamics_steps(self, i: int, props, prop_index, rho0, num_steps: int,
                       stream: Optional[int] = None) -> np.ndarray:
        """compute_dynamics for ``H`` systems whose propagators change per
        step (``otb_dyn_run_steps``).  ``props``: ``[n_props, 2, D, D]``
        pairs (transforms and control operations already folded in);
        ``prop_index``: ``[H, num_steps]`` pair of system h at step k;
        ``rho0``: ``[H, D]``.  Returns states ``[num_steps+1, H, D]``."""
        D = self.meta[i]["D"]
        tab = nat.cplx(np.asarray(props, dtype=np.complex128).reshape(-1, 2, D, D))
        n = int(num_steps)
        r0a = np.asarray(rho0, dtype=np.complex128).reshape(-1, D)
        H = r0a.shape[0]
        idx = np.zeros((H, max(n, 1)), dtype=np.int32)
        if n:
            idx[:] = np.asarray(prop_index, dtype=np.int32).reshape(H, n)
        r0 = nat.cplx(r0a)
        out = np.zeros((n + 1, H, D, 2))
        nat.check(nat.lib().otb_dyn_run_steps(
            self._h, int(i), H, nat.dptr(tab), int(tab.shape[0]),
            idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), nat.dptr(r0), n,
            nat.dptr(out), ctypes.c_void_p(stream or 0)))
        return out.view(np.complex128)[..., 0]

    def session(self, i: int, rho0) -> "DynSession":
        """A sweep over process tensor ``i`` advanced one step per call, for
        ``H`` systems starting at ``rho0`` ``[H, D]``."""
        return DynSession(self, i, rho0)

    def gradient_cores(self, i: int, props, prop_index, rho0, target, num_steps: int,
                       stream: Optional[int] = None):
        """Forward and adjoint sweeps of the gradient (``otb_dyn_gradient``)
        for ``H`` systems: ``props`` ``[n_props, 2, D, D]``, ``prop_index``
        ``[H, num_steps]``, ``rho0`` and ``target`` ``[H, D]``.  Returns
        ``(states[num_steps+1, H, D], cores[H, num_steps, D, D, D])``."""
        D = self.meta[i]["D"]
        tab = nat.cplx(np.asarray(props, dtype=np.complex128).reshape(-1, 2, D, D))
        n = int(num_steps)
        r0a = np.asarray(rho0, dtype=np.complex128).reshape(-1, D)
        H = r0a.shape[0]
        idx = np.ascontiguousarray(np.asarray(prop_index, dtype=np.int32).reshape(H, n))
        tg = nat.cplx(np.asarray(target, dtype=np.complex128).reshape(H, D))
        states = np.zeros((n + 1, H, D, 2))
        cores = np.zeros((H, n, D, D, D, 2))
        nat.check(nat.lib().otb_dyn_gradient(
            self._h, int(i), H, nat.dptr(tab), int(tab.shape[0]),
            idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), nat.dptr(nat.cplx(r0a)), nat.dptr(tg),
            n, nat.dptr(states), nat.dptr(cores), ctypes.c_void_p(stream or 0)))
        return states.view(np.complex128)[..., 0], cores.view(np.complex128)[..., 0]


class DynSession:
    """A process-tensor sweep advanced one step per call
    (``otb_dyn_session_*``), for sweeps whose next propagators depend on the
    states so far.  ``step(props)`` takes ``[H, 2, D, D]`` pairs (transforms
    and controls folded in) and returns the ``[H, D]`` states after the
    step."""

    def __init__(self, batch: "PtBatch", i: int, rho0):
        self.D = batch.meta[i]["D"]
        r0 = np.asarray(rho0, dtype=np.complex128).reshape(-1, self.D)
        self.n = r0.shape[0]
        self._batch = batch          # the process tensor outlives the session
        h = ctypes.c_void_p()
        nat.check(nat.lib().otb_dyn_session_create(batch._h, int(i), self.n, nat.dptr(nat.cplx(r0)),
                                                   ctypes.byref(h)))
        self._h = h

    def step(self, props, stream: Optional[int] = None) -> np.ndarray:
        tab = nat.cplx(np.asarray(props, dtype=np.complex128).reshape(self.n, 2, self.D, self.D))
        out = np.zeros((self.n, self.D, 2))
        nat.check(nat.lib().otb_dyn_session_step(self._h, nat.dptr(tab), nat.dptr(out),
                                                 ctypes.c_void_p(stream or 0)))
        return out.view(np.complex128)[..., 0]

    def state(self, step: int) -> np.ndarray:
        out = np.zeros((self.n, self.D, 2))
        nat.check(nat.lib().otb_dyn_session_state(self._h, int(step), nat.dptr(out)))
        return out.view(np.complex128)[..., 0]

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            nat.lib().otb_dyn_session_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuPtTempoBackend:
    """Drop-in for ``oqupy.backends.pt_tempo_backend.PtTempoBackend``
    (pt_tempo_backend.py:56-316): same constructor, ``step``/``num_steps``,
    ``initialize()``, ``compute_step() -> bool``, ``get_mpo_tensor(step)``,
    ``update_process_tensor()`` (host copies into the process tensor handed
    in, caps computed as in the reference).  ``device_process_tensor()``
    returns the build as a ``DeviceProcessTensor`` (``device_pt.py``) whose
    tensors stay on the GPU; ``PtTempo.get_process_tensor`` returns that once
    ``oqupy_gb300.install`` has run.

    ``config`` keys used: ``precision`` ("complex128" | "mixed"),
    ``chi_cap`` (initial bond capacity; a build whose bonds outgrow it is
    rebuilt with twice the capacity, up to 1152 / D), ``qr_cut``."""

    def __init__(self, dimension, influence: Callable[[int], np.ndarray], process_tensor,
                 sum_north, sum_west, num_steps, dkmax, epsrel, config: Dict,
                 degeneracy_maps=None):
        if degeneracy_maps is not None:
            raise NotImplementedError("the GPU PT-TEMPO engine needs unique=False")
        if not (np.allclose(sum_north, 1.0) and np.allclose(sum_west, 1.0)):
            raise NotImplementedError("the GPU PT-TEMPO engine needs all-ones sums")
        self._d = int(dimension)
        self._influence = influence
        self._process_tensor = process_tensor
        self._num_steps = int(num_steps)
        self._dkmax = int(dkmax)
        self._epsrel = float(epsrel)
        self._config = {} if config is None else config
        self._num_infl = min(self._num_steps, self._dkmax + 1)
        self._step = None
        self._batch: Optional[PtBatch] = None

    @property
    def step(self):
        return self._step

    @property
    def num_steps(self):
        return self._num_steps

    def initialize(self):
        infl = np.array([self._influence(k) for k in range(self._num_infl)],
                        dtype=np.complex128)
        neg = None
        # the grow phase (steps 2 .. num_steps - num_infl + 1) asks for the
        # dk = -step influences (pt_tempo_backend.py:236-263); without a grow
        # phase the reference never asks for them
        grows = self._num_infl < self._num_steps
        first_neg = self._influence(-2) if grows else None
        if first_neg is not None:
            D = self._d ** 2
            neg = np.zeros((self._num_steps + 1, D, D), dtype=np.complex128)
            last_grow = self._num_steps - self._num_infl + 1
            for s in range(2, last_grow + 1):
                m = self._influence(-s)
                if m is not None:
                    neg[s] = m
                else:
                    neg[s] = infl[-1]
        self._inst = dict(hs_dim=self._d, num_steps=self._num_steps, dkmax=self._dkmax,
                          epsrel=self._epsrel, influences=infl, neg_influences=neg)
        self._cap = int(self._config.get("chi_cap", DEFAULT_CHI_CAP))
        self._new_batch()
        self._batch.advance(0)
        self._step = 1
        self._check_grow()

    def _new_batch(self):
        if self._batch is not None:
            self._batch.close()
        self._batch = PtBatch([self._inst], precision=self._config.get("precision", "complex128"),
                              chi_cap=self._cap, grid=1,
                              qr_cut=float(self._config.get("qr_cut", 0.0)))

    def _check_grow(self):
        """A bond beyond the capacity stops the build on the device: rebuild
        with twice the capacity (up to 1152 / D) and replay the steps done so
        far (the build is deterministic, so the replay repeats them)."""
        while True:
            st = self._batch.info(0)["status"]
            if st == 0:
                return
            cap_max = nat.MAX_COLUMNS // (self._d * self._d)
            if st != nat.OTB_ERR_CHI_OVERFLOW or self._cap >= cap_max:
                raise nat.DeviceError(st, f"PT-TEMPO step {self._step}")
            self._cap = min(2 * self._cap, cap_max)
            self._new_batch()
            self._batch.advance(self._step - 1)      # initialise, then replay

    def compute_step(self) -> bool:
        self._batch.advance(1)
        self._step += 1
        self._check_grow()
        return self._step < self._num_steps

    def get_mpo_tensor(self, step: int) -> np.ndarray:
        return self._batch.mpo_tensor(0, step)

    def update_process_tensor(self) -> None:
        self._batch.check_status()
        for step in reversed(range(self._num_steps)):
            self._process_tensor.set_mpo_tensor(step, self.get_mpo_tensor(step))
        self._process_tensor.compute_caps()

    def device_process_tensor(self, base_cls=None):
        """The build as a ``DeviceProcessTensor`` with the dt, transforms,
        name and description of the process tensor handed in; ``base_cls``
        is the reference's ``BaseProcessTensor`` (default: the base class of
        that process tensor's class hierarchy)."""
        from .device_pt import device_process_tensor_class
        self._batch.check_status()
        pt = self._process_tensor
        if base_cls is None:
            base_cls = next(c for c in type(pt).__mro__ if c.__name__ == "BaseProcessTensor")
        cls = device_process_tensor_class(base_cls)
        return cls(self._batch, 0, pt.hilbert_space_dimension, pt.dt, pt.transform_in,
                   pt.transform_out, getattr(pt, "name", None), getattr(pt, "description", None))


def device_compute_dynamics(process_tensor, propagator_pairs, initial_states,
                            num_steps: Optional[int] = None) -> np.ndarray:
    """GPU sweep for several systems on a ``DeviceProcessTensor`` (or a
    ``(PtBatch, index)`` pair).  ``propagator_pairs``: list of ``(P1, P2)``;
    returns ``[num_steps+1, H, D]`` states."""
    if isinstance(process_tensor, tuple):
        batch, idx = process_tensor
        tin = tout = None
    else:
        batch, idx = process_tensor.device
        tin, tout = process_tensor.transform_in, process_tensor.transform_out
    p1 = np.array([p[0] for p in propagator_pairs])
    p2 = np.array([p[1] for p in propagator_pairs])
    return batch.dynamics(idx, p1, p2, np.asarray(initial_states), num_steps,
                          transform_in=tin, transform_out=tout)
