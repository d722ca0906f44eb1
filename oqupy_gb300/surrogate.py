"""Learned screening surrogate for batched TEMPO parameter sweeps.

An MLP maps (alpha, omega_c, T, Omega, epsilon) of a spin-boson model
(H = Omega/2 sigma_x + epsilon/2 sigma_z, bath sigma_z/2, ohmic exponential
cutoff) to the Bloch-vector trajectory (x, y, z) over ``nsteps`` steps.  It
is trained on trajectories that the batched TEMPO solver (``TempoBatch``)
generates, with hand-written kernels: BF16 GEMMs on the 5th-generation tensor
cores (``otb_mlp_gemm``, tcgen05), fused bias / GELU / GELU-gradient
epilogues, bias-gradient column sums, the MSE gradient and AdamW on FP32
master weights.  Device memory comes from torch; every arithmetic operation
of training and inference runs in ``liboqupy_gb300.so``.

Screening: a point outside the training box, or in a region of parameter
space whose validation error exceeds the stated budget, falls back to the
TEMPO solve; the surrogate answers the rest.
"""

import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _native as nat
from .bath import half_step_propagators, influences
from .tempo import TempoBatch

BOX = {"alpha": (0.01, 0.5), "wc": (1.0, 10.0), "T": (0.0, 5.0),
       "Omega": (0.5, 2.0), "eps": (-1.0, 1.0)}
KEYS = ["alpha", "wc", "T", "Omega", "eps"]


def _torch():
    import torch
    return torch


class Mlp:
    """``sizes[0] -> GELU hidden layers -> sizes[-1]``, BF16 compute, FP32
    master weights, AdamW."""

    def __init__(self, sizes: Sequence[int], seed: int = 0, device: str = "cuda:0"):
        torch = _torch()
        self.torch = torch
        self.sizes = list(sizes)
        self.dev = torch.device(device)
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.W, self.b, self.m, self.v, self.mb, self.vb = [], [], [], [], [], []
        for fin, fout in zip(self.sizes[:-1], self.sizes[1:]):
            w = torch.randn(fout, fin, generator=g) * (2.0 / fin) ** 0.5
            self.W.append(w.to(self.dev).contiguous())
            self.b.append(torch.zeros(fout, device=self.dev))
            self.m.append(torch.zeros(fout, fin, device=self.dev))
            self.v.append(torch.zeros(fout, fin, device=self.dev))
            self.mb.append(torch.zeros(fout, device=self.dev))
            self.vb.append(torch.zeros(fout, device=self.dev))
        self.Wb = [torch.empty(w.shape, dtype=torch.bfloat16, device=self.dev) for w in self.W]
        self.WbT = [torch.empty((w.shape[1], w.shape[0]), dtype=torch.bfloat16, device=self.dev)
                    for w in self.W]
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.steps = 0
        for l in range(len(self.W)):
            self._refresh(l)

    # -- primitives -------------------------------------------------------
    def _p(self, t):
        return None if t is None else t.data_ptr()

    def _gemm(self, A, B, M, N, K, bias=None, epi=0, zin=None, zout=None, outf=None, outb=None):
        nat.check(nat.lib().otb_mlp_gemm(self._p(A), self._p(B), M, N, K, self._p(bias), epi,
                                         self._p(zin), self._p(zout), self._p(outf), self._p(outb),
                                         self._p(self.err), None))

    def _transpose(self, x):
        R, C = x.shape
        out = self.torch.empty((C, R), dtype=self.torch.bfloat16, device=self.dev)
        nat.check(nat.lib().otb_mlp_transpose_bf16(x.data_ptr(), out.data_ptr(), R, C, None))
        return out

    def _refresh(self, l):
        nat.check(nat.lib().otb_mlp_f32_to_bf16(self.W[l].data_ptr(), self.Wb[l].data_ptr(),
                                                self.W[l].numel(), None))
        w = self.Wb[l]
        nat.check(nat.lib().otb_mlp_transpose_bf16(w.data_ptr(), self.WbT[l].data_ptr(),
                                                   w.shape[0], w.shape[1], None))

    # -- passes -----------------------------------------------------------
    def forward(self, X, keep: bool = False):
        """X: [B, sizes[0]] (FP32 or bf16, device).  Returns Y [B, sizes[-1]]
        FP32; with ``keep`` the pre-activations and activations are kept for
        ``backward``."""
        torch = self.torch
        H = X.to(torch.bfloat16).contiguous()
        Bn = H.shape[0]
        Hs, Zs = [H], []
        L = len(self.W)
        for l in range(L):
            fout, fin = self.W[l].shape
            if l < L - 1:
                Z = torch.empty((Bn, fout), device=self.dev) if keep else None
                Hn = torch.empty((Bn, fout), dtype=torch.bfloat16, device=self.dev)
                self._gemm(H, self.Wb[l], Bn, fout, fin, bias=self.b[l], epi=1, zout=Z, outb=Hn)
                H = Hn
                if keep:
                    Zs.append(Z)
                    Hs.append(H)
            else:
                Y = torch.empty((Bn, fout), device=self.dev)
                self._gemm(H, self.Wb[l], Bn, fout, fin, bias=self.b[l], epi=0, outf=Y)
        if keep:
            self._cache = (Zs, Hs)
        return Y

    def loss_and_grads(self, X, T, loss=None):
        """Parameter gradients (FP32) of the MSE loss for a batch.  The sum of
        squared errors is added to the device scalar ``loss`` (FP64, one
        element; a fresh one when None), which is returned with the
        gradients: reading it is the only host synchronisation."""
        torch = self.torch
        Y = self.forward(X, keep=True)
        Zs, Hs = self._cache
        n = Y.numel()
        dZf = torch.empty_like(Y)
        dZb = torch.empty(Y.shape, dtype=torch.bfloat16, device=self.dev)
        if loss is None:
            loss = torch.zeros(1, dtype=torch.float64, device=self.dev)
        nat.check(nat.lib().otb_mlp_mse_grad(Y.data_ptr(), T.contiguous().data_ptr(), dZf.data_ptr(),
                                             dZb.data_ptr(), n, loss.data_ptr(), None))
        Bn = Y.shape[0]
        gW, gb = [None] * len(self.W), [None] * len(self.W)
        for l in reversed(range(len(self.W))):
            fout, fin = self.W[l].shape
            gW[l] = torch.empty((fout, fin), device=self.dev)
            self._gemm(self._transpose(dZb), self._transpose(Hs[l]), fout, fin, Bn, outf=gW[l])
            gb[l] = torch.empty(fout, device=self.dev)
            nat.check(nat.lib().otb_mlp_colsum(dZf.data_ptr(), gb[l].data_ptr(), Bn, fout, None))
            if l > 0:
                nf = torch.empty((Bn, fin), device=self.dev)
                nb = torch.empty((Bn, fin), dtype=torch.bfloat16, device=self.dev)
                self._gemm(dZb, self.WbT[l], Bn, fin, fout, epi=2, zin=Zs[l - 1], outf=nf, outb=nb)
                dZf, dZb = nf, nb
        self._cache = None
        return loss, gW, gb

    def step(self, gW, gb, lr=1e-3, weight_decay=0.0, beta1=0.9, beta2=0.999, eps=1e-8):
        self.steps += 1
        L = nat.lib()
        for l in range(len(self.W)):
            nat.check(L.otb_mlp_adamw(self.W[l].data_ptr(), gW[l].data_ptr(), self.m[l].data_ptr(),
                                      self.v[l].data_ptr(), self.Wb[l].data_ptr(), self.W[l].numel(),
                                      lr, beta1, beta2, eps, weight_decay, self.steps, None))
            nat.check(L.otb_mlp_adamw(self.b[l].data_ptr(), gb[l].data_ptr(), self.mb[l].data_ptr(),
                                      self.vb[l].data_ptr(), None, self.b[l].numel(), lr, beta1, beta2,
                                      eps, 0.0, self.steps, None))
            w = self.Wb[l]
            nat.check(L.otb_mlp_transpose_bf16(w.data_ptr(), self.WbT[l].data_ptr(), w.shape[0],
                                               w.shape[1], None))

    def check_errors(self):
        if int(self.err.item()) != 0:
            raise nat.DeviceError(nat.OTB_ERR_TIMEOUT, "tensor-core completion wait timed out")


# ---------------------------------------------------------------------------
# data from the batched TEMPO solver
# ---------------------------------------------------------------------------

def sample_params(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(*BOX[k], size=n) for k in KEYS], axis=1)


def tempo_instances(params: np.ndarray, dt: float, dkmax: int, epsrel: float) -> List[Dict]:
    sx = np.array([[0, 1], [1, 0]], dtype=complex)
    sz = np.diag([1.0, -1.0]).astype(complex)
    out = []
    for a, wc, T, om, ep in params:
        infl, U = influences(a, 1.0, wc, "exponential", T, dt, dkmax, 0.5 * sz)
        p1, p2 = half_step_propagators(0.5 * om * sx + 0.5 * ep * sz, dt)
        out.append(dict(hs_dim=2, dkmax=dkmax, epsrel=epsrel, influences=infl, prop1=p1,
                        prop2=p2, rho0=np.diag([1.0, 0.0]).astype(complex), unitary=U))
    return out


def bloch(states: np.ndarray) -> np.ndarray:
    """[..., 4] vectorised density matrices -> [..., 3] Bloch vectors."""
    r01 = states[..., 1]
    return np.stack([2 * r01.real, -2 * r01.imag, (states[..., 0] - states[..., 3]).real], axis=-1)


def free_bloch(params: np.ndarray, nsteps: int, dt: float = 0.05) -> np.ndarray:
    """Bloch trajectories [N, 3, nsteps] (steps 1..nsteps) of the system
    without the bath: precession of (0, 0, 1) about (Omega, 0, eps) at
    angular frequency sqrt(Omega^2 + eps^2) (Rodrigues' rotation)."""
    p = np.asarray(params)
    om, ep = p[:, 3], p[:, 4]
    w = np.sqrt(om ** 2 + ep ** 2)
    n = np.stack([om / w, np.zeros_like(om), ep / w], axis=1)          # axis
    t = dt * np.arange(1, nsteps + 1)
    th = w[:, None] * t[None, :]                                         # [N, T]
    v = np.array([0.0, 0.0, 1.0])
    ndv = n @ v                                                          # [N]
    cross = np.cross(n, v)                                               # [N, 3]
    out = (v[None, :, None] * np.cos(th)[:, None, :]
           + cross[:, :, None] * np.sin(th)[:, None, :]
           + (n * ndv[:, None])[:, :, None] * (1.0 - np.cos(th))[:, None, :])
    return out


def tempo_bloch(params: np.ndarray, nsteps: int, dt: float = 0.05, dkmax: int = 8,
                epsrel: float = 1e-6, precision: str = "mixed", chi_cap: int = 64,
                chunk: int = 4096) -> Tuple[np.ndarray, float]:
    """Bloch trajectories [N, 3, nsteps] (steps 1..nsteps) from the batched
    TEMPO solver (``chunk`` instances per batch) and the seconds it took."""
    out = np.empty((len(params), 3, nsteps))
    total = 0.0
    for c0 in range(0, len(params), chunk):
        part = params[c0:c0 + chunk]
        b = TempoBatch(tempo_instances(part, dt, dkmax, epsrel), precision=precision,
                       chi_cap=chi_cap, out_cap=nsteps + 1)
        t0 = time.perf_counter()
        b.advance(nsteps)
        st = b.states(1, nsteps)
        total += time.perf_counter() - t0
        b.check_status()
        b.close()
        out[c0:c0 + len(part)] = np.transpose(bloch(st), (0, 2, 1))
    return out, total


# ---------------------------------------------------------------------------
# surrogate with fallback
# ---------------------------------------------------------------------------

class Surrogate:
    """MLP screening model with a validation-calibrated error map and TEMPO
    fallback (see the module docstring)."""

    def __init__(self, nsteps: int = 500, hidden: Sequence[int] = (512, 512, 512, 512),
                 dt: float = 0.05, dkmax: int = 8, epsrel: float = 1e-6, seed: int = 0,
                 bins: int = 4, chi_cap: int = 64, residual: bool = True):
        self.nsteps, self.dt, self.dkmax, self.epsrel = nsteps, dt, dkmax, epsrel
        self.chi_cap = chi_cap
        # learn the bath's correction to the closed-system precession
        self.residual = residual
        self.net = Mlp([5] + list(hidden) + [3 * nsteps], seed=seed)
        self.bins = bins
        self.err_map = None
        self.lo = np.array([BOX[k][0] for k in KEYS])
        self.hi = np.array([BOX[k][1] for k in KEYS])

    def _x(self, params):
        torch = self.net.torch
        z = 2.0 * (np.asarray(params) - self.lo) / (self.hi - self.lo) - 1.0
        return torch.tensor(z, dtype=torch.float32, device=self.net.dev)

    def fit(self, params, traj, epochs: int = 200, batch: int = 256, lr: float = 2e-3,
            lr_final: float = 5e-5, weight_decay: float = 0.0, seed: int = 0) -> List[float]:
        torch = self.net.torch
        X = self._x(params)
        tgt = np.asarray(traj)
        if self.residual:
            tgt = tgt - free_bloch(params, self.nsteps, self.dt)
        T = torch.tensor(tgt.reshape(len(params), -1), dtype=torch.float32, device=self.net.dev)
        n = X.shape[0]
        rng = np.random.default_rng(seed)
        losses = []
        total = epochs * max(1, n // batch)
        it = 0
        nb = max(1, n // batch)
        for ep in range(epochs):
            perm = torch.tensor(rng.permutation(n), device=self.net.dev)
            acc = torch.zeros(1, dtype=torch.float64, device=self.net.dev)
            for k in range(nb):
                idx = perm[k * batch:(k + 1) * batch]
                lr_t = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * it / total))
                _, gW, gb = self.net.loss_and_grads(X[idx], T[idx], acc)
                self.net.step(gW, gb, lr=lr_t, weight_decay=weight_decay)
                it += 1
            losses.append(float(acc.item()) / (nb * min(batch, n) * T.shape[1]))
        self.net.check_errors()
        return losses

    def predict(self, params) -> np.ndarray:
        """Bloch trajectories [N, 3, nsteps] (float32) for ``params``."""
        torch = self.net.torch
        p = np.asarray(params)
        Y = self.net.forward(self._x(p))
        if self.residual:
            oe = torch.tensor(p[:, 3:5], dtype=torch.float32, device=self.net.dev)
            nat.check(nat.lib().otb_mlp_bloch_free_add(Y.data_ptr(), oe.data_ptr(), len(p), self.nsteps,
                                                       float(self.dt), None))
        return Y.cpu().numpy().reshape(len(p), 3, self.nsteps)

    def _bin(self, params):
        p = np.asarray(params)
        u = (p[:, [0, 2]] - self.lo[[0, 2]]) / (self.hi[[0, 2]] - self.lo[[0, 2]])
        ij = np.clip((u * self.bins).astype(int), 0, self.bins - 1)
        return ij[:, 0] * self.bins + ij[:, 1]

    def calibrate(self, params, traj):
        """Per-region (alpha x T bins) maximum Bloch error on validation data."""
        err = np.abs(self.predict(params) - np.asarray(traj)).max(axis=(1, 2))
        b = self._bin(params)
        self.err_map = np.full(self.bins * self.bins, np.inf)
        for k in range(self.bins * self.bins):
            if np.any(b == k):
                self.err_map[k] = err[b == k].max()
        return err

    def in_box(self, params):
        p = np.asarray(params)
        return np.all((p >= self.lo) & (p <= self.hi), axis=1)

    def screen(self, params, budget: float = 1e-3, precision: str = "mixed"):
        """Bloch trajectories for ``params``: surrogate where its calibrated
        error is within ``budget`` inside the training box, TEMPO elsewhere.
        Returns (trajectories, fallback mask, timings)."""
        p = np.asarray(params)
        t0 = time.perf_counter()
        out = self.predict(p).astype(np.float64)
        t_sur = time.perf_counter() - t0
        trusted = self.in_box(p) & (self.err_map[self._bin(p)] <= budget)
        fb = ~trusted
        t_fb = 0.0
        if fb.any():
            traj, t_fb = tempo_bloch(p[fb], self.nsteps, self.dt, self.dkmax, self.epsrel,
                                     precision, self.chi_cap)
            out[fb] = traj
        return out, fb, {"surrogate_s": t_sur, "fallback_s": t_fb,
                         "points_per_s": len(p) / (t_sur + t_fb)}
