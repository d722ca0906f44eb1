"""Host-side influence inputs for the batched engine.

The reference integrates the bath correlation function with scipy ``quad``
(4 adaptive integrals per time difference, oqupy/bath_correlations.py:518-591)
for every instance.  Here:

* ohmic (zeta = 1) baths with exponential cutoff use the closed form
      eta(t) = a ln(1 + wc^2 t^2)
               + 4 a [ln G(1 + T/wc) - Re ln G(1 + T/wc + i T t)]
               - 2 i a (wc t - arctan(wc t))
  (Frullani integrals; the coth factor expanded as 1 + 2 sum_n e^{-n w/T}
  and the resulting product summed with the Gamma function);
* every other power-law bath uses a vectorised composite Gauss-Legendre
  quadrature of the same integrand the reference integrates.

``influence_matrix`` then follows oqupy/tempo.py:969-1020 (unique=False).
"""

from typing import Optional, Sequence

import numpy as np
from scipy.linalg import expm
from scipy.special import loggamma


def _eta_ohmic_exp(tau, alpha, wc, T):
    tau = np.asarray(tau, dtype=np.float64)
    re = alpha * np.log1p((wc * tau) ** 2)
    if T > 0.0:
        c = T / wc
        re = re + 4.0 * alpha * (loggamma(1.0 + c).real
                                 - loggamma(1.0 + c + 1j * T * tau).real)
    im = -2.0 * alpha * (wc * tau - np.arctan(wc * tau))
    return re + 1j * im


_GL_X, _GL_W = np.polynomial.legendre.leggauss(16)


def _eta_quadrature(tau, alpha, zeta, wc, cutoff_type, T):
    """eta(t) = -int_0^inf J(w)/w^2 [coth(w/2T)(cos wt - 1) + i(wt - sin wt)] dw
    (the integrand of bath_correlations.py:556-575 rewritten in real form)."""
    tau = np.atleast_1d(np.asarray(tau, dtype=np.float64))
    tmax = max(float(np.max(np.abs(tau))), 1e-12)
    if cutoff_type == "hard":
        wmax = wc
    elif cutoff_type == "gaussian":
        wmax = 8.0 * wc
    else:
        wmax = 60.0 * wc
    width = min(np.pi / (2.0 * tmax), wc / 8.0)
    npan = int(np.ceil(wmax / width))
    edges = np.linspace(0.0, wmax, npan + 1)
    a, b = edges[:-1, None], edges[1:, None]
    w = (0.5 * (b - a) * _GL_X[None, :] + 0.5 * (a + b)).ravel()
    wt = (0.5 * (b - a) * _GL_W[None, :]).ravel()
    if cutoff_type == "hard":
        X = np.ones_like(w)
    elif cutoff_type == "gaussian":
        X = np.exp(-(w / wc) ** 2)
    else:
        X = np.exp(-w / wc)
    J = 2.0 * alpha * w ** zeta * wc ** (1.0 - zeta) * X
    coth = 1.0 / np.tanh(w / (2.0 * T)) if T > 0.0 else np.ones_like(w)
    base = wt * J / w ** 2
    out = np.empty(tau.shape, dtype=np.complex128)
    for k0 in range(0, tau.size, 64):
        t = tau[k0:k0 + 64, None]
        wt_ = w[None, :] * t
        re = (base * coth * (np.cos(wt_) - 1.0)).sum(axis=1)
        im = (base * (wt_ - np.sin(wt_))).sum(axis=1)
        out[k0:k0 + 64] = -(re + 1j * im)
    return out


def eta(tau, alpha, zeta, cutoff, cutoff_type="exponential", temperature=0.0):
    """Bath correlation double integral eta(tau) of a PowerLawSD bath."""
    if zeta == 1.0 and cutoff_type == "exponential":
        return _eta_ohmic_exp(tau, alpha, cutoff, temperature)
    return _eta_quadrature(tau, alpha, zeta, cutoff, cutoff_type, temperature)


def coupling_diagonals(coupling_op):
    """bath.py:68-85: (comm diagonal, acomm diagonal, unitary)."""
    op = np.asarray(coupling_op, dtype=np.complex128)
    d = op.shape[0]
    if np.allclose(np.diag(op.diagonal()), op):
        diag, unitary = op, np.identity(d)
    else:
        w, v = np.linalg.eig(op)
        diag, unitary = np.diag(w), v
    eye = np.identity(d)
    comm = (np.kron(diag, eye) - np.kron(eye, diag.T)).diagonal()
    acomm = (np.kron(diag, eye) + np.kron(eye, diag.T)).diagonal()
    return comm, acomm, unitary


def influences(alpha, zeta, cutoff, cutoff_type, temperature, dt, dkmax,
               coupling_op) -> tuple:
    """Influence matrices dk = 0..dkmax (tempo.py:969-1020, square /
    upper-triangle shapes) and the coupling unitary."""
    comm, acomm, unitary = coupling_diagonals(coupling_op)
    taus = dt * np.arange(-1, dkmax + 2, dtype=np.float64)
    e = eta(np.abs(taus), alpha, zeta, cutoff, cutoff_type, temperature)
    e = np.where(taus < 0, np.conj(e), e)      # eta(-t) = conj(eta(t))
    e_at = dict(zip(range(-1, dkmax + 2), e))
    D = comm.size
    out = np.empty((dkmax + 1, D, D), dtype=np.complex128)
    for dk in range(dkmax + 1):
        if dk == 0:
            et = e_at[1] - e_at[0]
            out[0] = np.diag(np.exp(-comm * (et.real * comm + 1j * et.imag * acomm)))
        else:
            et = e_at[dk + 1] - 2.0 * e_at[dk] + e_at[dk - 1]
            out[dk] = np.exp(-np.outer(et.real * comm + 1j * et.imag * acomm, comm))
    return out, unitary


def half_step_propagators(h, dt, gammas: Sequence[float] = (),
                          lindblad_ops: Sequence = ()):
    """expm(L dt/2) for the Lindblad Liouvillian of system.py:1118-1126."""
    h = np.asarray(h, dtype=np.complex128)
    d = h.shape[0]
    eye = np.identity(d)
    L = -1j * (np.kron(h, eye) - np.kron(eye, h.T))
    for g, op in zip(gammas, lindblad_ops):
        op = np.asarray(op, dtype=np.complex128)
        opd = op.conjugate().T
        n = opd @ op
        L = L + g * (np.kron(op, opd.T) - 0.5 * (np.kron(n, eye) + np.kron(eye, n.T)))
    p = expm(L * dt / 2.0)
    return p, p.copy()
