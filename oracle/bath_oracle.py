"""Bath correlation integrals and influence matrices, restated (scipy quad).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates, with the same quadrature calls and tolerances:

* ``oqupy/bath_correlations.py:303-307``   cutoff functions
* ``oqupy/bath_correlations.py:518-591``   ``CustomSD.eta_function``
* ``oqupy/bath_correlations.py:593-664``   ``correlation_2d_integral``
* ``oqupy/bath_correlations.py:743-744``   ``PowerLawSD`` spectral density
* ``oqupy/tempo.py:969-1020``              ``influence_matrix`` (unique=False)
* ``oqupy/operators.py:127-137``           commutator / anticommutator
* ``oqupy/system.py:121-129, 1118-1126``   Lindblad Liouvillian, propagators
"""

from functools import lru_cache

import numpy as np
from scipy import integrate
from scipy.linalg import expm

INTEGRATE_EPSREL = 2 ** (-26)     # oqupy/config.py:25
SUBDIV_LIMIT = 256                # oqupy/config.py:28

_CUTOFFS = {
    "hard": lambda w, wc: np.heaviside(wc - w, 0),
    "exponential": lambda w, wc: np.exp(-w / wc),
    "gaussian": lambda w, wc: np.exp(-(w / wc) ** 2),
}


class PowerLawBath:
    """J(w) = 2 alpha w^zeta wc^(1-zeta) X(w, wc) at temperature T."""

    def __init__(self, alpha, zeta, cutoff, cutoff_type="exponential",
                 temperature=0.0):
        self.alpha = float(alpha)
        self.zeta = float(zeta)
        self.cutoff = float(cutoff)
        self.cutoff_type = cutoff_type
        self.temperature = float(temperature)
        self._x = _CUTOFFS[cutoff_type]

    def spectral_density(self, w):
        return (2.0 * self.alpha * w ** self.zeta
                * self.cutoff ** (1 - self.zeta) * self._x(w, self.cutoff))

    @staticmethod
    def _complex_integral(f, a, b, epsrel):
        re = integrate.quad(lambda x: np.real(f(x)), a=a, b=b,
                            epsrel=epsrel, limit=SUBDIV_LIMIT)[0]
        im = integrate.quad(lambda x: np.imag(f(x)), a=a, b=b,
                            epsrel=epsrel, limit=SUBDIV_LIMIT)[0]
        return re + 1j * im

    @lru_cache(maxsize=2 ** 12)
    def eta(self, tau: float, epsrel: float = INTEGRATE_EPSREL) -> complex:
        """bath_correlations.py:518-591 (matsubara=False).  ``influence_matrix``
        passes the TEMPO ``epsrel`` as the quadrature tolerance
        (tempo.py:996-1001)."""
        J = self.spectral_density
        T = self.temperature
        if T == 0.0:
            def f(w):
                return J(w) / w ** 2 * ((np.exp(-1j * w * tau) - 1)
                                        + 1j * w * tau)
        else:
            def f(w):
                if np.exp(-w / T) > np.finfo(float).eps:
                    return J(w) / w ** 2 * (
                        ((np.exp(-1j * tau * w)
                          + np.exp(-(w / T - 1j * tau * w)))
                         - np.exp(-w / T) - 1)
                        / (1 - np.exp(-w / T)) + 1j * tau * w)
                return J(w) / w ** 2 * (np.exp(-1j * w * tau) - 1
                                        + 1j * w * tau)
        val = self._complex_integral(f, 0.0, self.cutoff, epsrel)
        if self.cutoff_type != "hard":
            val += self._complex_integral(f, self.cutoff, np.inf, epsrel)
        return -val

    def correlation_2d_integral(self, delta, time_1, time_2=None,
                                shape="square", epsrel=INTEGRATE_EPSREL):
        """bath_correlations.py:593-664."""
        def e(tau):
            return self.eta(tau, epsrel)
        if shape == "upper-triangle":
            return e(time_1 + delta) - e(time_1)
        if shape == "square":
            return e(time_1 + delta) - 2.0 * e(time_1) + e(time_1 - delta)
        if shape == "rectangle":
            return (e(time_2) - e(time_1) - e(time_2 - delta)
                    + e(time_1 - delta))
        raise NotImplementedError(shape)


def commutator(op):
    d = op.shape[0]
    return np.kron(op, np.identity(d)) - np.kron(np.identity(d), op.T)


def acommutator(op):
    d = op.shape[0]
    return np.kron(op, np.identity(d)) + np.kron(np.identity(d), op.T)


def coupling_diagonals(coupling_op):
    """bath.py:68-85: diagonalise, return (comm_diag, acomm_diag, unitary)."""
    op = np.asarray(coupling_op, dtype=np.complex128)
    d = op.shape[0]
    if np.allclose(np.diag(op.diagonal()), op):
        diag_op, unitary = op, np.identity(d)
    else:
        w, v = np.linalg.eig(op)
        diag_op, unitary = np.diag(w), v
    return (commutator(diag_op).diagonal(), acommutator(diag_op).diagonal(),
            unitary)


def influence_matrix(dk, dt, dkmax, bath: PowerLawBath, comm, acomm,
                     add_correlation_time=None, epsrel=INTEGRATE_EPSREL):
    """tempo.py:969-1020 with ``deg_positions=None``."""
    if dk == 0:
        t1, t2, shape = 0.0, None, "upper-triangle"
    elif dk < 0:
        t1 = float(dkmax) * dt
        if add_correlation_time is None:
            return None
        t2 = float(dkmax) * dt + np.min([float(-dk) * dt,
                                         1.0 * dt + add_correlation_time])
        shape = "rectangle"
    else:
        t1, t2, shape = float(dk) * dt, None, "square"
    eta_dk = bath.correlation_2d_integral(dt, t1, t2, shape, epsrel)
    op_p, op_m = acomm, comm
    if dk == 0:
        return np.diag(np.exp(-op_m * (eta_dk.real * op_m
                                       + 1j * eta_dk.imag * op_p)))
    return np.exp(-np.outer(eta_dk.real * op_m + 1j * eta_dk.imag * op_p,
                            op_m))


def liouvillian(h, gammas=(), lindblad_ops=()):
    """system.py:1118-1126."""
    h = np.asarray(h, dtype=np.complex128)
    L = -1j * commutator(h)
    for g, op in zip(gammas, lindblad_ops):
        op = np.asarray(op, dtype=np.complex128)
        opd = op.conjugate().T
        L = L + g * (np.kron(op, opd.T) - 0.5 * acommutator(opd @ op))
    return L


def half_step_propagators(h, dt, gammas=(), lindblad_ops=()):
    """system.py:121-129: both halves are expm(L dt / 2)."""
    p = expm(liouvillian(h, gammas, lindblad_ops) * dt / 2.0)
    return p, p.copy()
