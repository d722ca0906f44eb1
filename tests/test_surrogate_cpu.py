"""Host-side pieces of the surrogate: the closed-system baseline and the
density-matrix -> Bloch-vector map."""
import numpy as np
from scipy.linalg import expm

from oqupy_gb300 import surrogate as sg

SX = np.array([[0, 1], [1, 0]], dtype=complex)
SY = np.array([[0, -1j], [1j, 0]])
SZ = np.diag([1.0, -1.0]).astype(complex)


def test_free_bloch_matches_unitary_evolution():
    P = sg.sample_params(4, 7)
    nsteps, dt = 30, 0.05
    fb = sg.free_bloch(P, nsteps, dt)
    for i, p in enumerate(P):
        U = expm(-1j * (0.5 * p[3] * SX + 0.5 * p[4] * SZ) * dt)
        rho = np.diag([1.0, 0.0]).astype(complex)
        for k in range(nsteps):
            rho = U @ rho @ U.conj().T
            b = [np.trace(rho @ s).real for s in (SX, SY, SZ)]
            np.testing.assert_allclose(fb[i, :, k], b, atol=1e-12)


def test_bloch_of_vectorised_states():
    rng = np.random.default_rng(2)
    for _ in range(5):
        a = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
        rho = a @ a.conj().T
        rho /= np.trace(rho)
        b = sg.bloch(rho.reshape(1, 4))[0]
        np.testing.assert_allclose(b, [np.trace(rho @ s).real for s in (SX, SY, SZ)], atol=1e-14)


def test_sampled_parameters_lie_in_the_box():
    P = sg.sample_params(1000, 3)
    lo = np.array([sg.BOX[k][0] for k in sg.KEYS])
    hi = np.array([sg.BOX[k][1] for k in sg.KEYS])
    assert np.all(P >= lo) and np.all(P <= hi)
