"""Mean-field TEMPO cases shared by the fixture script and the tests.

Each case is a ``MeanFieldSystem`` of two-level systems coupled to a
coherent field, as in the reference's tests/physics/mean_field_tempo_test.py
(case G, the driven Dicke model) and mean_field_tempo_multi_test.py.  The
field-dependent half-step propagators are restated here without OQuPy:
``TimeDependentSystemWithField.get_propagators`` with ``subdiv_limit=None``
(oqupy/system.py:434-452) samples the Liouvillian at t + dt/4 and
t + 3 dt/4 with the field linearised from its value and derivative at the
step's start (system.py:349-368) and exponentiates it over dt/2; the
Liouvillian is ``-i [H, .] + sum_n g_n (A . A^+ - {A^+ A, .}/2)``
(system.py:1118-1126, superoperators of operators.py:127-153).  The field
is advanced by the second-order Runge-Kutta rule of
``MeanFieldTempo._compute_field`` (oqupy/tempo.py:867-891).
"""

import numpy as np
from scipy.linalg import expm

SX = np.array([[0, 1], [1, 0]], dtype=np.complex128)
SY = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
SZ = np.array([[1, 0], [0, -1]], dtype=np.complex128)
SP = np.array([[0, 1], [0, 0]], dtype=np.complex128)
SM = np.array([[0, 0], [1, 0]], dtype=np.complex128)


def _commutator(h):
    d = h.shape[0]
    return np.kron(h, np.identity(d)) - np.kron(np.identity(d), h.T)


def _acommutator(h):
    d = h.shape[0]
    return np.kron(h, np.identity(d)) + np.kron(np.identity(d), h.T)


def liouvillian(h, gammas=(), lops=()):
    out = -1j * _commutator(h)
    for g, a in zip(gammas, lops):
        ad = a.conjugate().T
        out = out + g * (np.kron(a, ad.T) - 0.5 * _acommutator(ad @ a))
    return out


# -- case definitions ------------------------------------------------------

def dicke_hamiltonian(t, field):
    """Case G of the reference's mean-field test."""
    return 0.5 * SZ + np.real(field) * SX


def dicke_field_eom(t, states, field):
    return -(1j + 1) * field - 0.5j * np.matmul(SX, states[0]).trace().real


def pair_hamiltonian(omega0, rabi):
    def h(t, field):
        return 0.5 * omega0 * SZ + 0.5 * rabi * (field * SP + np.conj(field) * SM)
    return h


PAIR_FRACTIONS = (0.6, 0.4)
PAIR_RABI = 2.0


def pair_field_eom(t, states, field):
    s = sum(f * np.matmul(SM, st).trace() for f, st in zip(PAIR_FRACTIONS, states))
    return -(1j * (-0.5) + 0.5) * field - 0.5j * PAIR_RABI * s


CASES = {
    # reference tests/physics/mean_field_tempo_test.py case G: ohmic gaussian
    # bath alpha 0.1, wc 5, T 0, coupling sz/2, dt 0.05, full memory,
    # epsrel 1e-7, 20 steps
    "dicke_G": dict(
        systems=[dict(h=dicke_hamiltonian, gammas=[], lops=[],
                      coupling=0.5 * SZ, alpha=0.1, zeta=1.0, wc=5.0,
                      cutoff_type="gaussian", T=0.0,
                      rho0=np.array([[0.5, 0.5], [0.5, 0.5]], dtype=np.complex128))],
        field_eom=dicke_field_eom, field0=1.0 + 0j, dt=0.05, tcut=None,
        epsrel=1e-7, nsteps=20),
    # two different systems on one field: one with a diagonal coupling and
    # a decay channel, one coupled through sigma_x (a non-identity coupling
    # eigenbasis); finite memory (dkmax 6), 40 steps
    "pair_finite_memory": dict(
        systems=[dict(h=pair_hamiltonian(0.3, PAIR_RABI), gammas=[0.2], lops=[SM],
                      coupling=0.5 * SZ, alpha=0.2, zeta=1.0, wc=4.0,
                      cutoff_type="exponential", T=0.5,
                      rho0=np.array([[0, 0], [0, 1]], dtype=np.complex128)),
                 dict(h=pair_hamiltonian(-0.2, PAIR_RABI), gammas=[], lops=[],
                      coupling=0.5 * SX, alpha=0.15, zeta=1.0, wc=3.0,
                      cutoff_type="exponential", T=0.2,
                      rho0=np.array([[0.3, 0.1 - 0.2j], [0.1 + 0.2j, 0.7]], dtype=np.complex128))],
        field_eom=pair_field_eom, field0=0.3 + 0.1j, dt=0.05, tcut=0.3,
        epsrel=1e-7, nsteps=40),
}


def propagators(system, dt, start_time=0.0):
    """``get_propagators(dt, start_time, None, .)`` of a
    ``TimeDependentSystemWithField`` (system.py:434-452)."""
    h, gammas, lops = system["h"], system["gammas"], system["lops"]

    def props(step, field, deriv):
        t = start_time + step * dt

        def liou(tau):
            return liouvillian(h(tau, field + deriv * (tau - t)), gammas, lops)
        return expm(liou(t + dt / 4.0) * dt / 2.0), expm(liou(t + 3.0 * dt / 4.0) * dt / 2.0)
    return props


def field_functions(case, start_time=0.0):
    """``(compute_field, compute_field_derivative)`` of oqupy/tempo.py:867-891."""
    eom, dt = case["field_eom"], case["dt"]
    dims = [int(round(np.sqrt(np.asarray(s["rho0"]).size))) for s in case["systems"]]

    def mats(states):
        return [np.asarray(s).reshape(d, d) for s, d in zip(states, dims)]

    def compute_field(step, states, field, next_states):
        t = start_time + step * dt
        rk1 = eom(t, mats(states), field)
        rk2 = eom(t + dt, mats(next_states), field + rk1 * dt)
        return field + dt * (rk1 + rk2) / 2

    def compute_field_derivative(step, states, field):
        return eom(start_time + step * dt, mats(states), field)

    return compute_field, compute_field_derivative


def backend_args(name, fixture):
    """Positional arguments of ``MeanFieldTempoBackend`` (and of the oracle /
    the GPU backend) for a case, with the influence matrices and coupling
    eigenbases the reference computed (stored in the fixture)."""
    case = CASES[name]
    n = len(case["systems"])
    infl = [fixture[f"{name}/influences{i}"] for i in range(n)]

    def make_influence(arr):
        def influence(dk):
            return None if dk < 0 else arr[dk]
        return influence

    cf, cfd = field_functions(case)
    dkmax = int(fixture[f"{name}/dkmax"])
    return dict(
        initial_state_list=[np.asarray(s["rho0"]).reshape(-1) for s in case["systems"]],
        initial_field=case["field0"],
        influence_list=[make_influence(a) for a in infl],
        unitary_transform_list=[fixture[f"{name}/unitary{i}"] for i in range(n)],
        propagators_list=[propagators(s, case["dt"]) for s in case["systems"]],
        compute_field=cf, compute_field_derivative=cfd,
        dkmax=None if dkmax < 0 else dkmax, epsrel=case["epsrel"])



def patch_field_hamiltonian_check(oqupy):
    """See ``tests/reference_compat.py``."""
    from tests.reference_compat import patch_vectorize_checks
    patch_vectorize_checks(oqupy)
