"""Run the unmodified OQuPy reference under numpy 2.5.

The reference checks time-dependent (and field-dependent) Hamiltonians and
time-dependent Lindblad operators by wrapping them in ``np.vectorize``
(oqupy/system.py:983-1005, 1045-1074) and keeps the wrappers; numpy 2.5 no
longer converts the matrix that such a wrapper returns for scalar
arguments, so the reference cannot build ``TimeDependentSystem`` or
``TimeDependentSystemWithField`` here.  ``patch_vectorize_checks`` replaces
the matrix-valued wrappers by the callables themselves, with the same
checks; a scalar call returns the same matrix either way, so no number the
reference computes changes.  (Idempotent.)
"""

import numpy as np


def patch_vectorize_checks(oqupy):
    sysm = oqupy.system
    if getattr(sysm, "_vectorize_patched", False):
        return

    def square(h, what):
        h = np.asarray(h)
        if h.ndim != 2 or h.shape[0] != h.shape[1]:
            raise AssertionError(f"{what} must return a square matrix.")

    def check_t(hamiltonian):
        square(hamiltonian(1.0), "Time dependent Hamiltonian")
        return hamiltonian

    def check_tf(hamiltonian):
        square(hamiltonian(1.0, 1.0 + 1.0j), "Time and field dependent Hamiltonian")
        return hamiltonian

    ref_lists = sysm._check_dissipator_lists

    def check_gl(gammas, lindblad_operators):
        gammas, lindblad_operators = ref_lists(gammas, lindblad_operators)
        for g in gammas:
            float(g(1.0))
        for op in lindblad_operators:
            np.array(op(1.0))
        return [np.vectorize(g) for g in gammas], list(lindblad_operators)

    sysm._check_tdependent_hamiltonian = check_t
    sysm._check_tfielddependent_hamiltonian = check_tf
    sysm._check_tdependent_gammas_lindblad_operators = check_gl
    sysm._vectorize_patched = True
