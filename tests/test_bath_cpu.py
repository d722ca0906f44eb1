"""Host influence generation of the product vs the restated reference quad."""

import numpy as np
import pytest

from oracle import bath_oracle as bo
from oqupy_gb300 import bath


@pytest.mark.parametrize("alpha,zeta,wc,ctype,T", [
    (0.08, 1.0, 4.0, "exponential", 0.0),
    (0.4, 1.0, 8.0, "exponential", 3.0),
    (0.3, 1.0, 1.0, "exponential", 5.0),
    (0.12, 3.0, 3.0, "exponential", 1.0),
    (0.2, 1.0, 4.0, "gaussian", 0.3),
])
def test_influences_match_reference_quadrature(alpha, zeta, wc, ctype, T):
    dt, dkmax = 0.05, 12
    op = 0.5 * np.diag([1.0, -1.0])
    got, _ = bath.influences(alpha, zeta, wc, ctype, T, dt, dkmax, op)
    ref_bath = bo.PowerLawBath(alpha, zeta, wc, ctype, T)
    comm, acomm, _ = bo.coupling_diagonals(op)
    for dk in range(dkmax + 1):
        ref = bo.influence_matrix(dk, dt, dkmax, ref_bath, comm, acomm,
                                  None, 1e-12)
        np.testing.assert_allclose(got[dk], ref, rtol=0, atol=2e-9)


def test_propagators_match_reference():
    h = np.array([[0.3, 0.5 - 0.1j], [0.5 + 0.1j, -0.2]])
    sm = np.array([[0, 0], [1.0, 0]])
    p, _ = bath.half_step_propagators(h, 0.05, [0.1], [sm])
    q, _ = bo.half_step_propagators(h, 0.05, [0.1], [sm])
    np.testing.assert_allclose(p, q, atol=1e-14)
