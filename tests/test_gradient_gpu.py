"""Gradients on the GPU: ``compute_gradient_and_dynamics``
(oqupy/gradient.py:169-437) with the process tensor built on the device from
the reference's influences (``PtBatch``) and the forward sweep, the adjoint
sweep and the per-step derivative cores on the device
(``otb_dyn_gradient``), against the unmodified reference's derivative
tensors and states in ``tests/golden/gradient.npz``, with and without
control operations: complex128 at 1e-10 (10x the reference's own spread
where that is larger), the mixed-precision build at 1e-6.  Where the
reference is importable, its ``compute_gradient_and_dynamics`` on a
``PtTempo(..., backend gb300)`` process tensor runs the same path end to
end."""

import numpy as np
import pytest

from tests import golden_cases as gc
from tests.test_gradient_cpu import CASES, check, controls, get, load, propagators

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["complex128", "mixed"])
@pytest.mark.parametrize("tag", ["plain", "control"])
@pytest.mark.parametrize("name", CASES)
def test_gpu_gradient_matches_reference(name, tag, precision):
    from oqupy_gb300 import correlations as corr
    from oqupy_gb300.pt import PtBatch
    g = load()
    d = int(g[f"{name}/d"])
    b = PtBatch([dict(hs_dim=d, num_steps=int(g[f"{name}/nsteps"]), dkmax=int(g[f"{name}/dkmax"]),
                      epsrel=float(g[f"{name}/epsrel"]), influences=g[f"{name}/influences"])],
                precision=precision, chi_cap=1152 // (d * d))
    b.build()

    class Pt:
        device = (b, 0)
        transform_in = get(g, name, "transform_in")
        transform_out = get(g, name, "transform_out")
    ctl = controls(g, name) if tag == "control" else None
    derivs, states = corr.device_gradient(Pt(), propagators(g, name), g[f"{name}/rho0"],
                                          g[f"{name}/target"], int(g[f"{name}/nsteps"]), ctl)
    b.close()
    tol = gc.PARITY_ABS if precision == "complex128" else gc.MIXED_ABS
    bad, ed, es = check(g, name, tag, derivs, states, tol)
    print(f"\n{name} {tag} {precision}: derivs {ed:.1e}, states {es:.1e}")
    assert not bad, bad


def test_gradient_end_to_end():
    from tests.reference_import import import_reference
    from tests.reference_compat import patch_vectorize_checks
    oqupy = import_reference()
    patch_vectorize_checks(oqupy)
    import oqupy.gradient  # noqa: F401
    import oqupy_gb300
    g = load()
    name = "grad_nondiag"
    sx, sz, sm = oqupy.operators.sigma("x"), oqupy.operators.sigma("z"), oqupy.operators.sigma("-")
    corr_sd = oqupy.PowerLawSD(alpha=0.15, zeta=1.0, cutoff=3.0, cutoff_type="exponential",
                               temperature=0.5)
    bath = oqupy.Bath(0.5 * sx, corr_sd)
    params_t = oqupy.TempoParameters(dt=0.1, dkmax=6, epsrel=1e-7)
    h = lambda hx, hz: hx * sx + hz * sz   # noqa: E731
    ps = oqupy.ParameterizedSystem(h, gammas=[lambda hx, hz: 0.1], lindblad_operators=[lambda hx, hz: sm])
    ps._hamiltonian = h
    n = int(g[f"{name}/nsteps"])
    params = np.random.default_rng(42).uniform(-1.0, 1.0, size=(2 * n, 2))
    oqupy_gb300.install(oqupy)
    try:
        ptt = oqupy.PtTempo(bath, 0.0, n * 0.1, params_t, backend_config={"backend": "gb300"})
        pt = ptt.get_process_tensor(progress_type="silent")
        derivs, dyn = oqupy.gradient.compute_gradient_and_dynamics(
            system=ps, initial_state=g[f"{name}/rho0"].reshape(2, 2),
            target_derivative=g[f"{name}/target"].reshape(2, 2), process_tensors=[pt],
            parameters=params, dt=0.1, num_steps=n, progress_type="silent")
    finally:
        oqupy_gb300.uninstall(oqupy)
    states = np.array(dyn.states).reshape(len(dyn.states), -1)
    bad, ed, es = check(g, name, "plain", np.array(derivs), states)
    print(f"\nend to end: derivs {ed:.1e}, states {es:.1e}")
    assert not bad, bad
