"""n-time correlations and controlled / time-dependent process-tensor
dynamics on the GPU: the process tensor built on the device from the
reference's influences (``PtBatch``), every correlation run of the
reference's schedule as one slot of a single batched sweep and the control
operations folded into the sweep's propagator table
(``oqupy_gb300.correlations``, ``otb_dyn_run_steps``), against the
unmodified reference's outputs in ``tests/golden/correlations.npz``:
complex128 at 1e-10 (10x the reference's own spread where that is larger),
the mixed-precision build at 1e-6.  Where the reference is importable,
``oqupy.compute_correlations`` on a ``PtTempo(..., backend gb300)`` process
tensor runs the same path end to end."""

import numpy as np
import pytest

from tests import correlation_cases as cc
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


def gpu_pt(g, name, precision):
    from oqupy_gb300.pt import PtBatch
    d = int(g[f"{name}/d"])
    b = PtBatch([dict(hs_dim=d, num_steps=int(g[f"{name}/nsteps"]), dkmax=int(g[f"{name}/dkmax"]),
                      epsrel=float(g[f"{name}/epsrel"]), influences=g[f"{name}/influences"])],
                precision=precision, chi_cap=min(128, 1152 // (d * d)))
    b.build()

    class Pt:
        device = (b, 0)
        transform_in = cc.get(g, name, "transform_in")
        transform_out = cc.get(g, name, "transform_out")
    return b, Pt()


@pytest.mark.parametrize("precision", ["complex128", "mixed"])
@pytest.mark.parametrize("name", cc.CASES)
def test_gpu_correlations_match_reference(name, precision):
    from oqupy_gb300 import correlations as corr
    g = cc.load()
    batch, pt = gpu_pt(g, name, precision)

    def sweep(props, rho0, n, ctl):
        return corr.device_dynamics(pt, [props], [rho0], n, [ctl])[:, 0]

    def correl(props, rho0, ops, steps, order):
        return corr.device_correlations_nt(pt, props, rho0, ops, steps, order)
    out = cc.run(g, name, sweep, correl)
    batch.close()
    tol = gc.PARITY_ABS if precision == "complex128" else gc.MIXED_ABS
    bad, worst = cc.check(g, name, out, tol)
    print(f"\n{name} {precision}:", {k: f"{v:.1e}" for k, v in worst.items()})
    assert not bad, bad


def test_gpu_many_slot_sweep_matches_single_slots():
    """1100 slots (two launches of the 1024-slot sweep), each with its own
    control step, against the same slots run one at a time."""
    from oqupy_gb300 import correlations as corr
    g = cc.load()
    name = "corr_nondiag"
    batch, pt = gpu_pt(g, name, "complex128")
    p1, p2 = g[f"{name}/prop1"], g[f"{name}/prop2"]

    def props(step):
        return p1, p2
    n = int(g[f"{name}/nsteps"])
    op = np.kron(np.array([[0, 1], [1, 0]]), np.identity(2)).astype(complex)
    ctls = [{"pre": {1 + (h % (n - 1)): op}} for h in range(1100)]
    rho0 = g[f"{name}/rho0"]
    many = corr.device_dynamics(pt, [props] * 1100, [rho0] * 1100, n, ctls)
    for h in (0, 5, 1023, 1024, 1099):
        one = corr.device_dynamics(pt, [props], [rho0], n, [ctls[h]])[:, 0]
        np.testing.assert_allclose(many[:, h], one, rtol=0, atol=1e-14)
    batch.close()


def test_compute_correlations_end_to_end():
    from tests.reference_import import import_reference
    from tests.reference_compat import patch_vectorize_checks
    oqupy = import_reference()
    patch_vectorize_checks(oqupy)
    import oqupy_gb300
    g = cc.load()
    name = "corr_nondiag"
    sx, sz = oqupy.operators.sigma("x"), oqupy.operators.sigma("z")
    sm, sp = oqupy.operators.sigma("-"), oqupy.operators.sigma("+")
    corr_sd = oqupy.PowerLawSD(alpha=0.15, zeta=1.0, cutoff=3.0, cutoff_type="exponential",
                               temperature=0.5)
    bath = oqupy.Bath(0.5 * sx, corr_sd)
    params = oqupy.TempoParameters(dt=0.1, dkmax=6, epsrel=1e-7)
    oqupy_gb300.install(oqupy)
    try:
        ptt = oqupy.PtTempo(bath, 0.0, 1.8, params, backend_config={"backend": "gb300"})
        pt = ptt.get_process_tensor(progress_type="silent")
        system = oqupy.System(0.5 * sz + 0.3 * sx)
        t, c = oqupy.compute_correlations(system, pt, sm, sp, slice(0, 10, 3), slice(0, None),
                                          initial_state=g[f"{name}/rho0"].reshape(2, 2),
                                          progress_type="silent")
    finally:
        oqupy_gb300.uninstall(oqupy)
    ref = g[f"{name}/ordered"]
    assert np.array_equal(np.isnan(c), np.isnan(ref))
    err = np.abs(np.nan_to_num(c) - np.nan_to_num(ref)).max()
    print(f"\nend to end: max |error| {err:.1e}")
    assert err <= max(gc.PARITY_ABS, gc.ENVELOPE_FACTOR * g[f"{name}/ordered_envelope"].max())
