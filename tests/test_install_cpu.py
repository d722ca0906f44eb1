"""The drop-in hook dispatches on backend_config without touching the GPU."""

import numpy as np
import pytest

from tests.reference_import import import_reference


def _tempo(oqupy, backend_config=None, unique=False):
    sys = oqupy.System(0.5 * oqupy.operators.sigma("x"))
    corr = oqupy.PowerLawSD(alpha=0.1, zeta=1.0, cutoff=4.0,
                            cutoff_type="exponential", temperature=0.0)
    bath = oqupy.Bath(0.5 * oqupy.operators.sigma("z"), corr)
    params = oqupy.TempoParameters(dt=0.05, dkmax=5, epsrel=1e-6)
    return oqupy.Tempo(sys, bath, params, oqupy.operators.spin_dm("up"), 0.0,
                       unique=unique, backend_config=backend_config)


def test_install_routes_gb300_config_to_gpu_backend():
    oqupy = import_reference()
    import oqupy_gb300
    from oqupy_gb300 import GpuTempoBackend
    oqupy_gb300.install(oqupy)
    try:
        t = _tempo(oqupy, {"backend": "gb300", "precision": "mixed"})
        assert isinstance(t._backend_instance, GpuTempoBackend)
        t2 = _tempo(oqupy)
        assert not isinstance(t2._backend_instance, GpuTempoBackend)
        # unique=True needs degeneracy maps: routed to the reference backend
        t3 = _tempo(oqupy, {"backend": "gb300"}, unique=True)
        assert not isinstance(t3._backend_instance, GpuTempoBackend)
    finally:
        oqupy_gb300.uninstall(oqupy)
    t4 = _tempo(oqupy, {})
    assert not isinstance(t4._backend_instance, GpuTempoBackend)
