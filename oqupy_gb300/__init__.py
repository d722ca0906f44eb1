"""GB300-native backend for OQuPy's TEMPO / PT-TEMPO / process-tensor path.

The compute path is ``liboqupy_gb300.so`` (hand-written sm_103a CUDA, C ABI in
``include/oqupy_gb300.h``).  This package is the host side: the batched API
(``TempoBatch``), the drop-in backends that ``oqupy.Tempo`` / ``oqupy.PtTempo``
/ ``oqupy.MeanFieldTempo`` select through ``backend_config={"backend": "gb300", ...}`` once
``install()`` has run, and a device process tensor for ``compute_dynamics``.
"""

from .tempo import TempoBatch, GpuTempoBackend, fold_propagators  # noqa: F401
from .pt import PtBatch, GpuPtTempoBackend, device_compute_dynamics  # noqa: F401
from .mean_field import GpuMeanFieldTempoBackend  # noqa: F401
from .install import install, uninstall  # noqa: F401

__all__ = ["TempoBatch", "GpuTempoBackend", "fold_propagators", "PtBatch",
           "GpuPtTempoBackend", "device_compute_dynamics", "GpuMeanFieldTempoBackend",
           "install", "uninstall"]
