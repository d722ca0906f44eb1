"""Hook the GPU backends into an imported ``oqupy`` package.

``oqupy.Tempo`` builds its backend as ``TempoBackend(..., config=
backend_config)`` (oqupy/tempo.py:424-435) and ``oqupy.PtTempo`` builds
``PtTempoBackend(..., config=...)`` (oqupy/pt_tempo.py:218-228); both names
are module globals.  ``install()`` rebinds them to factories that return the
GPU backend when ``backend_config["backend"] == "gb300"`` and the reference
class otherwise, so existing code selects the GPU path through its existing
configuration.  The factory dispatches before the reference constructor runs,
so the reference never sees the unknown backend name.
"""

from typing import Any, Dict, Optional

BACKEND_NAME = "gb300"
_installed: Dict[str, Any] = {}


def _wants_gpu(config: Optional[dict]) -> bool:
    return isinstance(config, dict) and config.get("backend") == BACKEND_NAME


def install(oqupy_module: Any = None) -> None:
    """Rebind the backend constructors of ``oqupy`` (idempotent)."""
    if oqupy_module is None:
        import oqupy as oqupy_module  # noqa: F401
    import importlib
    tempo_mod = importlib.import_module(oqupy_module.__name__ + ".tempo")
    from .tempo import GpuTempoBackend

    if "TempoBackend" not in _installed:
        ref_cls = tempo_mod.TempoBackend
        _installed["TempoBackend"] = ref_cls

        def tempo_backend(*args, config=None, degeneracy_maps=None, **kwargs):
            if _wants_gpu(config) and degeneracy_maps is None:
                return GpuTempoBackend(*args, config=config, degeneracy_maps=None, **kwargs)
            if _wants_gpu(config):
                config = {k: v for k, v in config.items() if k != "backend"}
            return ref_cls(*args, config=config, degeneracy_maps=degeneracy_maps, **kwargs)

        tempo_backend.reference_class = ref_cls
        tempo_mod.TempoBackend = tempo_backend


def uninstall(oqupy_module: Any = None) -> None:
    if oqupy_module is None:
        import oqupy as oqupy_module  # noqa: F401
    import importlib
    tempo_mod = importlib.import_module(oqupy_module.__name__ + ".tempo")
    if "TempoBackend" in _installed:
        tempo_mod.TempoBackend = _installed.pop("TempoBackend")
