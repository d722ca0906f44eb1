"""Import the unmodified OQuPy reference for integration tests, when its
sources are available (development container); tests skip otherwise."""

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CANDIDATES = [os.environ.get("OQUPY_REFERENCE_SRC", ""), "/root/reference"]


def import_reference():
    import pytest
    try:
        import oqupy  # installed copy
        return oqupy
    except ImportError:
        pass
    for c in CANDIDATES:
        if c and os.path.isdir(os.path.join(c, "oqupy")):
            shim = os.path.join(ROOT, "oracle", "tnshim")
            for p in (shim, c):
                if p not in sys.path:
                    sys.path.insert(0, p)
            import warnings
            warnings.simplefilter("ignore", DeprecationWarning)
            import oqupy
            oqupy.config.PROGRESS_TYPE = "silent"
            return oqupy
    pytest.skip("OQuPy reference sources not available")
