"""Import the unmodified OQuPy reference for integration tests, when it is
available; tests skip otherwise.

Looked up, in order: an importable ``oqupy``; the copy installed under
``baseline/_ref`` (``pip install --target baseline/_ref <reference>``); the
source tree named by the ``OQUPY_REFERENCE_SRC`` environment variable.  The
third-party ``tensornetwork`` package it imports is provided by the
from-scratch stand-in in ``oracle/tnshim``."""

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CANDIDATES = [os.path.join(ROOT, "baseline", "_ref"), os.environ.get("OQUPY_REFERENCE_SRC", "")]


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
            # appended, so that this repository's own packages (tests, oracle)
            # keep precedence over same-named directories of the install
            for p in (shim, c):
                if p not in sys.path:
                    sys.path.append(p)
            import warnings
            warnings.simplefilter("ignore", DeprecationWarning)
            import oqupy
            oqupy.config.PROGRESS_TYPE = "silent"
            return oqupy
    pytest.skip("OQuPy reference sources not available")
