"""Import surface of ``tensornetwork.backends`` (test infrastructure only)."""
from . import base_backend  # noqa: F401
