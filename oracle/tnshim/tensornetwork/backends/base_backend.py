"""Import surface of ``tensornetwork.backends.base_backend``."""


class BaseBackend:
    """Placeholder type; the reference only uses it in type hints."""
