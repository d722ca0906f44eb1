"""Import stub for numdifftools (absent here).  Any use raises."""


class Jacobian:
    def __init__(self, *args, **kwargs):
        raise ImportError("numdifftools is not available in this environment")
