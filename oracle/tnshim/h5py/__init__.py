"""Import stub for h5py (absent here).  Any use raises.  Test infrastructure."""


def File(*args, **kwargs):
    raise ImportError("h5py is not available in this environment")


def vlen_dtype(*args, **kwargs):
    raise ImportError("h5py is not available in this environment")
