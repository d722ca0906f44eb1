"""Import stub for matplotlib.pyplot.  Any use raises."""


def __getattr__(name):
    raise ImportError("matplotlib is not available in this environment")
