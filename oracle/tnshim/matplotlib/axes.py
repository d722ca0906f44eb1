"""Import stub for matplotlib.axes."""


class Axes:
    pass
