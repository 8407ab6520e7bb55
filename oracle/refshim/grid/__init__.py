"""Stand-in for qc-grid's top-level names (test infrastructure only).

The reference's molecular-grid path never calls these objects; they exist so
that ``from grid import ...`` statements succeed. A duck-typed molecular grid
(points, weights, size, integrate) is passed to the reference instead.
"""


class _Unavailable:
    def __init__(self, *args, **kwargs):
        raise NotImplementedError("qc-grid is not installed; this is an import stand-in")


class AtomGrid(_Unavailable):
    pass


class OneDGrid(_Unavailable):
    pass


class BeckeRTransform(_Unavailable):
    pass


class GaussChebyshev(_Unavailable):
    pass


class UniformGrid(_Unavailable):
    pass


class UniformInteger(_Unavailable):
    pass


class ExpRTransform(_Unavailable):
    pass


class PowerRTransform(_Unavailable):
    pass


class MolGrid(_Unavailable):
    pass


class BeckeWeights(_Unavailable):
    pass


# Lebedev degree -> number of points table, used by the reference for logging.
LEBEDEV_DEGREES = {}
