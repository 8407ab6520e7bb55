"""Stand-in for ``grid.onedgrid`` (test infrastructure only)."""
from . import GaussChebyshev, OneDGrid, UniformInteger  # noqa: F401
