"""Stand-in for ``grid.becke`` (test infrastructure only)."""
from . import BeckeWeights  # noqa: F401
