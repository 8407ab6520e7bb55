"""Stand-in for ``grid.rtransform`` (test infrastructure only)."""
from . import BeckeRTransform, ExpRTransform, PowerRTransform  # noqa: F401
