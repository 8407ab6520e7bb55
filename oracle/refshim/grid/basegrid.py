"""Stand-in for ``grid.basegrid`` (test infrastructure only)."""
from . import OneDGrid  # noqa: F401
