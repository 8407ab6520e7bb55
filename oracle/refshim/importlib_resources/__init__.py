"""Stand-in for the ``importlib_resources`` backport (test infrastructure only)."""
from importlib.resources import files  # noqa: F401
