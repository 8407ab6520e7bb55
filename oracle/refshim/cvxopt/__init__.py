"""Stand-in for ``cvxopt`` (test infrastructure only).

Only the import succeeds; any use raises, so the reference's cvxopt solvers are
reported as unavailable rather than silently replaced.
"""


def __getattr__(name):
    raise NotImplementedError("cvxopt is not installed; this is an import stand-in")
