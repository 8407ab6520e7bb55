"""Import shim that lets the reference package run in this container.

Test infrastructure only. The reference (horton-part) imports third-party
packages that are not installed here: qc-grid (``grid``), ``yaml``,
``importlib_resources``, ``cvxopt`` and ``qpsolvers``. The modules in this
folder are small stand-ins written for this project. They provide only the
names the reference imports at module level, plus the two behaviours the
partitioning path on the molecular grid needs:

* ``yaml.safe_load`` for the flow-style ``constants.yaml`` table, and
* ``importlib_resources.files`` (mapped onto ``importlib.resources.files``).

``qpsolvers.solve_qp`` is routed to this project's own active-set QP so that
the reference's GISA class can run end to end.

Use :func:`activate` with the reference source folder; it prepends this shim
and that folder to ``sys.path``. Nothing in the product imports this package.
"""

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def activate(reference_src):
    """Put the shim and the reference's ``src`` folder first on ``sys.path``.

    Returns ``True`` when the reference package could be imported.
    """
    os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
    sys.dont_write_bytecode = True
    for p in (reference_src, HERE):
        if p not in sys.path:
            sys.path.insert(0, p)
    try:
        import horton_part  # noqa: F401
    except Exception:  # pragma: no cover - only when the reference is absent
        return False
    return True
