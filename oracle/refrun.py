"""Run the unmodified reference (horton-part) on given arrays.

TEST INFRASTRUCTURE ONLY: used in this container to pin the oracle and to
write the golden fixtures under ``tests/golden``. It needs the reference
source tree (``REFERENCE_SRC``) and is never used on the GPU machine.

The reference runs on the molecular grid (``grid_type=3``) with a duck-typed
grid object (``points``, ``weights``, ``size``, ``integrate``), as its
molecular-grid code path requires (``core/base.py:416-499``).
"""

from __future__ import annotations

import logging
import os

import numpy as np

from oracle import refshim

REFERENCE_SRC = os.environ.get("HP_REFERENCE_SRC", "/root/reference/src")


class DuckGrid:
    def __init__(self, points, weights):
        self.points = points
        self.weights = weights
        self.size = weights.size
        self.atgrids = None
        self.indices = None

    def integrate(self, *arrays):
        prod = arrays[0]
        for a in arrays[1:]:
            prod = prod * a
        return float(np.dot(self.weights, prod))


def available():
    return os.path.isdir(os.path.join(REFERENCE_SRC, "horton_part")) and refshim.activate(
        REFERENCE_SRC)


def _quiet_logger():
    lg = logging.getLogger("hp-reference")
    lg.setLevel(logging.ERROR)
    if not lg.handlers:
        lg.addHandler(logging.NullHandler())
    lg.propagate = False
    return lg


def run(scheme, coordinates, numbers, pseudo_numbers, points, weights, rho, **kwargs):
    """Construct the reference class for ``scheme`` and run ``do_partitioning``.

    Returns the reference's ``cache`` items as a plain dict.
    """
    if not available():
        raise RuntimeError("reference source not found")
    from horton_part.utils import wpart_schemes

    cls = wpart_schemes(scheme)
    part = cls(np.asarray(coordinates, dtype=float), np.asarray(numbers, dtype=np.int64),
               np.asarray(pseudo_numbers, dtype=float), DuckGrid(points, weights), rho,
               logger=_quiet_logger(), grid_type=3, **kwargs)
    part.do_partitioning()
    out = {}
    for key in part.cache.iterkeys():
        k = key if isinstance(key, str) else "_".join(str(x) for x in key)
        out[k] = part.cache.load(key)
    out["_ranges"] = np.asarray(part._ranges)
    return out
