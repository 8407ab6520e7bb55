"""Run the unmodified reference (horton-part) on given arrays.

TEST INFRASTRUCTURE ONLY: used in this container to pin the oracle and to
write the golden fixtures under ``tests/golden``. It needs the reference
source tree (``REFERENCE_SRC``) and is never used on the GPU machine.

The reference runs on the molecular grid (``grid_type=3``) with a duck-typed
grid object (``points``, ``weights``, ``size``, ``integrate``), as its
molecular-grid code path requires (``core/base.py:416-499``), or on atom
grids (``grid_type=1``) with duck-typed atom grids (``rgrid``, ``degrees``,
``spherical_average``; ``mbis.py:174-187``, ``core/iterstock.py:43-44``).
"""

from __future__ import annotations

import logging
import os

import numpy as np

from oracle import refshim

# The reference source tree (its ``src`` directory); no default: the fixture
# scripts that import the reference name it explicitly.
REFERENCE_SRC = os.environ.get("HP_REFERENCE_SRC", "")


def _integrate(weights, arrays):
    prod = arrays[0]
    for a in arrays[1:]:
        prod = prod * a
    return float(np.dot(weights, prod))


class DuckGrid:
    def __init__(self, points, weights, atgrids=None, indices=None):
        self.points = points
        self.weights = weights
        self.size = weights.size
        self.atgrids = atgrids
        self.indices = indices

    def integrate(self, *arrays):
        return _integrate(self.weights, arrays)


class DuckRadialGrid:
    def __init__(self, points, weights):
        self.points = points
        self.weights = weights
        self.size = points.size

    def integrate(self, *arrays):
        return _integrate(self.weights, arrays)


# Lebedev rule size -> degree (the reference only logs the degrees)
_LEBEDEV_DEGREE = {50: 11, 110: 17, 194: 23, 302: 29, 590: 41}


class DuckAtomGrid:
    """One atom's grid for the reference's grid_type 1 path: radial nodes and
    weights, and per point its radial shell and angular weight / 4 pi.
    ``spherical_average`` returns a cubic spline through the shell averages
    (qc-grid's AtomGrid.spherical_average)."""

    def __init__(self, rpoints, rweights, shell, wsph, nang):
        self.rgrid = DuckRadialGrid(np.asarray(rpoints, dtype=float), np.asarray(rweights, dtype=float))
        self.shell = np.asarray(shell)
        self.wsph = np.asarray(wsph, dtype=float)
        self.size = self.shell.size
        self.degrees = np.full(self.rgrid.size, _LEBEDEV_DEGREE.get(nang, 0))

    def spherical_average(self, values):
        from scipy.interpolate import CubicSpline

        avg = np.bincount(self.shell, weights=self.wsph * values, minlength=self.rgrid.size)
        return CubicSpline(self.rgrid.points, avg)


def available():
    if not REFERENCE_SRC or not os.path.isdir(os.path.join(REFERENCE_SRC, "horton_part")):
        return False
    return refshim.activate(REFERENCE_SRC)


def _quiet_logger():
    lg = logging.getLogger("hp-reference")
    lg.setLevel(logging.ERROR)
    if not lg.handlers:
        lg.addHandler(logging.NullHandler())
    lg.propagate = False
    return lg


def run(scheme, coordinates, numbers, pseudo_numbers, points, weights, rho, local=None,
        **kwargs):
    """Construct the reference class for ``scheme`` and run ``do_partitioning``.

    ``local`` (the atom-grid description of ``hp_oracle.mbis``, plus ``nang``
    Lebedev points per shell) selects grid_type 1; else grid_type 3.
    Returns the reference's ``cache`` items as a plain dict.
    """
    if not available():
        raise RuntimeError("reference source not found")
    from horton_part.utils import wpart_schemes

    cls = wpart_schemes(scheme)
    if local is None:
        grid, grid_type = DuckGrid(points, weights), 3
    else:
        import grid as qc_grid_stub

        ind = np.asarray(local["indices"])
        atgrids = [DuckAtomGrid(local["rpoints"][a], local["rweights"][a],
                                local["shell"][ind[a]:ind[a + 1]], local["wsph"][ind[a]:ind[a + 1]],
                                local.get("nang", 0)) for a in range(len(numbers))]
        qc_grid_stub.LEBEDEV_DEGREES.update({d: n for n, d in _LEBEDEV_DEGREE.items()})
        grid, grid_type = DuckGrid(points, weights, atgrids, ind), 1
    part = cls(np.asarray(coordinates, dtype=float), np.asarray(numbers, dtype=np.int64),
               np.asarray(pseudo_numbers, dtype=float), grid, rho,
               logger=_quiet_logger(), grid_type=grid_type, **kwargs)
    part.do_partitioning()
    out = {}
    for key in part.cache.iterkeys():
        k = key if isinstance(key, str) else "_".join(str(x) for x in key)
        out[k] = part.cache.load(key)
    out["_ranges"] = np.asarray(part._ranges)
    return out
