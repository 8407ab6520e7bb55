"""Becke-partitioned molecular integration grids.

The reference takes a qc-grid ``MolGrid`` and uses only a small part of it on
the molecular-grid path: ``points`` (N, 3), ``weights`` (N,), ``size`` and
``integrate(*arrays)`` (``core/base.py:139``, ``core/stockholder.py:150``,
``core/iterstock.py:41``). qc-grid is not a dependency of this package, so
:class:`MolecularGrid` provides exactly that surface, plus ``indices`` (the
first point of each atom's block, as qc-grid's ``MolGrid.indices``).

:func:`becke_molecular_grid` builds such a grid from atom-centred radial x
Lebedev product grids and Becke's (1988) fuzzy-cell partition with k = 3
smoothing steps and no atomic-size adjustment. The grid is an *input* of the
partitioning loop: the GPU path and the CPU oracle receive the same arrays.
"""

from __future__ import annotations

import os

import numpy as np

__all__ = [
    "MolecularGrid",
    "lebedev",
    "radial_becke_gauss_chebyshev",
    "becke_molecular_grid",
    "becke_partition_weights",
]

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
_LEBEDEV_CACHE = {}


class MolecularGrid:
    """Molecular integration grid: points, weights and ``integrate``.

    Parameters
    ----------
    points : (N, 3) float64 array
    weights : (N,) float64 array, including the Becke partition factor.
    indices : optional (natom + 1,) int array; atom ``a`` owns points
        ``indices[a]:indices[a+1]``.
    atgrids : optional per-atom grids (only needed by ``grid_type=1/2``).
    """

    def __init__(self, points, weights, indices=None, atgrids=None):
        points = np.ascontiguousarray(points, dtype=np.float64)
        weights = np.ascontiguousarray(weights, dtype=np.float64)
        if points.ndim != 2 or points.shape[1] != 3:
            raise ValueError("points must have shape (N, 3)")
        if weights.shape != (points.shape[0],):
            raise ValueError("weights must have shape (N,)")
        self._points = points
        self._weights = weights
        self._indices = None if indices is None else np.asarray(indices, dtype=np.int64)
        self.atgrids = atgrids

    @property
    def points(self):
        return self._points

    @property
    def weights(self):
        return self._weights

    @property
    def size(self):
        return self._weights.size

    @property
    def indices(self):
        return self._indices

    def integrate(self, *value_arrays):
        """Return sum_p w_p * prod_i f_i(p), as qc-grid's ``Grid.integrate``."""
        if len(value_arrays) == 0:
            raise ValueError("integrate needs at least one array")
        prod = value_arrays[0]
        for arr in value_arrays[1:]:
            prod = prod * arr
        return float(np.dot(self._weights, prod))


def lebedev(npoint):
    """Lebedev rule with ``npoint`` points: (points (n,3) on the unit sphere,
    weights (n,) summing to 4*pi). Tabulated for 50, 110, 194, 302 and 590
    points (generated once with ``scipy.integrate.lebedev_rule``)."""
    if npoint not in _LEBEDEV_CACHE:
        with np.load(os.path.join(_DATA, "lebedev.npz")) as f:
            key = f"points_{npoint}"
            if key not in f.files:
                raise ValueError(f"no Lebedev rule with {npoint} points is tabulated")
            _LEBEDEV_CACHE[npoint] = (f[key].copy(), f[f"weights_{npoint}"].copy())
    pts, wts = _LEBEDEV_CACHE[npoint]
    return pts.copy(), wts.copy()


def radial_becke_gauss_chebyshev(nrad, rmin=1e-4, radius=1.5):
    """Radial grid: Gauss-Chebyshev (first kind) nodes on (-1, 1) mapped by
    Becke's transform r = rmin + R (1 + x) / (1 - x).

    Returns (r, w) with sum_i w_i f(r_i) ~ int_0^inf f(r) dr; the 3-D radial
    weight is ``w * r**2``.
    """
    i = np.arange(1, nrad + 1, dtype=np.float64)
    x = np.cos((2.0 * i - 1.0) * np.pi / (2.0 * nrad))
    # Gauss-Chebyshev of the first kind written as a rule for int_{-1}^{1} f(x) dx
    wx = np.pi / nrad * np.sqrt(1.0 - x * x)
    r = rmin + radius * (1.0 + x) / (1.0 - x)
    drdx = 2.0 * radius / (1.0 - x) ** 2
    order = np.argsort(r)
    return r[order], (wx * drdx)[order]


def _becke_step(mu, k=3):
    f = mu
    for _ in range(k):
        f = 1.5 * f - 0.5 * f * f * f
    return 0.5 * (1.0 - f)


def becke_partition_weights(points, coordinates, owner, chunk=16384):
    """Becke fuzzy-cell weight of each point for the atom that owns it.

    w_a(p) = P_a(p) / sum_b P_b(p), P_a = prod_{b != a} s(mu_ab),
    mu_ab = (|p - R_a| - |p - R_b|) / |R_a - R_b|.
    """
    coordinates = np.asarray(coordinates, dtype=np.float64)
    natom = coordinates.shape[0]
    out = np.empty(points.shape[0], dtype=np.float64)
    if natom == 1:
        out[:] = 1.0
        return out
    rab = np.linalg.norm(coordinates[:, None, :] - coordinates[None, :, :], axis=2)
    np.fill_diagonal(rab, 1.0)
    inv_rab = 1.0 / rab
    eye = np.eye(natom, dtype=bool)
    for s in range(0, points.shape[0], chunk):
        p = points[s : s + chunk]
        d = np.linalg.norm(p[:, None, :] - coordinates[None, :, :], axis=2)  # (n, A)
        mu = (d[:, :, None] - d[:, None, :]) * inv_rab[None]
        sv = _becke_step(mu)
        sv[:, eye] = 1.0
        cell = np.prod(sv, axis=2)  # (n, A)
        own = owner[s : s + chunk]
        out[s : s + chunk] = cell[np.arange(p.shape[0]), own] / cell.sum(axis=1)
    return out


def becke_molecular_grid(coordinates, nrad, nang, rmin=1e-4, radius=1.5):
    """Atom-centred radial x Lebedev grids joined with Becke weights.

    Points are ordered atom by atom, and within an atom radial shell by
    radial shell; ``indices`` marks each atom's block.
    """
    coordinates = np.asarray(coordinates, dtype=np.float64)
    natom = coordinates.shape[0]
    r, wr = radial_becke_gauss_chebyshev(nrad, rmin, radius)
    ang, wang = lebedev(nang)
    shell_pts = (r[:, None, None] * ang[None, :, :]).reshape(-1, 3)
    shell_w = ((wr * r * r)[:, None] * wang[None, :]).reshape(-1)
    npa = shell_pts.shape[0]
    points = np.empty((natom * npa, 3), dtype=np.float64)
    weights = np.empty(natom * npa, dtype=np.float64)
    owner = np.repeat(np.arange(natom), npa)
    for a in range(natom):
        points[a * npa : (a + 1) * npa] = shell_pts + coordinates[a]
        weights[a * npa : (a + 1) * npa] = shell_w
    weights *= becke_partition_weights(points, coordinates, owner)
    indices = np.arange(natom + 1, dtype=np.int64) * npa
    return MolecularGrid(points, weights, indices=indices)
