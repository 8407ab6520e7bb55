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
    "RadialGrid",
    "AtomGrid",
    "atom_grid_arrays",
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


class RadialGrid:
    """Radial nodes and weights (qc-grid ``OneDGrid`` surface used by the
    reference: ``points``, ``weights``, ``size``, ``integrate``)."""

    def __init__(self, points, weights):
        self.points = np.ascontiguousarray(points, dtype=np.float64)
        self.weights = np.ascontiguousarray(weights, dtype=np.float64)

    @property
    def size(self):
        return self.points.size

    def integrate(self, *value_arrays):
        prod = value_arrays[0]
        for arr in value_arrays[1:]:
            prod = prod * arr
        return float(np.dot(self.weights, prod))


# Lebedev rule size -> degree (the reference logs the degrees)
_LEBEDEV_DEGREE = {50: 11, 110: 17, 194: 23, 302: 29, 590: 41}


class AtomGrid:
    """One atom's radial x Lebedev grid (the parts of qc-grid's ``AtomGrid``
    that grid_type 1 uses: ``rgrid``, ``size``, ``degrees`` and
    ``spherical_average``). Its points are ordered shell by shell: shell i
    owns points ``shell_offsets[i]:shell_offsets[i+1]`` with angular weights
    ``sphere_weights`` (Lebedev weight / 4 pi, summing to 1 over a shell)."""

    def __init__(self, rpoints, rweights, nang):
        self.rgrid = RadialGrid(rpoints, rweights)
        ang, wang = lebedev(nang)
        self.shell_offsets = np.arange(self.rgrid.size + 1, dtype=np.int64) * nang
        self.sphere_weights = np.tile(wang / (4.0 * np.pi), self.rgrid.size)
        self.degrees = np.full(self.rgrid.size, _LEBEDEV_DEGREE.get(nang, 0))

    @property
    def size(self):
        return int(self.shell_offsets[-1])

    def spherical_average(self, values):
        """Cubic spline through the angular averages of ``values`` on the
        radial nodes (evaluated at the nodes it returns the averages)."""
        from scipy.interpolate import CubicSpline

        shell = np.repeat(np.arange(self.rgrid.size), np.diff(self.shell_offsets))
        avg = np.bincount(shell, weights=self.sphere_weights * values, minlength=self.rgrid.size)
        return CubicSpline(self.rgrid.points, avg)


def atom_grid_arrays(grid):
    """The grid_type 1 arrays of the C ABI from a molecular grid with atom
    grids (``grid.atgrids``, ``grid.indices``): radial offsets per atom,
    point offsets per radial shell, angular weight / 4 pi per point, radial
    nodes and weights. Accepts this package's :class:`AtomGrid` and qc-grid
    atom grids (whose ``indices`` delimit the shells and whose weights are
    w_r r^2 w_Lebedev)."""
    roff, spo, wsph, rr, rw = [0], [0], [], [], []
    base = 0
    for a, ag in enumerate(grid.atgrids):
        r = np.asarray(ag.rgrid.points, dtype=np.float64)
        w = np.asarray(ag.rgrid.weights, dtype=np.float64)
        if hasattr(ag, "shell_offsets"):
            offs = np.asarray(ag.shell_offsets, dtype=np.int64)
            ws = np.asarray(ag.sphere_weights, dtype=np.float64)
        else:
            offs = np.asarray(ag.indices, dtype=np.int64)
            shell = np.repeat(np.arange(r.size), np.diff(offs))
            ws = np.asarray(ag.weights, dtype=np.float64) / (4.0 * np.pi * r[shell] ** 2 * w[shell])
        if grid.indices is not None and int(grid.indices[a]) != base:
            raise ValueError("atom grids must follow each other in the molecular grid")
        spo.extend((base + offs[1:]).tolist())
        base += int(offs[-1])
        roff.append(roff[-1] + r.size)
        wsph.append(ws)
        rr.append(r)
        rw.append(w)
    return dict(radial_offsets=np.asarray(roff, dtype=np.int32),
                shell_point_offsets=np.asarray(spo, dtype=np.int64),
                point_sphere_weights=np.concatenate(wsph), radial_points=np.concatenate(rr),
                radial_weights=np.concatenate(rw))


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
    atgrids = [AtomGrid(r, wr, nang) for _ in range(natom)]
    return MolecularGrid(points, weights, indices=indices, atgrids=atgrids)
