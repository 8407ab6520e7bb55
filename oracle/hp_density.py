"""CPU oracle of the density generator: FP64 NumPy restatement of the
contracted-Gaussian density of horton-part's ``part-gen``
(``scripts/generate_density.py:119-204``: basis functions on the points,
then rho = einsum("ab,bp,ap->p", D, phi, phi) at :186-188).

TEST INFRASTRUCTURE ONLY: the checker of the GPU density kernel and the
timed CPU baseline of its bench section; the product never imports it.

The reference evaluates the basis with gbasis after iodata has read the
file; both are absent here, so the functions are restated in the
conventions of Gaussian's fchk files (the densities stored beside the
reference's test files pin them: ``tests/cached/*.fchk`` with the matching
``*.npz``, to 1e-14 relative for s, p and sp shells). The d and f forms
below (file-order Cartesian components; pure functions m = 0, +1, -1, ...)
are written from the textbook real solid harmonics; no reference fixture
has a d or f shell, so those conventions are unpinned.
"""

from __future__ import annotations

import math

import numpy as np

_R38 = math.sqrt(3.0 / 8.0)
_R58 = math.sqrt(5.0 / 8.0)
_R3 = math.sqrt(3.0)
_R15 = math.sqrt(15.0)


def _dfact(n):
    return 1 if n <= 0 else n * _dfact(n - 2)


def _angular(l, pure, x, y, z):
    """Angular factors of the shell's functions (file order), in units where
    x^l is the normalised component."""
    if l == 0:
        return [np.ones_like(x)]
    if l == 1:
        return [x, y, z]
    if l == 2:
        if not pure:
            return [x * x, y * y, z * z, x * y, x * z, y * z]
        return [(2 * z * z - x * x - y * y) / 2, _R3 * x * z, _R3 * y * z,
                _R3 / 2 * (x * x - y * y), _R3 * x * y]
    if l == 3:
        if not pure:
            return [x ** 3, y ** 3, z ** 3, x * y * y, x * x * y, x * x * z, x * z * z, y * z * z,
                    y * y * z, x * y * z]
        return [z * (2 * z * z - 3 * x * x - 3 * y * y) / 2, _R38 * x * (4 * z * z - x * x - y * y),
                _R38 * y * (4 * z * z - x * x - y * y), _R15 / 2 * z * (x * x - y * y),
                _R15 * x * y * z, _R58 * x * (x * x - 3 * y * y), _R58 * y * (3 * x * x - y * y)]
    raise NotImplementedError(f"angular momentum {l}")


def basis_values(shells, points):
    """(nbasis, N) values of the contracted functions at the points. A
    primitive is N(a, l) x^i y^j z^k exp(-a r^2), N(a, l) = (2a/pi)^(3/4)
    (4a)^(l/2) / sqrt((2l-1)!!); contractions are not renormalised."""
    points = np.asarray(points, dtype=np.float64)
    out = []
    for s in shells:
        d = points - s.center
        r2 = np.einsum("pi,pi->p", d, d)
        a = np.asarray(s.exponents, dtype=np.float64)
        norm = (2 * a / math.pi) ** 0.75 * (4 * a) ** (s.l / 2) / math.sqrt(_dfact(2 * s.l - 1))
        radial = np.exp(-np.outer(r2, a)) @ (np.asarray(s.coeffs) * norm)
        out.extend(f * radial for f in _angular(s.l, s.pure, d[:, 0], d[:, 1], d[:, 2]))
    return np.array(out)


def density(one_rdm, shells, points, chunk=20000):
    """rho(p) = sum_ab D_ab phi_a(p) phi_b(p) in chunks of points."""
    points = np.asarray(points, dtype=np.float64)
    out = np.empty(len(points))
    for s in range(0, len(points), chunk):
        phi = basis_values(shells, points[s:s + chunk])
        out[s:s + chunk] = np.einsum("ab,bp,ap->p", one_rdm, phi, phi, optimize=True)
    return out
