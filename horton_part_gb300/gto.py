"""Contracted Gaussian basis functions in the conventions of Gaussian's
formatted checkpoint files, as tables for the density kernel.

A primitive of angular momentum l is N(a, l) x^i y^j z^k exp(-a r^2) with
N(a, l) = (2a/pi)^(3/4) (4a)^(l/2) / sqrt((2l-1)!!), the normalisation of the
pure power x^l, shared by every Cartesian component of the shell (the mixed
components such as xy are not unit-normalised). Contraction coefficients
multiply these normalised primitives; the contracted function is not
renormalised (the density matrices of the files refer to these functions:
checked to 1e-14 against the densities horton-part's test data store beside
its fchk files).

Cartesian order (fchk): s; x, y, z; xx, yy, zz, xy, xz, yz; xxx, yyy, zzz,
xyy, xxy, xxz, xzz, yzz, yyz, xyz. Pure functions: real regular solid
harmonics in the order m = 0, +1, -1, +2, -2, ..., each a combination of the
shell's Cartesian components normalised to one (the coefficients of the
standard expansion of Helgaker, Jorgensen and Olsen, "Molecular
Electronic-Structure Theory", eq. 6.4.47, with the norm taken from the exact
Cartesian overlaps).
"""

from __future__ import annotations

import math
from functools import lru_cache

import numpy as np

__all__ = ["MAX_L", "cartesian_powers", "pure_matrix", "primitive_norm", "shell_tables"]

MAX_L = 3

_CART = {
    0: [(0, 0, 0)],
    1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
    2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)],
    3: [(3, 0, 0), (0, 3, 0), (0, 0, 3), (1, 2, 0), (2, 1, 0), (2, 0, 1), (1, 0, 2), (0, 1, 2),
        (0, 2, 1), (1, 1, 1)],
}


def cartesian_powers(l):
    """(i, j, k) of the shell's Cartesian components in file order."""
    if l not in _CART:
        raise NotImplementedError(f"angular momentum {l} (only up to {MAX_L})")
    return list(_CART[l])


def _dfact(n):
    return 1 if n <= 0 else n * _dfact(n - 2)


def primitive_norm(alpha, l):
    """N(a, l) for an array of exponents."""
    alpha = np.asarray(alpha, dtype=np.float64)
    return (2.0 * alpha / math.pi) ** 0.75 * (4.0 * alpha) ** (0.5 * l) / math.sqrt(_dfact(2 * l - 1))


def _cart_overlap(l):
    """Overlap of the shell's Cartesian components relative to that of x^l."""
    pw = cartesian_powers(l)
    n = len(pw)
    g = np.zeros((n, n))
    for a, p in enumerate(pw):
        for b, q in enumerate(pw):
            s = [p[k] + q[k] for k in range(3)]
            if all(v % 2 == 0 for v in s):
                g[a, b] = (_dfact(s[0] - 1) * _dfact(s[1] - 1) * _dfact(s[2] - 1)) / _dfact(2 * l - 1)
    return g


def _solid_harmonic(l, m):
    """Coefficients of the real regular solid harmonic (l, m) on the
    monomials x^i y^j z^k, up to a positive factor: a dict (i, j, k) -> c."""
    am = abs(m)
    odd = 0 if m >= 0 else 1  # 2 v_m: cosine-type terms have even, sine-type odd powers of y
    out = {}
    for t in range((l - am) // 2 + 1):
        for u in range(t + 1):
            for two_v in range(odd, am + 1, 2):
                sign = -1 if (t + (two_v - odd) // 2) % 2 else 1
                c = (sign * 0.25 ** t * math.comb(l, t) * math.comb(l - t, am + t) * math.comb(t, u)
                     * math.comb(am, two_v))
                key = (2 * t + am - 2 * u - two_v, 2 * u + two_v, l - 2 * t - am)
                out[key] = out.get(key, 0.0) + c
    return {k: c for k, c in out.items() if c != 0.0}


@lru_cache(maxsize=None)
def pure_matrix(l):
    """(2l+1, ncart) matrix T with pure_m = sum_c T[m, c] cart_c, rows in the
    order m = 0, +1, -1, ..., each pure function normalised to one."""
    pw = cartesian_powers(l)
    index = {p: i for i, p in enumerate(pw)}
    g = _cart_overlap(l)
    rows = []
    for m in [0] + [s * k for k in range(1, l + 1) for s in (1, -1)]:
        v = np.zeros(len(pw))
        for key, c in _solid_harmonic(l, m).items():
            v[index[key]] += c
        v /= math.sqrt(v @ g @ v)
        rows.append(v)
    return np.array(rows)


def shell_tables(shells):
    """Flat tables of a list of :class:`~horton_part_gb300.fchk.Shell` for the
    density kernel: per shell (centre x, y, z), (l, pure, nprim, first
    primitive, first basis function), per primitive (exponent, normalised
    coefficient)."""
    centers = np.array([s.center for s in shells], dtype=np.float64).reshape(-1, 3)
    info = np.zeros((len(shells), 5), dtype=np.int32)
    exps, coefs = [], []
    p0 = f0 = 0
    for i, s in enumerate(shells):
        if s.l > MAX_L:
            raise NotImplementedError(f"angular momentum {s.l} (only up to {MAX_L})")
        n = len(s.exponents)
        info[i] = (s.l, int(s.pure), n, p0, f0)
        exps.append(s.exponents)
        coefs.append(s.coeffs * primitive_norm(s.exponents, s.l))
        p0 += n
        f0 += s.nfunc
    return (centers, info, np.concatenate(exps) if exps else np.zeros(0),
            np.concatenate(coefs) if coefs else np.zeros(0), f0)
