"""Radial basis functions of the GISA / LISA pro-atoms.

A shell is ``g(r) = N(alpha, n) exp(-alpha r**n)`` with the normalisation
``N(alpha, n) = n alpha**(3/n) / (4 pi Gamma(3/n))`` so that its integral over
space is one (Slater, n = 1: alpha**3 / (8 pi); Gaussian, n = 2:
(alpha/pi)**1.5). This mirrors ``evaluate_function`` and
``ExpBasisFuncHelper`` in the reference (``core/basis.py:85-186``,
``core/basis.py:241-327``): the same parameter tables, the same names and the
same error behaviour. The GPU kernels evaluate the shells themselves; the
helpers here supply per-atom (order, exponent, initial) tables and the
host-side prefactors.

The default tables (``gauss`` and ``slater``) hold the same published
exponents and initial populations as the reference's data files
(``data/gauss.json``, ``data/slater.json``); partitioning results depend on
them, so they have to be identical.
"""

from __future__ import annotations

import json
import math

import numpy as np

__all__ = [
    "evaluate_function",
    "shell_prefactor",
    "BasisFuncHelper",
    "AnalyticBasisFuncHelper",
    "ExpBasisFuncHelper",
    "load_params",
]

# (orders, exponents, initials) per atomic number.
_GAUSS = {
    1: ([2.0] * 4, [5.672, 1.505, 0.5308, 0.2204], [0.0429, 0.2639, 0.479, 0.2127]),
    3: ([2.0] * 6, [25.5115, 7.3253, 2.6324, 0.9655, 0.0965, 0.0311],
        [0.1993, 0.7643, 0.8928, 0.0898, 1.0111, 0.025]),
    5: ([2.0] * 6, [98.2299, 27.7169, 9.7959, 0.5004, 0.1942, 0.0618],
        [0.1356, 0.6428, 1.0597, 1.9693, 1.1509, 0.0412]),
    6: ([2.0] * 6, [148.3, 42.19, 15.33, 6.146, 0.7846, 0.2511],
        [0.133, 0.5955, 1.0749, 0.0202, 2.7117, 1.4779]),
    7: ([2.0] * 6, [178.0, 52.42, 19.87, 1.276, 0.6291, 0.2857],
        [0.1627, 0.6567, 0.9993, 2.3257, 1.8949, 0.9479]),
    8: ([2.0] * 6, [220.1, 65.66, 25.98, 1.685, 0.686, 0.2311],
        [0.1869, 0.6576, 0.9751, 3.0657, 2.5622, 0.5528]),
    9: ([2.0] * 6, [232.2846, 73.1726, 30.0344, 2.4199, 1.0096, 0.3263],
        [0.2326, 0.7623, 0.8161, 2.9602, 3.3411, 0.8988]),
    14: ([2.0] * 9, [366.5112, 104.3665, 15.5123, 9.5104, 7.8724, 5.3849, 3.702, 0.3241, 0.1076],
         [0.5063, 1.1758, 0.0, 1.7484, 0.4014, 2.5315, 3.0395, 3.5767, 1.0358]),
    16: ([2.0] * 9, [528.7272, 147.5558, 17.6378, 17.5077, 15.1251, 7.1494, 0.5499, 0.2713, 0.1013],
         [0.4472, 1.1959, 0.0, 0.0, 1.471, 6.043, 4.2959, 2.289, 0.2565]),
    17: ([2.0] * 9, [622.3137, 180.7931, 98.9482, 69.1275, 20.2219, 8.9831, 0.6418, 0.3052, 0.137],
         [0.4127, 1.1066, 0.121, 0.0, 0.9133, 6.5025, 5.5666, 2.0125, 0.3716]),
    35: ([2.0] * 12, [1027.3862, 84.3671, 67.8966, 64.9399, 30.7992, 6.4459, 5.3029, 4.495, 2.6361,
                      0.7183, 0.3682, 0.139],
         [1.4011, 0.0, 0.0, 6.6184, 0.0, 0.0, 16.7407, 0.0, 1.0632, 3.3418, 5.0013, 0.7444]),
}

_SLATER_EXPONENTS = {
    1: [6.6, 4.62, 3.23, 2.26, 1.58, 1.1, 0.77, 1.0],
    6: [22.8, 17.35, 13.2, 8.79, 10.83, 7.91, 5.78, 4.22, 4.51, 3.46, 2.65, 2.03, 1.56],
    7: [25.7, 19.83, 15.3, 10.21, 12.58, 9.2, 6.72, 4.92, 5.26, 4.03, 3.1, 2.38, 1.82, 1.4],
    8: [29.6, 22.76, 17.5, 11.58, 14.16, 10.29, 7.48, 5.43, 5.78, 4.41, 3.37, 2.57, 1.96, 1.5],
    9: [34.6, 26.37, 20.1, 13.37, 16.44, 12.0, 8.75, 6.39, 6.81, 5.22, 4.0, 3.07, 2.35, 1.8],
    16: [110.7, 84.96, 65.2, 50.04, 38.4, 24.21, 28.2, 19.74, 20.24, 14.97, 11.08, 10.82, 8.3,
         6.36, 4.88, 4.65, 3.66, 2.88, 2.26, 1.78, 1.4],
    17: [128.0, 96.41, 72.62, 54.7, 41.2, 25.97, 30.25, 21.17, 21.71, 16.06, 11.88, 11.6, 8.89,
         6.82, 5.23, 4.99, 3.92, 3.08, 2.43, 1.91, 1.5],
}


def _table(name):
    orders, exps, inits = {}, {}, {}
    if name == "gauss":
        for z, (o, e, i) in _GAUSS.items():
            orders[z], exps[z], inits[z] = np.asarray(o), np.asarray(e), np.asarray(i)
    elif name == "slater":
        for z, e in _SLATER_EXPONENTS.items():
            k = len(e)
            orders[z], exps[z], inits[z] = np.ones(k), np.asarray(e), np.full(k, 1.0 / k)
    else:
        raise ValueError(name)
    return orders, exps, inits


def shell_prefactor(n, alpha):
    """N(alpha, n) = n alpha**(3/n) / (4 pi Gamma(3/n)) (``core/basis.py:161``)."""
    return n * alpha ** (3.0 / n) / (4.0 * math.pi * math.gamma(3.0 / n))


def evaluate_function(n, population, alpha, r, nderiv=0, axis=None):
    """``population * N(alpha, n) exp(-alpha r**n)`` and optionally the
    derivative term ``-n r**(n-1) f`` (``core/basis.py:85-186``).

    The derivative omits the factor ``alpha``, exactly as the reference
    computes it (``core/basis.py:164-165``); nothing on the partitioning path
    uses it.

    Scalars or 1-D arrays for ``n``, ``population`` and ``alpha``; with arrays
    the result has one row per shell and ``axis`` sums over shells.
    """
    if np.any(np.asarray(n) <= 0):
        raise ValueError("n must be positive")
    if np.any(np.asarray(alpha) < 0):
        raise ValueError("alpha must be non-negative")
    if not isinstance(r, np.ndarray):
        raise ValueError("r must be a numpy array")
    vec = not np.isscalar(n)
    if vec:
        n = np.asarray(n, dtype=float)
        alpha = np.asarray(alpha, dtype=float)
        population = np.asarray(population, dtype=float)
        gam = np.array([math.gamma(3.0 / x) for x in n])
        pref = (population * n * alpha ** (3.0 / n) / (4.0 * np.pi * gam))[:, None]
        alpha_, n_, r_ = alpha[:, None], n[:, None], r[None, :]
    else:
        pref = population * n * alpha ** (3.0 / n) / (4.0 * np.pi * math.gamma(3.0 / n))
        alpha_, n_, r_ = alpha, n, r
    f = pref * np.exp(-alpha_ * r_**n_)
    if nderiv > 0:
        df = -n_ * r_ ** (n_ - 1) * f
    if vec and axis is not None:
        f = np.sum(f, axis=axis)
        if nderiv > 0:
            df = np.sum(df, axis=axis)
    if nderiv == 0:
        return f
    if nderiv == 1:
        return f, df
    raise NotImplementedError


def load_params(filename, extension="json"):
    """Read ``{Z: [orders, exponents, initials]}`` from a JSON file.

    (YAML input needs PyYAML, which is optional here.)"""
    if extension.lower() == "json":
        with open(filename) as fh:
            data = json.load(fh)
    elif extension.lower() == "yaml":
        import yaml  # optional dependency

        with open(filename) as fh:
            data = yaml.safe_load(fh)
    else:
        raise AssertionError("Format must be 'json' or 'yaml'.")
    orders, exps, inits = {}, {}, {}
    for number, values in data.items():
        z = int(number)
        orders[z] = np.asarray(values[0], dtype=float)
        exps[z] = np.asarray(values[1], dtype=float)
        inits[z] = np.asarray(values[2], dtype=float)
    return orders, exps, inits


class BasisFuncHelper:
    """Base of the basis-function helpers (per-element shell tables)."""

    def __init__(self, initials, *args, **kwargs):
        self._initials = initials

    @property
    def initials(self):
        return self._initials

    def get_nshell(self, number):
        raise NotImplementedError

    def get_initial(self, number, ishell=None):
        v = np.asarray(self.initials[number], dtype=float)
        return v.copy() if ishell is None else v[ishell]

    def compute_proshell_dens(self, number, ishell, population, points, nderiv=0):
        raise NotImplementedError

    def compute_proatom_dens(self, number, populations, points, nderiv=0):
        y = d = 0.0
        for i in range(self.get_nshell(number)):
            res = self.compute_proshell_dens(number, i, populations[i], points, nderiv)
            if nderiv == 0:
                y = y + res
            elif nderiv == 1:
                y = y + res[0]
                d = d + res[1]
            else:
                raise NotImplementedError
        if nderiv == 0:
            return y
        if nderiv == 1:
            return y, d
        raise RuntimeError("The argument `nderiv` should only be 0 or 1.")


class AnalyticBasisFuncHelper(BasisFuncHelper):
    """Analytic (closed-form) basis functions."""


class ExpBasisFuncHelper(AnalyticBasisFuncHelper):
    """Shells ``N(alpha, n) exp(-alpha r**n)`` with per-element tables of
    orders ``n``, exponents ``alpha`` and initial populations."""

    def __init__(self, exponents_orders, exponents=None, initials=None):
        super().__init__(initials)
        self._orders = exponents_orders
        self._exponents = exponents

    @property
    def orders(self):
        return self._orders

    @property
    def exponents(self):
        return self._exponents

    def get_nshell(self, number):
        return len(self.exponents[number])

    def get_order(self, number, ishell=None):
        v = np.asarray(self.orders[number], dtype=float)
        return v if ishell is None else float(v[ishell])

    def get_exponent(self, number, ishell=None):
        v = np.asarray(self.exponents[number], dtype=float)
        return v.copy() if ishell is None else float(v[ishell])

    def get_prefactors(self, number):
        """N(alpha_k, n_k) for every shell of element ``number``."""
        return np.array([shell_prefactor(n, a) for n, a in
                         zip(self.get_order(number), self.get_exponent(number))])

    def compute_proshell_dens(self, number, ishell, population, points, nderiv=0):
        return evaluate_function(self.get_order(number, ishell), population,
                                 self.get_exponent(number, ishell), points, nderiv)

    @classmethod
    def from_function_type(cls, func_type="gauss"):
        assert func_type in ["gauss", "slater"]
        return cls(*_table(func_type))

    @classmethod
    def from_file(cls, filename):
        ext = "yaml" if str(filename).endswith(".yaml") else "json"
        orders, exponents, initials = load_params(filename, extension=ext)
        for number, exps in exponents.items():
            if number not in initials:
                initials[number] = np.ones_like(exps) / len(exps)
        return cls(orders, exponents, initials)

    from_json = from_file
    from_yaml = from_file
