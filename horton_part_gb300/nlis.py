"""NLIS and GMBIS on the GPU.

Same class names, constructors and results as horton-part's ``nlis.py``
(``NLISWPart`` ``nlis.py:198-367``) and ``gmbis.py`` (``GMBISWPart``
``gmbis.py:55-156``). The pro-atom of atom a is a sum of shells
N_k n_k S_k^(3/n_k) exp(-S_k r^n_k) / (4 pi Gamma(3/n_k)) with fixed orders
n_k (``exp_n_dict``); the inner fixed point N_k <- m0_k, S_k <- 3 / (n_k m1_k)
runs for all atoms at once on the device (``nlis.py:99-195``), in FP64. GMBIS
is NLIS with the MBIS shell count and initial populations.
"""

from __future__ import annotations

import numpy as np

from .mbis import get_nshell
from .part import GPUStockholderWPart

__all__ = ["NLISWPart", "GMBISWPart", "get_nlis_nshell", "get_initial_nlis_propars",
           "get_initial_gmbis_propars"]


def get_nlis_nshell(number, nshell_dict):
    """Shells of an element (``nlis.py:23-35``)."""
    return nshell_dict.get(number, get_nshell(number))


def get_initial_nlis_propars(number, exp_n_dict, nshell_dict, logger=None):
    """Initial (N, S, n) triples (``nlis.py:38-96``): N = Z / nshell, S from
    2 Z down to 0.5 geometrically, n from ``exp_n_dict[(Z, k)]`` (else 1)."""
    nbs = get_nlis_nshell(number, nshell_dict)
    propars = np.ones(3 * nbs, float)
    s0 = 2.0 * number
    alpha = (0.5 / s0) ** (1.0 / (nbs - 1)) if nbs > 1 else 1.0
    for ibs in range(nbs):
        propars[3 * ibs] = number / nbs
        propars[3 * ibs + 1] = s0 * alpha**ibs
        propars[3 * ibs + 2] = exp_n_dict[(number, ibs)] if (number, ibs) in exp_n_dict else 1.0
    return propars


def get_initial_gmbis_propars(number, exp_n_dict, logger=None):
    """Initial (N, S, n) triples of GMBIS (``gmbis.py:17-52``): the MBIS shell
    populations and exponents, n from ``exp_n_dict`` (else 1)."""
    nshell = get_nshell(number)
    propars = np.zeros(3 * nshell, float)
    s0 = 2.0 * number
    alpha = (2.0 / s0) ** (1.0 / (nshell - 1)) if nshell > 1 else 1.0
    nel_in_shell = np.array([2.0, 8.0, 8.0, 18.0, 18.0, 32.0, 32.0])
    for ishell in range(nshell):
        propars[3 * ishell] = nel_in_shell[ishell]
        propars[3 * ishell + 1] = s0 * alpha**ishell
        propars[3 * ishell + 2] = (exp_n_dict[(number, ishell)]
                                   if (number, ishell) in exp_n_dict else 1.0)
    propars[-3] = number - propars[:-3:3].sum()
    return propars


def _unit_shell(s, n, r):
    from math import gamma

    return n * s ** (3.0 / n) * np.exp(-s * r**n) / (4 * np.pi * gamma(3.0 / n))


class NLISWPart(GPUStockholderWPart):
    """Non-Linear approximation of Iterative Stockholder (NLIS)."""

    name = "nlis"
    _scheme = "nlis"
    _inner_warning = "NLIS not converged, but still go ahead!"
    _supports_atom_grids = True  # grid_type 1 (the class default): radial inner solve

    def __init__(self, coordinates, numbers, pseudo_numbers, grid, moldens, spindens=None, lmax=3,
                 logger=None, threshold=1e-6, maxiter=500, inner_threshold=1e-8, exp_n_dict=1.0,
                 nshell_dict=None, grid_type=1, **kwargs):
        self._exp_n_dict = exp_n_dict
        self._nshell_dict = nshell_dict or {}
        super().__init__(coordinates, numbers, pseudo_numbers, grid, moldens, spindens=spindens,
                         lmax=lmax, logger=logger, threshold=threshold, maxiter=maxiter,
                         inner_threshold=inner_threshold, grid_type=grid_type, **kwargs)

    def _nshell_of(self, z):
        return int(get_nlis_nshell(z, self._nshell_dict))

    def _initial_of(self, z):
        return get_initial_nlis_propars(z, self._exp_n_dict, self._nshell_dict, logger=self.logger)

    def _shell_tables(self):
        self._ranges = [0]
        self._nshells = []
        for z in self.numbers:
            nshell = self._nshell_of(int(z))
            self._ranges.append(self._ranges[-1] + 3 * nshell)
            self._nshells.append(nshell)
        offsets = np.concatenate([[0], np.cumsum(self._nshells)]).astype(np.int32)
        init = np.concatenate([self._initial_of(int(z)) for z in self.numbers])
        return offsets, init, None, None

    def _job_extra(self):
        return {"inner_maxiter": 2000}

    def _finalize_extra(self, res):
        """Core/valence split (``nlis.py:351-367``)."""
        propars = res["propars"]
        valence_charges = np.array([-propars[self._ranges[a + 1] - 3] for a in range(self.natom)])
        valence_widths = np.array([1.0 / propars[self._ranges[a + 1] - 2] for a in range(self.natom)])
        self.cache.dump("core_charges", res["charges"] - valence_charges, tags="o")
        self.cache.dump("valence_charges", valence_charges, tags="o")
        self.cache.dump("valence_widths", valence_widths, tags="o")

    def get_proatom_rho(self, iatom, propars=None, **kwargs):
        """Pro-atom density and its radial derivative on the molecular grid
        (``nlis.py:281-296``)."""
        if propars is None:
            propars = self.cache.load("propars")
        r = self.radial_distances[iatom]
        y = np.zeros(len(r))
        d = np.zeros(len(r))
        my = propars[self._ranges[iatom]:self._ranges[iatom + 1]]
        for k in range(self._nshells[iatom]):
            nk, s, n = my[3 * k:3 * k + 3]
            f = nk * _unit_shell(s, n, r)
            y += f
            d -= nk * s * n * r ** (n - 1) * f
        return y, d


class GMBISWPart(NLISWPart):
    """Generalized Minimal Basis Iterative Stockholder (GMBIS)."""

    name = "gmbis"

    def __init__(self, coordinates, numbers, pseudo_numbers, grid, moldens, spindens=None, lmax=3,
                 logger=None, threshold=1e-6, maxiter=500, inner_threshold=1e-8, exp_n_dict=1.0,
                 grid_type=1, **kwargs):
        super().__init__(coordinates, numbers, pseudo_numbers, grid, moldens, spindens=spindens,
                         lmax=lmax, logger=logger, threshold=threshold, maxiter=maxiter,
                         inner_threshold=inner_threshold, exp_n_dict=exp_n_dict, nshell_dict={},
                         grid_type=grid_type, **kwargs)

    def _nshell_of(self, z):
        return int(get_nshell(z))

    def _initial_of(self, z):
        return get_initial_gmbis_propars(z, self._exp_n_dict, logger=self.logger)
