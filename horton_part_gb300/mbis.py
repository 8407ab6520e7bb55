"""Minimal Basis Iterative Stockholder (MBIS) on the GPU.

Same class name, constructor and results as horton-part's ``mbis.py``
(``MBISWPart`` ``mbis.py:206-362``). The pro-atom of atom a is a sum of
Slater shells N_k S_k^3 exp(-S_k r) / (8 pi); the inner fixed point
N_k <- int w rho_a t_k/pro, S_k <- 3 N_k / int w rho_a t_k r / pro runs for all
atoms at once on the device (``mbis.py:81-163``).
"""

from __future__ import annotations

import numpy as np

from .part import GPUStockholderWPart

__all__ = ["MBISWPart", "get_nshell", "get_initial_mbis_propars"]


def get_nshell(number: int):
    """Number of Slater shells of an element (``mbis.py:36-46``)."""
    noble = np.array([2, 10, 18, 36, 54, 86, 118])
    return noble.searchsorted(number) + 1


def get_initial_mbis_propars(number: int):
    """Initial (N_k, S_k) pairs (``mbis.py:49-78``)."""
    nshell = get_nshell(number)
    propars = np.zeros(2 * nshell, float)
    s0 = 2.0 * number
    alpha = (2.0 / s0) ** (1.0 / (nshell - 1)) if nshell > 1 else 1.0
    nel_in_shell = np.array([2.0, 8.0, 8.0, 18.0, 18.0, 32.0, 32.0])
    for ishell in range(nshell):
        propars[2 * ishell] = nel_in_shell[ishell]
        propars[2 * ishell + 1] = s0 * alpha**ishell
    propars[-2] = number - propars[:-2:2].sum()
    return propars


class MBISWPart(GPUStockholderWPart):
    """Minimal Basis Iterative Stockholder (MBIS)."""

    name = "mbis"
    _scheme = "mbis"
    _inner_warning = "MBIS not converged, but still go ahead!"
    _supports_atom_grids = True  # grid_type 1: spherical averages on the radial grids

    def _shell_tables(self):
        self._ranges = [0]
        self._nshells = []
        for z in self.numbers:
            nshell = int(get_nshell(z))
            self._ranges.append(self._ranges[-1] + 2 * nshell)
            self._nshells.append(nshell)
        offsets = np.concatenate([[0], np.cumsum(self._nshells)]).astype(np.int32)
        init = np.concatenate([get_initial_mbis_propars(z) for z in self.numbers])
        return offsets, init, None, None

    def _job_extra(self):
        return {"inner_maxiter": 2000}

    def _finalize_extra(self, res):
        """Core/valence split (``mbis.py:347-362``)."""
        propars = res["propars"]
        valence_charges = np.array([-propars[self._ranges[a + 1] - 2] for a in range(self.natom)])
        valence_widths = np.array([1.0 / propars[self._ranges[a + 1] - 1] for a in range(self.natom)])
        self.cache.dump("core_charges", res["charges"] - valence_charges, tags="o")
        self.cache.dump("valence_charges", valence_charges, tags="o")
        self.cache.dump("valence_widths", valence_widths, tags="o")

    def get_proatom_rho(self, iatom, propars=None, **kwargs):
        """Pro-atom density and derivative on the molecular grid (``mbis.py:234-261``)."""
        if propars is None:
            propars = self.cache.load("propars")
        r = self.radial_distances[iatom]
        y = np.zeros(len(r))
        d = np.zeros(len(r))
        my = propars[self._ranges[iatom]:self._ranges[iatom + 1]]
        for k in range(self._nshells[iatom]):
            n, s = my[2 * k:2 * k + 2]
            f = n * s**3 * np.exp(-s * r) / (8 * np.pi)
            y += f
            d -= s * f
        return y, d
