"""Gaussian Iterative Stockholder Analysis (GISA) on the GPU.

Mirrors ``GaussianISAWPart`` (``gisa.py:109-345`` in horton-part): fixed
s-type Gaussian shells per element; per outer iteration each atom's
populations solve the quadratic program

    min 1/2 c^T P c + q^T c,  c >= 0,  sum c = int w rho_a
    P_kl = 2 / pi^1.5 (a_k a_l)^1.5 / (a_k + a_l)^1.5,  q_k = -2 int w g_k rho_a

(``gisa.py:348-421``). The q-vector moments run on the GPU; the QP is solved
on the device by an exact primal active-set method, one thread per atom.
The reference hands the same program to quadprog (through qpsolvers); any
``solver`` name is accepted and solved exactly.
"""

from __future__ import annotations

import numpy as np

from .basis import AnalyticBasisFuncHelper, ExpBasisFuncHelper
from .part import GPUStockholderWPart

__all__ = ["GaussianISAWPart", "init_propars", "shell_tables_from_helper"]


def init_propars(part):
    """Per-atom initial populations (``gisa.py:68-88``): initials below 1e-4
    are raised to 1e-4 and each atom is normalised to its pseudo number. The
    device then rescales all populations to the integrated density."""
    part._ranges = [0]
    part._nshells = []
    parts = []
    for iatom in range(part.natom):
        nshell = part.bs_helper.get_nshell(part.numbers[iatom])
        part._ranges.append(part._ranges[-1] + nshell)
        part._nshells.append(nshell)
        inits = np.array(part.bs_helper.get_initial(part.numbers[iatom]), dtype=float)
        inits[inits < 1e-4] = 1e-4
        parts.append(inits / np.sum(inits) * part.pseudo_numbers[iatom])
    return np.concatenate(parts)


def get_proatom_rho_basis(part, iatom, propars=None):
    """Pro-atom density and derivative term on the molecular grid (``gisa.py:42-65``)."""
    if propars is None:
        propars = part.cache.load("propars")
    pops = propars[part._ranges[iatom]:part._ranges[iatom + 1]]
    return part.bs_helper.compute_proatom_dens(part.numbers[iatom], pops,
                                               part.radial_distances[iatom], 1)


def shell_tables_from_helper(part):
    if not isinstance(part.bs_helper, AnalyticBasisFuncHelper):
        raise NotImplementedError("numeric basis functions are not available on the GPU path")
    init = init_propars(part)
    orders = np.concatenate([part.bs_helper.get_order(z) for z in part.numbers]).astype(float)
    exps = np.concatenate([part.bs_helper.get_exponent(z) for z in part.numbers]).astype(float)
    offsets = np.asarray(part._ranges, dtype=np.int32)
    return offsets, init, orders, exps


class GaussianISAWPart(GPUStockholderWPart):
    """Iterative Stockholder Partitioning with Gaussian pro-atoms (GISA)."""

    name = "gisa"
    _scheme = "gisa"
    # grid_type 1: the update works on the spherical averages on the radial
    # grids (aLISA: the sc solver)
    _supports_atom_grids = True

    def __init__(self, coordinates, numbers, pseudo_numbers, grid, moldens, spindens=None, lmax=3,
                 logger=None, threshold=1e-6, maxiter=500, inner_threshold=1e-8,
                 radius_cutoff=np.inf, solver="quadprog", solver_options=None, grid_type=1,
                 **kwargs):
        if callable(solver):
            raise NotImplementedError("custom solver callables do not run on the GPU path")
        self._solver = solver
        self._solver_options = solver_options or {}
        self._bs_helper = kwargs.pop("bs_helper", None)
        super().__init__(coordinates, numbers, pseudo_numbers, grid, moldens, spindens, lmax, logger,
                         threshold=threshold, maxiter=maxiter, inner_threshold=inner_threshold,
                         grid_type=grid_type, **kwargs)

    @property
    def bs_helper(self):
        if self._bs_helper is None:
            self._bs_helper = ExpBasisFuncHelper.from_function_type()
        return self._bs_helper

    def _shell_tables(self):
        return shell_tables_from_helper(self)

    def _solver_name(self):
        return "quadprog"

    def get_proatom_rho(self, iatom, propars=None, **kwargs):
        return get_proatom_rho_basis(self, iatom, propars)
