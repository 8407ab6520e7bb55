"""Linear Iterative Stockholder Analysis (aLISA) on the GPU.

Mirrors ``LinearISAWPart`` (``alisa.py:1155-1335`` in horton-part). Each atom's
pro-atom is sum_k c_k g_k(r) with fixed shells; per outer iteration the
coefficients are refitted by one of the reference's inner solvers, run for
all atoms at once on the device:

``sc``        c_k <- int w c_k g_k rho_a / pro (``alisa.py:193-291``)
``sc-1-iter`` one such update per outer iteration (``alisa.py:294-353``): the
              ``sc`` kernels with one inner iteration and no inner
              convergence test (so no warning)
``newton``    exact Newton on the KL objective (``alisa.py:543-602``)
``m-newton``  Newton with the positivity line search (``alisa.py:605-664``)
``quasi-newton`` BFGS on the inverse Hessian with the same line search
              (``alisa.py:683-750``, ``_solver_general_newton`` mode "bfgs")

``cvxopt`` (the reference's class default) needs the cvxopt package; its
optimum is the non-negative KL minimiser, which the multiplicative ``sc``
update also reaches, so ``cvxopt`` is served by ``sc``. Other reference
solvers (``diis``, ``cdiis``, ``trust-region``, ``sc-plus-convex``) are not
on the GPU path and raise ``NotImplementedError``.
"""

from __future__ import annotations

import numpy as np

from .basis import AnalyticBasisFuncHelper, ExpBasisFuncHelper
from .gisa import GaussianISAWPart, shell_tables_from_helper

__all__ = ["LinearISAWPart", "setup_bs_helper"]

_SOLVERS = {"sc": "sc", "sc-1-iter": "sc", "cvxopt": "sc", "newton": "newton",
            "m-newton": "m-newton", "quasi-newton": "quasi-newton"}


def setup_bs_helper(part):
    """Basis helper from ``basis_func`` (``alisa.py:1130-1152``)."""
    if part._bs_helper is None:
        if isinstance(part.basis_func, str):
            name = part.basis_func.lower()
            if name in ("gauss", "slater"):
                if part.basis_type != "analytic":
                    raise NotImplementedError("numeric basis functions are not available on the GPU path")
                part._bs_helper = ExpBasisFuncHelper.from_function_type(name)
            else:
                part._bs_helper = ExpBasisFuncHelper.from_file(part.basis_func)
        elif isinstance(part.basis_func, AnalyticBasisFuncHelper):
            part._bs_helper = part.basis_func
        else:
            raise NotImplementedError(
                "The type of basis_func should be one of string or class BasisFuncHelper.")
    return part._bs_helper


class LinearISAWPart(GaussianISAWPart):
    """Linear Iterative Stockholder Analysis (aLISA)."""

    name = "lisa"

    def __init__(self, coordinates, numbers, pseudo_numbers, grid, moldens, spindens=None, lmax=3,
                 logger=None, threshold=1e-6, maxiter=500, inner_threshold=1e-8,
                 radius_cutoff=np.inf, solver="cvxopt", solver_options=None, basis_func="gauss",
                 basis_type="analytic", grid_type=1, **kwargs):
        self.basis_func = basis_func
        self.basis_type = basis_type
        if callable(solver):
            raise NotImplementedError("custom solver callables do not run on the GPU path")
        if solver not in _SOLVERS:
            raise NotImplementedError(f"aLISA solver {solver!r} is not on the GPU path "
                                      f"(available: {sorted(_SOLVERS)})")
        super().__init__(coordinates, numbers, pseudo_numbers, grid, moldens, spindens, lmax, logger,
                         threshold, maxiter, inner_threshold, radius_cutoff, "quadprog",
                         solver_options, grid_type, **kwargs)
        self._solver = solver
        self._scheme = "lisa"

    @property
    def bs_helper(self):
        return setup_bs_helper(self)

    def _shell_tables(self):
        return shell_tables_from_helper(self)

    def _solver_name(self):
        return _SOLVERS[self._solver]

    def _report_warnings(self, info):
        if self._solver == "sc-1-iter":  # one update by design: no inner convergence test
            from . import _lib

            info.warnings &= ~_lib.WARN_INNER_NOT_CONVERGED
        super()._report_warnings(info)

    def _job_extra(self):
        opts = dict(self._solver_options)
        if self._solver == "sc-1-iter":
            return {"inner_maxiter": 1}
        if _SOLVERS[self._solver] == "sc":
            return {"inner_maxiter": int(float(opts.get("max_niter_inner", 100000)))}
        extra = {"inner_maxiter": int(opts.get("niter", 10000))}
        if _SOLVERS[self._solver] in ("m-newton", "quasi-newton"):
            extra["linspace_size"] = int(opts.get("linspace_size", 20))
            extra["tau"] = float(opts.get("tau", 1.0))
        return extra
