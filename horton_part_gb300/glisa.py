"""Global Linear Iterative Stockholder Analysis (gLISA) on the GPU.

Mirrors ``GlobalLinearISAWPart`` (``glisa.py:55-1028`` in horton-part): all
shell populations of the molecule form one convex problem. Per solver
iteration the device evaluates the promolecule rho0 = G^T c, the gradient
-int rho g_i / rho0 and the Hessian int rho g_i g_j / rho0^2 =
(G^T diag(w rho / rho0^2) G)_ij over the molecular grid
(``glisa.py:411-479``), solves the Newton system by Cholesky and applies the
step (``newton``), the positivity line search (``m-newton``) or the
self-consistent update (``sc``, ``glisa.py:805-879``).

``cvxopt`` (the class default in the reference) needs the cvxopt package; it
is served by a projected Newton method on c >= 0 (solver name ``pnewton``),
which reaches the same non-negative optimum of the convex objective.

``diis``, ``cdiis``, ``quasi-newton`` and ``trust-region`` iterate on the host
(:mod:`horton_part_gb300.glisa_solvers`) with every pass over the grid on the
device; they run in FP64 (``precision="fp64"``).
"""

from __future__ import annotations

import numpy as np

from .alisa import setup_bs_helper
from .gisa import get_proatom_rho_basis, shell_tables_from_helper
from .glisa_solvers import HOST_SOLVERS
from .part import GPUStockholderWPart

__all__ = ["GlobalLinearISAWPart"]

_SOLVERS = {"newton": "newton", "m-newton": "m-newton", "sc": "sc", "cvxopt": "pnewton",
            "pnewton": "pnewton"}
# solvers whose iterations run on the host, every grid pass on the device
# (horton_part_gb300.glisa_solvers); the job itself is an FP64 job
for _name in HOST_SOLVERS:
    _SOLVERS[_name] = "newton"


class GlobalLinearISAWPart(GPUStockholderWPart):
    name = "glisa"
    _scheme = "glisa"
    _supports_atom_grids = True  # grid_type 1: the change is measured on the radial grids
    _has_charge_history = False
    _dumps_change = False

    def __init__(self, coordinates, numbers, pseudo_numbers, grid, moldens, spindens=None, lmax=3,
                 logger=None, threshold=1e-6, maxiter=500, solver="cvxopt", solver_options=None,
                 basis_func="gauss", grid_type=1, basis_type="analytic", **kwargs):
        if callable(solver):
            raise NotImplementedError("custom solver callables do not run on the GPU path")
        if solver not in _SOLVERS:
            raise NotImplementedError(f"gLISA solver {solver!r} is not on the GPU path "
                                      f"(available: {sorted(_SOLVERS)})")
        self.basis_func = basis_func
        self.basis_type = basis_type
        self._bs_helper = None
        self._solver = solver
        self._solver_options = solver_options or {}
        kwargs.pop("inner_threshold", None)
        super().__init__(coordinates, numbers, pseudo_numbers, grid, moldens, spindens, lmax, logger,
                         threshold=threshold, maxiter=maxiter, grid_type=grid_type, **kwargs)

    @property
    def bs_helper(self):
        return setup_bs_helper(self)

    @property
    def maxiter(self):
        return self._maxiter

    @property
    def threshold(self):
        return self._threshold

    @property
    def mol_pop(self):
        return self.grid.integrate(self._moldens)

    def _shell_tables(self):
        return shell_tables_from_helper(self)

    def _solver_name(self):
        return _SOLVERS[self._solver]

    def _host_solver(self):
        return self._solver if self._solver in HOST_SOLVERS else None

    def _run_job(self, job):
        """Newton-type and sc solvers run whole on the device; the host solvers
        drive the job's evaluation service and end it with ``finish``."""
        name = self._host_solver()
        if name is None:
            job.run()
            return None
        from . import glisa_solvers as hs

        opts = dict(self._solver_options)
        offsets, x0, _, _ = self._shell_tables()
        mol_pop = self.grid.integrate(self._moldens)
        x0 = x0 / x0.sum() * mol_pop  # gisa.py:85-86, as the device does at job start
        exps = [self.bs_helper.get_exponent(z) for z in self.numbers]
        changes = None
        if name == "diis":
            maxiter = int(opts.pop("maxiter", 1000))
            x, niter, hist = hs.solve_diis(job, x0, self._threshold, maxiter=maxiter, **opts)
            hist = hist[1:]
        elif name == "cdiis":
            maxiter = int(opts.pop("maxiter", self._maxiter))
            conv, niter, norms, x, hist = hs.solve_cdiis(job, x0, self._threshold, maxiter=maxiter,
                                                          **opts)
            if not conv:
                raise RuntimeError("Not converged!")
            hist, changes = hist[1:], list(norms)
        elif name == "quasi-newton":
            maxiter = int(opts.pop("maxiter", 1000))
            opts.pop("mode", None)
            x, niter, hist, ents, changes = hs.solve_quasi_newton(
                job, x0, self._threshold, exps, np.asarray(offsets), maxiter=maxiter,
                niter_exact_newton=int(opts.get("niter_exact_newton", 0)))
        else:  # trust-region
            x, niter = hs.solve_trust_region(job, x0, self._threshold, self._maxiter, mol_pop,
                                             allow_neg_pars=bool(opts.get("allow_neg_pars", False)))
            hist = []
        if name != "quasi-newton":
            ents = [job.evaluate(h, 0)[0] for h in hist]
        job.finish(x, niter)
        return {"history_propars": np.array(hist, dtype=float).reshape(len(hist), x0.size),
                "history_entropies": np.array(ents), "history_changes": np.array(changes or []),
                "history_charges": np.zeros((0, self.natom))}

    def _make_job(self):
        if self._host_solver() and self._precision != "fp64":
            raise NotImplementedError(f"gLISA solver {self._solver!r} runs in FP64 (precision='fp64')")
        return self._make_job_device()

    def _job_extra(self):
        opts = dict(self._solver_options)
        name = _SOLVERS[self._solver]
        if self._host_solver():
            return {"maxiter": self._maxiter}
        # solver iteration limits: newton/m-newton 100 (glisa.py:573-591)
        maxiter = int(opts.get("maxiter", 100 if name != "sc" else self._maxiter))
        extra = {"maxiter": maxiter}
        if name == "m-newton":
            extra["linspace_size"] = int(opts.get("linspace_size", 40))
            extra["tau"] = float(opts.get("tau", 1.0))
        return extra

    def _make_job_device(self):
        # the solver's own iteration limit replaces the class maxiter
        saved = self._maxiter
        try:
            self._maxiter = self._job_extra()["maxiter"]
            extra = self._job_extra()
            extra.pop("maxiter")
            self._check_grid_type()
            offsets, init, orders, exps = self._shell_tables()
            from . import _lib
            from .molgrid import atom_grid_arrays

            ctx = self._context or _lib.default_context(0)
            # grid_type 1: the radial grids measure the change
            local = None if self.on_molgrid else atom_grid_arrays(self.grid)
            return _lib.Job(
                ctx, self._scheme, self.coordinates, self.pseudo_numbers, self.grid.points,
                self.grid.weights, self._moldens, offsets, init, shell_orders=orders,
                shell_exponents=exps, solver=self._solver_name(), precision=self._precision,
                grid_type=self.grid_type, threshold=self._threshold,
                inner_threshold=self._threshold, density_cutoff=self.density_cutoff,
                negative_cutoff=self.negative_cutoff, population_cutoff=self.population_cutoff,
                maxiter=self._maxiter, local=local, **extra)
        finally:
            self._maxiter = saved

    def get_proatom_rho(self, iatom, propars=None, **kwargs):
        return get_proatom_rho_basis(self, iatom, propars)
