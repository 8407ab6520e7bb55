"""Partitioning base classes: the reference's public API over the GPU path.

``Part``/``WPart`` keep horton-part's constructor arguments, properties and
``do_*`` entry points (``core/base.py:35-499``); ``GPUStockholderWPart``
replaces the Python stockholder loop (``core/stockholder.py``,
``core/iterstock.py``) with one call into ``libhpgpu.so`` and then fills
``part.cache`` with the same keys the reference stores.

GPU-only options (keyword arguments, all optional):

``precision``   ``"fp64"`` (default: every step in FP64), ``"mixed"`` (FP32
                evaluation with compensated sums and FP64 updates; gLISA: the
                Hessian on the tensor cores) or ``"ff"`` (MBIS: float-float
                evaluation on the FP32 pipes, FP64-class results).
``polish``      mixed precision: finish near the threshold in float-float
                (MBIS) or FP64 (default ``True``).
``context``     a :class:`horton_part_gb300._lib.Context` (device, stream,
                HBM budget); default: one shared context on device 0.
``store_at_weights``  fetch the per-atom ``at_weights_{i}`` arrays into the
                cache (default ``True``, as the reference).
"""

from __future__ import annotations

import logging
import time

import numpy as np

from . import _lib
from .cache import Cache, JustOnceClass, just_once
from .utils import DENSITY_CUTOFF, NEGATIVE_CUTOFF, POPULATION_CUTOFF, typecheck_geo

__all__ = ["Part", "WPart", "GPUStockholderWPart"]


def _setup_logger(logger):
    if not logger.handlers:
        handler = logging.StreamHandler()
        handler.setFormatter(logging.Formatter("%(levelname)s: %(message)s"))
        logger.addHandler(handler)
        logger.setLevel(logging.INFO)
        logger.propagate = False


class Part(JustOnceClass):
    """Geometry, density, grid and result cache of one partitioning problem.

    Public surface of horton-part's ``Part`` (``core/base.py:35-410``):
    constructor ``(coordinates, numbers, pseudo_numbers, grid, moldens,
    spindens, local, lmax, logger)``, the read-only properties, ``part[key]``
    for cached results and the ``do_*`` entry points. With ``local`` each atom
    integrates on its own atomic grid (``grid.atgrids[i]``), otherwise on the
    molecular grid.
    """

    name = None

    def __init__(self, coordinates, numbers, pseudo_numbers, grid, moldens, spindens, local, lmax,
                 logger, *args, **kwargs):
        super().__init__()
        checked = typecheck_geo(coordinates, numbers, pseudo_numbers)
        self._natom, self._coordinates, self._numbers, self._pseudo_numbers = checked
        self._grid, self._moldens, self._spindens = grid, moldens, spindens
        self._local, self._lmax = bool(local), lmax
        self._cache = Cache()
        self.logger = logger
        self._subgrids = grid.atgrids if self._local else None

    # -- read-only state ------------------------------------------------------
    natom = property(lambda self: self._natom)
    coordinates = property(lambda self: self._coordinates)
    numbers = property(lambda self: self._numbers)
    pseudo_numbers = property(lambda self: self._pseudo_numbers)
    local = property(lambda self: self._local)
    lmax = property(lambda self: self._lmax)
    cache = property(lambda self: self._cache)

    @property
    def grid(self):
        return self._grid

    @property
    def nelec(self):
        """Electrons in the molecular density (integral over the molecular grid)."""
        return self._grid.integrate(self._moldens)

    def __getitem__(self, key):
        return self._cache.load(key)

    def variables_stored_in_cache(self):
        return list(self._cache.iterkeys())

    def clear(self):
        """Forget every result: run-once marks and the cache."""
        super().clear()
        self._cache.clear()

    # -- grids and fields -------------------------------------------------------
    def get_grid(self, index=None):
        """Atom ``index``'s integration grid (its atomic grid when local)."""
        if index is None or not self._local:
            return self._grid
        return self._subgrids[index]

    def _field_on(self, index, field, output):
        values = field if index is None or not self._local else self.to_atomic_grid(index, field)
        if output is not None:
            output[:] = values
        return values

    def get_moldens(self, index=None, output=None):
        return self._field_on(index, self._moldens, output)

    def get_spindens(self, index=None, output=None):
        return self._field_on(index, self._spindens, output)

    def to_atomic_grid(self, index, data):
        raise NotImplementedError

    def get_wcor(self, index):
        """Weight correction of atom ``index``'s integrals (none here)."""
        return 1.0

    def _aim_integral(self, index, field):
        """Integral of ``at_weights_{index} * field`` over atom ``index``'s grid."""
        weights = self._cache.load(f"at_weights_{index}")
        if self._local and weights.shape == self._grid.weights.shape:
            weights = self.to_atomic_grid(index, weights)
        on_atom = self._field_on(index, field, None)
        return self.get_grid(index).integrate(weights, on_atom * self.get_wcor(index))

    def compute_pseudo_population(self, index):
        return self._aim_integral(index, self._moldens)

    # -- entry points -----------------------------------------------------------
    @just_once
    def do_partitioning(self):
        self.update_at_weights()

    def update_at_weights(self, *args, **kwargs):
        raise NotImplementedError

    @just_once
    def do_populations(self):
        """``populations`` = AIM electron counts + (numbers - pseudo_numbers)."""
        if "populations" in self._cache:
            return
        self.do_partitioning()
        pseudo = np.array([self.compute_pseudo_population(i) for i in range(self._natom)])
        self._cache.dump("pseudo_populations", pseudo, tags="o")
        self._cache.dump("populations", pseudo + (self._numbers - self._pseudo_numbers), tags="o")

    @just_once
    def do_charges(self):
        """``charges`` = numbers - populations."""
        if "charges" in self._cache:
            return
        self.do_populations()
        self._cache.dump("charges", self._numbers - self._cache.load("populations"), tags="o")

    @just_once
    def do_spin_charges(self):
        """``spin_charges``: AIM integrals of the spin density (when one was given)."""
        if self._spindens is None:
            return
        self.do_partitioning()
        spin = np.array([self._aim_integral(i, self._spindens) for i in range(self._natom)])
        self._cache.dump("spin_charges", spin, tags="o")

    def do_all(self):
        """Run every implemented ``do_*`` method; return the output keys."""
        self.do_partitioning()
        self.do_populations()
        self.do_charges()
        self.do_spin_charges()
        return list(self._cache.iterkeys(tags="o"))


# grid_type -> (integrals on the molecular grid, atomic grids not needed at all)
# 1: atomic grids for everything, the molecular grid only for the weights;
# 2: molecular grid for everything, atomic grids for constraints;
# 3: molecular grid only.
_GRID_TYPES = {1: (False, False), 2: (True, False), 3: (True, True)}


class WPart(Part):
    """Partitioning on a Becke molecular grid with optional atomic grids.

    Public surface of horton-part's ``WPart`` (``core/base.py:413-636``):
    ``grid_type`` (1, 2 or 3), the three numerical cutoffs, the iteration
    histories and the radial distances of the grid points to every atom.
    """

    def __init__(self, coordinates, numbers, pseudo_numbers, grid, moldens, spindens=None, lmax=3,
                 logger=None, grid_type=1, density_cutoff=DENSITY_CUTOFF,
                 negative_cutoff=NEGATIVE_CUTOFF, population_cutoff=POPULATION_CUTOFF, **kwargs):
        self._grid_type = grid_type
        self.setup_grids()
        local = not self._only_use_molgrid
        if local and getattr(grid, "atgrids", None) is None:
            raise ValueError(f"grid_type={grid_type} integrates on atomic grids, but the grid "
                             "object carries none (grid.atgrids is None)")
        if logger is None:
            logger = logging.getLogger(type(self).__name__)
            _setup_logger(logger)
        for name in ("propars", "charges", "entropies", "changes", "time_update_at_weights",
                     "time_update_propars"):
            setattr(self, "history_" + name, [])
        self._radial_distances = []
        self._density_cutoff = density_cutoff
        self._negative_cutoff = negative_cutoff
        self._population_cutoff = population_cutoff
        super().__init__(coordinates, numbers, pseudo_numbers, grid, moldens, spindens, local, lmax,
                         logger)

    def setup_grids(self):
        if self._grid_type not in _GRID_TYPES:
            raise AssertionError(f"grid_type must be 1, 2 or 3, not {self._grid_type!r}")
        self._on_molgrid, self._only_use_molgrid = _GRID_TYPES[self._grid_type]

    grid_type = property(lambda self: self._grid_type)
    on_molgrid = property(lambda self: self._on_molgrid)
    only_use_molgrid = property(lambda self: self._only_use_molgrid)
    density_cutoff = property(lambda self: self._density_cutoff)
    negative_cutoff = property(lambda self: self._negative_cutoff)
    population_cutoff = property(lambda self: self._population_cutoff)

    def to_atomic_grid(self, index, data):
        """The slice of a molecular-grid array that belongs to atom ``index``."""
        if index is None or not self._local:
            return data
        lo, hi = self._grid.indices[index], self._grid.indices[index + 1]
        return data[lo:hi]

    @property
    def radial_distances(self):
        """|r_p - R_a| for every atom a (list of arrays over the molecular grid)."""
        self.calc_radial_distances()
        return self._radial_distances

    @just_once
    def calc_radial_distances(self):
        points = np.asarray(self._grid.points)
        self._radial_distances = [np.sqrt(((points - c) ** 2).sum(axis=1))
                                  for c in self._coordinates]


class GPUStockholderWPart(WPart):
    """Iterative stockholder partitioning executed by ``libhpgpu.so``.

    Subclasses define ``_scheme`` and the per-atom shell tables; the whole
    ``do_partitioning`` loop (``core/iterstock.py:159-193`` or
    ``glisa.py:248-281``) runs on the GPU and the cache receives the
    reference's keys.
    """

    _scheme = None
    _has_charge_history = True
    _dumps_change = True

    def __init__(self, coordinates, numbers, pseudo_numbers, grid, moldens, spindens=None, lmax=3,
                 logger=None, threshold=1e-6, maxiter=500, inner_threshold=1e-8, grid_type=1,
                 precision="fp64", context=None, store_at_weights=True, polish=True, **kwargs):
        self._threshold = threshold
        self._inner_threshold = inner_threshold if inner_threshold < threshold else threshold
        self._maxiter = maxiter
        if precision not in ("fp64", "mixed", "ff"):
            raise ValueError("precision must be 'fp64', 'mixed' or 'ff'")
        self._precision = precision
        self._polish = polish
        self._context = context
        self._store_at_weights = store_at_weights
        self._ranges = None
        self._nshells = None
        self._job_info = None
        kwargs.pop("radius_cutoff", None)
        kwargs.pop("local", None)
        super().__init__(coordinates, numbers, pseudo_numbers, grid, moldens, spindens, lmax, logger,
                         grid_type=grid_type, **kwargs)

    # -- to be provided by the schemes -----------------------------------------
    def _shell_tables(self):
        """Return (shell_offsets, initial_propars, orders or None, exponents or None)."""
        raise NotImplementedError

    def _solver_name(self):
        return "default"

    def _job_extra(self):
        return {}

    def _finalize_extra(self, res):
        pass

    def _run_job(self, job):
        """Run the job to the end on the device; a scheme whose iterations run
        on the host returns the histories it kept (else None)."""
        job.run()
        return None

    # -- the partitioning ------------------------------------------------------
    _supports_atom_grids = False  # grid_type 1 on the GPU (set by the scheme classes)

    def _check_grid_type(self):
        if not self.on_molgrid and not self._supports_atom_grids:
            raise NotImplementedError(
                "grid_type=1 (spherical averages on the atomic radial grids) is available for "
                "MBIS, GISA, aLISA (sc) and gLISA on the GPU path; use grid_type=2 or 3")

    def _make_job(self):
        from .molgrid import atom_grid_arrays

        self._check_grid_type()
        offsets, init, orders, exps = self._shell_tables()
        ctx = self._context or _lib.default_context(0)
        local = None if self.on_molgrid else atom_grid_arrays(self.grid)
        return _lib.Job(
            ctx, self._scheme, self.coordinates, self.pseudo_numbers, self.grid.points,
            self.grid.weights, self._moldens, offsets, init, shell_orders=orders,
            shell_exponents=exps, solver=self._solver_name(), precision=self._precision,
            grid_type=self.grid_type, threshold=self._threshold,
            inner_threshold=self._inner_threshold, density_cutoff=self.density_cutoff,
            negative_cutoff=self.negative_cutoff, population_cutoff=self.population_cutoff,
            maxiter=self._maxiter, polish=self._polish, local=local, **self._job_extra())

    def _report_warnings(self, info):
        if info.warnings & _lib.WARN_INNER_NOT_CONVERGED:
            self.logger.warning(self._inner_warning)
        if info.warnings & _lib.WARN_POPULATION:
            self.logger.warning("The sum of pro-atom parameters is not equal to reference population.")
        if info.warnings & _lib.WARN_NEGATIVE_PARS:
            self.logger.warning("WARNING: Not all pro-atom parameters are positive!")
        if info.warnings & _lib.WARN_NOISE_FLOOR:
            self.logger.warning("Mixed precision stopped at its noise floor (change %.3e); "
                                "pass polish=True to finish in FP64." % info.change)

    _inner_warning = "Warning: Inner iteration is not converge!"

    @just_once
    def do_partitioning(self):
        new = any(f"at_weights_{i}" not in self.cache for i in range(self.natom))
        new |= "niter" not in self.cache
        if not new:
            return
        job = self._make_job()
        try:
            t0 = time.time()
            try:
                host_histories = self._run_job(job)
            except _lib.HPError as err:
                raise RuntimeError(str(err)) from err
            t1 = time.time()
            info = job.info()
            self._job_info = info
            self._report_warnings(info)
            res = job.results(at_weights=self._store_at_weights)
            if host_histories:
                res.update(host_histories)
        finally:
            job.close()
        niter = int(info.niter)
        self.history_propars = list(res["history_propars"])
        self.history_entropies = list(res["history_entropies"])
        self.history_changes = list(res["history_changes"])
        if self._has_charge_history:
            self.history_charges = list(res["history_charges"])
        self.history_time_update_at_weights.append(0.0)
        self.history_time_update_propars.append(t1 - t0)
        self.logger.info("Iteration       Change      Entropy")
        for i in range(min(niter, len(self.history_changes))):
            self.logger.info("%9i   %10.5e   %10.5e" % (i + 1, self.history_changes[i],
                                                      self.history_entropies[i]))
        self.cache.dump("propars", res["propars"], tags="o")
        self.cache.dump("charges", res["charges"], tags="o")
        self.cache.dump("promoldens", res["promoldens"])
        if self._store_at_weights:
            for i in range(self.natom):
                # grid_type 1: each atom's at_weights live on its own atom grid
                self.cache.dump(f"at_weights_{i}", self.to_atomic_grid(i, res["at_weights"][i]))
        if not self.on_molgrid:
            for i, ag in enumerate(self.grid.atgrids):
                self.cache.dump(f"radial_points_{i}", np.asarray(ag.rgrid.points), tags="o")
                self.cache.dump(f"radial_weights_{i}", np.asarray(ag.rgrid.weights), tags="o")
        charges = res["charges"]
        self.cache.dump("history_propars", np.array(self.history_propars), tags="o")
        self.cache.dump("history_charges", np.array(self.history_charges), tags="o")
        self.cache.dump("history_entropies", np.array(self.history_entropies), tags="o")
        self.cache.dump("history_changes", np.array(self.history_changes), tags="o")
        self.cache.dump("populations", self.numbers - charges, tags="o")
        self.cache.dump("pseudo_populations", self.pseudo_numbers - charges, tags="o")
        self.cache.dump("time_update_at_weights", np.sum(self.history_time_update_at_weights), tags="o")
        self.cache.dump("time_update_propars", np.sum(self.history_time_update_propars), tags="o")
        self._finalize_extra(res)
        self.cache.dump("niter", niter, tags="o")
        if self._dumps_change:
            self.cache.dump("change", float(info.change), tags="o")
        if not self._store_at_weights:
            # keep the do_partitioning bookkeeping consistent without the arrays
            self._done_just_once.add("do_partitioning")

    @property
    def job_info(self):
        """Counters of the last GPU run (niter, inner iterations, evaluations, bytes)."""
        return self._job_info
