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
    """Base class of the partitioning schemes (``core/base.py:35-410``)."""

    name = None

    def __init__(self, coordinates, numbers, pseudo_numbers, grid, moldens, spindens, local, lmax,
                 logger, *args, **kwargs):
        super().__init__()
        natom, coordinates, numbers, pseudo_numbers = typecheck_geo(coordinates, numbers,
                                                                    pseudo_numbers)
        self._natom = natom
        self._coordinates = coordinates
        self._numbers = numbers
        self._pseudo_numbers = pseudo_numbers
        self._grid = grid
        self._moldens = moldens
        self._spindens = spindens
        self._local = local
        self._lmax = lmax
        self._cache = Cache()
        self.logger = logger
        if local:
            self._init_subgrids()
        self._init_log_scheme()

    def __getitem__(self, key):
        return self.cache.load(key)

    def variables_stored_in_cache(self):
        return list(self.cache.iterkeys())

    @property
    def natom(self):
        return self._natom

    @property
    def coordinates(self):
        return self._coordinates

    @property
    def numbers(self):
        return self._numbers

    @property
    def pseudo_numbers(self):
        return self._pseudo_numbers

    @property
    def nelec(self):
        return self.grid.integrate(self._moldens)

    @property
    def grid(self):
        return self.get_grid()

    @property
    def local(self):
        return self._local

    @property
    def lmax(self):
        return self._lmax

    @property
    def cache(self):
        return self._cache

    def __clear__(self):
        self.clear()

    def clear(self):
        JustOnceClass.clear(self)
        self.cache.clear()

    def get_grid(self, index=None):
        if index is None or not self.local:
            return self._grid
        return self._subgrids[index]

    def get_moldens(self, index=None, output=None):
        result = self._moldens if index is None or not self.local else self.to_atomic_grid(
            index, self._moldens)
        if output is not None:
            output[:] = result
        return result

    def get_spindens(self, index=None, output=None):
        result = self._spindens if index is None or not self.local else self.to_atomic_grid(
            index, self._spindens)
        if output is not None:
            output[:] = result
        return result

    def _init_subgrids(self):
        raise NotImplementedError

    def _init_log_scheme(self):
        pass

    def to_atomic_grid(self, index, data):
        raise NotImplementedError

    def get_wcor(self, index):
        return 1.0

    def compute_pseudo_population(self, index):
        grid = self.get_grid(index)
        dens = self.get_moldens(index)
        at_weights = self.cache.load(f"at_weights_{index}")
        return grid.integrate(at_weights, dens)

    @just_once
    def do_partitioning(self):
        self.update_at_weights()

    def update_at_weights(self, *args, **kwargs):
        raise NotImplementedError

    @just_once
    def do_populations(self):
        """Atomic populations from the at_weights (``core/base.py:277-300``)."""
        populations, new = self.cache.load("populations", alloc=self.natom, tags="o")
        if new:
            self.do_partitioning()
            pseudo_populations = self.cache.load("pseudo_populations", alloc=self.natom, tags="o")[0]
            for index in range(self.natom):
                grid = self.get_grid(index)
                dens = self.get_moldens(index)
                at_weights = self.cache.load(f"at_weights_{index}")
                wcor = self.get_wcor(index)
                if at_weights.shape == self._grid.weights.shape:
                    at_weights = self.to_atomic_grid(index, at_weights)
                pseudo_populations[index] = grid.integrate(at_weights, dens * wcor)
            populations[:] = pseudo_populations
            populations += self.numbers - self.pseudo_numbers

    @just_once
    def do_charges(self):
        """Atomic charges (``core/base.py:302-311``)."""
        charges, new = self._cache.load("charges", alloc=self.natom, tags="o")
        if new:
            self.do_populations()
            populations = self._cache.load("populations")
            charges[:] = self.numbers - populations

    @just_once
    def do_spin_charges(self):
        """Atomic spin charges (``core/base.py:313-327``)."""
        if self._spindens is not None:
            spin_charges, _ = self._cache.load("spin_charges", alloc=self.natom, tags="o")
            self.do_partitioning()
            for index in range(self.natom):
                grid = self.get_grid(index)
                spindens = self.get_spindens(index)
                at_weights = self.cache.load(f"at_weights_{index}")
                spin_charges[index] = grid.integrate(at_weights, spindens * self.get_wcor(index))

    def do_all(self):
        """Run every implemented ``do_*`` method; return the output keys."""
        for name in ("do_partitioning", "do_populations", "do_charges", "do_spin_charges"):
            getattr(self, name)()
        return list(self.cache.iterkeys(tags="o"))


class WPart(Part):
    """Grid-based partitioning (``core/base.py:413-499``)."""

    def __init__(self, coordinates, numbers, pseudo_numbers, grid, moldens, spindens=None, lmax=3,
                 logger=None, grid_type=1, density_cutoff=DENSITY_CUTOFF,
                 negative_cutoff=NEGATIVE_CUTOFF, population_cutoff=POPULATION_CUTOFF, **kwargs):
        self._grid_type = grid_type
        self._on_molgrid = None
        self._only_use_molgrid = None
        self.setup_grids()
        local = not self._only_use_molgrid
        if local and getattr(grid, "atgrids", None) is None:
            raise ValueError("Atomic grids are discarded from molecular grid object, "
                             "but are needed for local integrations.")
        if logger is None:
            logger = logging.getLogger(self.__class__.__name__)
            _setup_logger(logger)
        self.history_propars = []
        self.history_charges = []
        self.history_entropies = []
        self.history_changes = []
        self.history_time_update_at_weights = []
        self.history_time_update_propars = []
        self._radial_distances = []
        self._density_cutoff = density_cutoff
        self._population_cutoff = population_cutoff
        self._negative_cutoff = negative_cutoff
        super().__init__(coordinates, numbers, pseudo_numbers, grid, moldens, spindens, local, lmax,
                         logger)

    def setup_grids(self):
        assert self.grid_type in [1, 2, 3]
        self._on_molgrid = self.grid_type in [2, 3]
        self._only_use_molgrid = self.grid_type in [3]

    @property
    def grid_type(self):
        return self._grid_type

    @property
    def only_use_molgrid(self):
        return self._only_use_molgrid

    @property
    def on_molgrid(self):
        return self._on_molgrid

    @property
    def radial_distances(self):
        self.calc_radial_distances()
        return self._radial_distances

    @property
    def density_cutoff(self):
        return self._density_cutoff

    @property
    def population_cutoff(self):
        return self._population_cutoff

    @property
    def negative_cutoff(self):
        return self._negative_cutoff

    def _init_subgrids(self):
        self._subgrids = self._grid.atgrids

    def to_atomic_grid(self, index, data):
        if index is None or not self.local:
            return data
        begin, end = self.grid.indices[index], self.grid.indices[index + 1]
        return data[begin:end]

    @just_once
    def calc_radial_distances(self):
        for iatom in range(self.natom):
            self._radial_distances.append(
                np.linalg.norm(self.grid.points - self.coordinates[iatom], axis=1))


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
                job.run()
            except _lib.HPError as err:
                raise RuntimeError(str(err)) from err
            t1 = time.time()
            info = job.info()
            self._job_info = info
            self._report_warnings(info)
            res = job.results(at_weights=self._store_at_weights)
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
