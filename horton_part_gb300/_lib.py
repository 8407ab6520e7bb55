"""ctypes binding of ``libhpgpu.so`` (the C ABI declared in ``include/hpgpu.h``).

There is no CPU fallback: if the library is missing or no sm_103 device is
available, the calls raise.
"""

from __future__ import annotations

import ctypes
import os
import threading
import weakref

import numpy as np

__all__ = ["lib", "Context", "Job", "default_context", "HPError", "SCHEMES", "SOLVERS"]

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhpgpu.so")

HP_OK, HP_ERR_INVALID, HP_ERR_NO_MEMORY, HP_ERR_NOT_CONVERGED = 0, 1, 2, 3
HP_ERR_NUMERIC, HP_ERR_TIMEOUT, HP_ERR_CUDA, HP_ERR_UNSUPPORTED, HP_ERR_STATE = 4, 5, 6, 7, 8

SCHEMES = {"mbis": 0, "gisa": 1, "lisa": 2, "glisa": 3, "nlis": 4}
SOLVERS = {"default": 0, "sc": 1, "newton": 2, "m-newton": 3, "quadprog": 4, "qp": 4,
           "pnewton": 5, "quasi-newton": 6}
PRECISIONS = {"fp64": 0, "mixed": 1, "ff": 2}

WARN_INNER_NOT_CONVERGED = 1
WARN_POPULATION = 2
WARN_NEGATIVE_PARS = 4
WARN_NOISE_FLOOR = 8

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)


class JobDesc(ctypes.Structure):
    _fields_ = [
        ("scheme", ctypes.c_int32), ("solver", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("grid_type", ctypes.c_int32), ("natom", ctypes.c_int64), ("npoint", ctypes.c_int64),
        ("coordinates", _dp), ("pseudo_numbers", _dp), ("points", _dp), ("weights", _dp),
        ("density", _dp), ("shell_offsets", _ip), ("shell_orders", _dp),
        ("shell_exponents", _dp), ("initial_propars", _dp), ("threshold", ctypes.c_double),
        ("inner_threshold", ctypes.c_double), ("density_cutoff", ctypes.c_double),
        ("negative_cutoff", ctypes.c_double), ("population_cutoff", ctypes.c_double),
        ("tau", ctypes.c_double), ("maxiter", ctypes.c_int32), ("inner_maxiter", ctypes.c_int32),
        ("linspace_size", ctypes.c_int32), ("polish", ctypes.c_int32),
        ("nrad", ctypes.c_int32), ("radial_offsets", _ip),
        ("shell_point_offsets", ctypes.POINTER(ctypes.c_int64)),
        ("point_sphere_weights", _dp), ("radial_points", _dp), ("radial_weights", _dp),
    ]


class JobInfo(ctypes.Structure):
    _fields_ = [
        ("natom", ctypes.c_int64), ("npoint", ctypes.c_int64), ("nparam", ctypes.c_int64),
        ("niter", ctypes.c_int64), ("inner_iterations", ctypes.c_int64),
        ("change", ctypes.c_double), ("done", ctypes.c_int32), ("status", ctypes.c_int32),
        ("warnings", ctypes.c_uint32), ("converged", ctypes.c_int32),
        ("device_bytes", ctypes.c_int64), ("point_atom_evals", ctypes.c_double),
        ("polish_iterations", ctypes.c_int32), ("f64_factors", ctypes.c_int32),
        ("g_active_values", ctypes.c_int64), ("point_atom_evals_skipped", ctypes.c_double),
    ]


class JobResults(ctypes.Structure):
    _fields_ = [(name, _dp) for name in (
        "charges", "propars", "history_propars", "history_charges", "history_entropies",
        "history_changes", "promoldens", "at_weights")]


class DensityDesc(ctypes.Structure):
    _fields_ = [
        ("nshell", ctypes.c_int32), ("centers", _dp), ("shell_info", _ip), ("nprim", ctypes.c_int32),
        ("exponents", _dp), ("coeffs", _dp), ("nbasis", ctypes.c_int32), ("nmat", ctypes.c_int32),
        ("mats", _dp), ("pure2", _dp), ("pure3", _dp),
    ]


class HPError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


EXPORTED = ("hp_abi_version", "hp_last_error", "hp_ctx_create", "hp_ctx_destroy",
            "hp_ctx_synchronize", "hp_ctx_memory", "hp_job_create", "hp_job_destroy", "hp_step",
            "hp_step_n",
            "hp_job_run", "hp_job_info_get", "hp_job_results_get", "hp_job_reset",
            "hp_ctx_profile", "hp_ctx_profile_get", "hp_mbis_inner_noalloc", "hp_glisa_evaluate",
            "hp_glisa_change", "hp_glisa_line_search", "hp_glisa_finish",
            "hp_density_plan_create", "hp_density_plan_eval", "hp_density_plan_stats",
            "hp_density_plan_destroy")

KERNEL_FAMILIES = {"promol": 0, "inner": 1, "change": 2, "glisa_pro": 3, "glisa_grad": 4,
                   "glisa_hess": 5, "glisa_solve": 6, "other": 7, "glisa_trials": 8}
KERNEL_FAMILY_COUNT = 9

_lib = None
_lock = threading.Lock()


def lib():
    """Load ``libhpgpu.so`` (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m horton_part_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        L.hp_abi_version.restype = ctypes.c_int32
        L.hp_last_error.restype = ctypes.c_char_p
        L.hp_ctx_create.argtypes = [ctypes.c_int32, ctypes.c_size_t, ctypes.c_void_p,
                                    ctypes.POINTER(ctypes.c_void_p)]
        L.hp_ctx_destroy.argtypes = [ctypes.c_void_p]
        L.hp_ctx_synchronize.argtypes = [ctypes.c_void_p]
        L.hp_ctx_memory.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t),
                                    ctypes.POINTER(ctypes.c_size_t)]
        L.hp_job_create.argtypes = [ctypes.c_void_p, ctypes.POINTER(JobDesc),
                                    ctypes.POINTER(ctypes.c_void_p)]
        L.hp_job_destroy.argtypes = [ctypes.c_void_p]
        L.hp_step.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32,
                              ctypes.POINTER(ctypes.c_int32)]
        L.hp_step_n.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32,
                                ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
        L.hp_job_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.hp_job_info_get.argtypes = [ctypes.c_void_p, ctypes.POINTER(JobInfo)]
        L.hp_job_results_get.argtypes = [ctypes.c_void_p, ctypes.POINTER(JobResults)]
        L.hp_job_reset.argtypes = [ctypes.c_void_p]
        L.hp_mbis_inner_noalloc.argtypes = [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
            ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
            ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p]
        L.hp_ctx_profile.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        L.hp_glisa_evaluate.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int32, _dp, _dp, _dp, _dp]
        L.hp_glisa_change.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_int32, _dp]
        L.hp_glisa_line_search.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp]
        L.hp_glisa_finish.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int32]
        L.hp_density_plan_create.argtypes = [ctypes.c_void_p, ctypes.POINTER(DensityDesc),
                                             ctypes.POINTER(ctypes.c_void_p)]
        L.hp_density_plan_eval.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int32]
        L.hp_density_plan_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
        L.hp_density_plan_destroy.argtypes = [ctypes.c_void_p]
        L.hp_ctx_profile_get.argtypes = [ctypes.c_void_p, ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_int64)]
        for name in EXPORTED:
            if name not in ("hp_last_error",):
                getattr(L, name).restype = ctypes.c_int32
        L.hp_last_error.restype = ctypes.c_char_p
        _lib = L
        return L


def _check(rc):
    if rc != HP_OK:
        msg = lib().hp_last_error().decode(errors="replace")
        if rc == HP_ERR_INVALID:
            raise ValueError(msg)
        if rc == HP_ERR_NO_MEMORY:
            raise MemoryError(msg)
        if rc == HP_ERR_UNSUPPORTED:
            raise NotImplementedError(msg)
        raise HPError(rc, msg)


def _ptr(arr, ctype=ctypes.c_double):
    return arr.ctypes.data_as(ctypes.POINTER(ctype))


class Context:
    """A device, a stream and an HBM budget (``hp_ctx``)."""

    def __init__(self, device=0, hbm_budget=0, stream=None):
        handle = ctypes.c_void_p()
        _check(lib().hp_ctx_create(int(device), int(hbm_budget),
                                   ctypes.c_void_p(stream) if stream else None,
                                   ctypes.byref(handle)))
        self._h = handle
        self.device = device
        self._jobs = weakref.WeakSet()

    @property
    def handle(self):
        return self._h

    def synchronize(self):
        _check(lib().hp_ctx_synchronize(self._h))

    def memory(self):
        used, budget = ctypes.c_size_t(), ctypes.c_size_t()
        _check(lib().hp_ctx_memory(self._h, ctypes.byref(used), ctypes.byref(budget)))
        return used.value, budget.value

    def profile(self, enable=True):
        """Start (and clear) or stop CUDA-event timing of the library's kernels."""
        _check(lib().hp_ctx_profile(self._h, 1 if enable else 0))

    def profile_get(self, family):
        """(milliseconds, launches) accumulated for a kernel family."""
        ms, n = ctypes.c_double(), ctypes.c_int64()
        _check(lib().hp_ctx_profile_get(self._h, KERNEL_FAMILIES[family], ctypes.byref(ms),
                                        ctypes.byref(n)))
        return ms.value, n.value

    def launch_count(self):
        """Kernel launches issued by the library since profiling was enabled."""
        ms, n = ctypes.c_double(), ctypes.c_int64()
        _check(lib().hp_ctx_profile_get(self._h, KERNEL_FAMILY_COUNT, ctypes.byref(ms),
                                        ctypes.byref(n)))
        return n.value

    def step(self, jobs, iterations=1):
        """Advance every live job by one outer iteration (``iterations`` > 1:
        up to that many in one host round trip, see ``hp_step_n``); returns
        the live count."""
        arr = (ctypes.c_void_p * len(jobs))(*[j.handle for j in jobs])
        live = ctypes.c_int32()
        if iterations == 1:
            _check(lib().hp_step(self._h, arr, len(jobs), ctypes.byref(live)))
        else:
            _check(lib().hp_step_n(self._h, arr, len(jobs), int(iterations), ctypes.byref(live)))
        return live.value

    def close(self):
        if getattr(self, "_h", None):
            for job in list(self._jobs):
                job._h = None  # destroyed together with the context
            lib().hp_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = {}


def default_context(device=0):
    if device not in _default:
        _default[device] = Context(device)
    return _default[device]


class Job:
    """One partitioning job on the device (``hp_job``)."""

    def __init__(self, ctx, scheme, coordinates, pseudo_numbers, points, weights, density,
                 shell_offsets, initial_propars, shell_orders=None, shell_exponents=None,
                 solver="default", precision="fp64", grid_type=3, threshold=1e-6,
                 inner_threshold=1e-8, density_cutoff=1e-15, negative_cutoff=-1e-12,
                 population_cutoff=1e-4, maxiter=500, inner_maxiter=0, linspace_size=0, tau=1.0,
                 polish=False, local=None):
        """``local`` (grid_type 1): dict with ``radial_offsets`` (natom + 1),
        ``shell_point_offsets`` (nrad + 1), ``point_sphere_weights`` (npoint),
        ``radial_points`` and ``radial_weights`` (nrad), as in hpgpu.h."""
        self.ctx = ctx
        keep = []

        def f64(a, shape=None):
            a = np.ascontiguousarray(a, dtype=np.float64)
            if shape is not None and a.shape != shape:
                raise ValueError(f"expected shape {shape}, got {a.shape}")
            keep.append(a)
            return a

        natom = len(pseudo_numbers)
        npoint = len(weights)
        d = JobDesc()
        d.scheme = SCHEMES[scheme]
        d.solver = SOLVERS[solver]
        d.precision = PRECISIONS[precision]
        d.grid_type = int(grid_type)
        d.natom, d.npoint = natom, npoint
        d.coordinates = _ptr(f64(coordinates, (natom, 3)))
        d.pseudo_numbers = _ptr(f64(pseudo_numbers, (natom,)))
        d.points = _ptr(f64(points, (npoint, 3)))
        d.weights = _ptr(f64(weights, (npoint,)))
        d.density = _ptr(f64(density, (npoint,)))
        off = np.ascontiguousarray(shell_offsets, dtype=np.int32)
        keep.append(off)
        d.shell_offsets = _ptr(off, ctypes.c_int32)
        if shell_orders is not None:
            d.shell_orders = _ptr(f64(shell_orders))
            d.shell_exponents = _ptr(f64(shell_exponents))
        init = f64(initial_propars)
        d.initial_propars = _ptr(init)
        d.threshold, d.inner_threshold = threshold, inner_threshold
        d.density_cutoff, d.negative_cutoff = density_cutoff, negative_cutoff
        d.population_cutoff, d.tau = population_cutoff, tau
        d.maxiter, d.inner_maxiter, d.linspace_size = int(maxiter), int(inner_maxiter), int(linspace_size)
        d.polish = 1 if polish else 0
        if local is not None:
            roff = np.ascontiguousarray(local["radial_offsets"], dtype=np.int32)
            spo = np.ascontiguousarray(local["shell_point_offsets"], dtype=np.int64)
            keep.extend([roff, spo])
            d.nrad = int(roff[-1])
            d.radial_offsets = _ptr(roff, ctypes.c_int32)
            d.shell_point_offsets = _ptr(spo, ctypes.c_int64)
            d.point_sphere_weights = _ptr(f64(local["point_sphere_weights"], (npoint,)))
            d.radial_points = _ptr(f64(local["radial_points"], (d.nrad,)))
            d.radial_weights = _ptr(f64(local["radial_weights"], (d.nrad,)))
        handle = ctypes.c_void_p()
        _check(lib().hp_job_create(ctx.handle, ctypes.byref(d), ctypes.byref(handle)))
        self._h = handle
        ctx._jobs.add(self)
        self.natom, self.npoint, self.nparam = natom, npoint, len(init)
        self.scheme = scheme

    @property
    def handle(self):
        return self._h

    def run(self):
        _check(lib().hp_job_run(self.ctx.handle, self._h))

    def reset(self):
        """Back to the initial parameters; the inputs stay on the device."""
        _check(lib().hp_job_reset(self._h))

    def info(self):
        inf = JobInfo()
        _check(lib().hp_job_info_get(self._h, ctypes.byref(inf)))
        return inf

    def results(self, at_weights=False, promoldens=True, histories=True):
        inf = self.info()
        nit = int(min(inf.niter, 1 << 30))
        out = {
            "charges": np.zeros(self.natom),
            "propars": np.zeros(self.nparam),
        }
        r = JobResults()
        r.charges = _ptr(out["charges"])
        r.propars = _ptr(out["propars"])
        if histories:
            out["history_propars"] = np.zeros((nit, self.nparam))
            out["history_charges"] = np.zeros((nit, self.natom))
            out["history_entropies"] = np.zeros(nit)
            out["history_changes"] = np.zeros(nit)
            for k in ("history_propars", "history_charges", "history_entropies", "history_changes"):
                setattr(r, k, _ptr(out[k]))
        if promoldens:
            out["promoldens"] = np.zeros(self.npoint)
            r.promoldens = _ptr(out["promoldens"])
        if at_weights:
            out["at_weights"] = np.zeros((self.natom, self.npoint))
            r.at_weights = _ptr(out["at_weights"])
        _check(lib().hp_job_results_get(self._h, ctypes.byref(r)))
        return out

    # -- evaluation service of the host-driven gLISA solvers ---------------
    def _vec(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.shape != (self.nparam,):
            raise ValueError(f"expected {self.nparam} parameters, got shape {x.shape}")
        return x

    def evaluate(self, x, nderiv=1):
        """(f, grad or None, hess or None, int rho0) at populations ``x``."""
        x = self._vec(x)
        f, pop = ctypes.c_double(), ctypes.c_double()
        grad = np.zeros(self.nparam) if nderiv >= 1 else None
        hess = np.zeros((self.nparam, self.nparam)) if nderiv == 2 else None
        _check(lib().hp_glisa_evaluate(self._h, _ptr(x), int(nderiv), ctypes.byref(f),
                                       _ptr(grad) if grad is not None else None,
                                       _ptr(hess) if hess is not None else None,
                                       ctypes.byref(pop)))
        return f.value, grad, hess, pop.value

    def change(self, x, y, kind=0):
        """kind 0: promolecule change; 1: the outer change (compute_change)."""
        out = ctypes.c_double()
        _check(lib().hp_glisa_change(self._h, _ptr(self._vec(x)), _ptr(self._vec(y)), int(kind),
                                     ctypes.byref(out)))
        return out.value

    def line_search(self, x, delta, keep):
        """(step, new populations) of the valid-promolecule line search; step < 0: none."""
        step = ctypes.c_double()
        out = np.zeros(self.nparam)
        _check(lib().hp_glisa_line_search(self._h, _ptr(self._vec(x)), _ptr(self._vec(delta)),
                                          _ptr(self._vec(keep)), ctypes.byref(step), _ptr(out)))
        return step.value, out

    def finish(self, x, niter):
        _check(lib().hp_glisa_finish(self._h, _ptr(self._vec(x)), int(niter)))

    def close(self):
        if getattr(self, "_h", None) and getattr(self.ctx, "_h", None):
            lib().hp_job_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
