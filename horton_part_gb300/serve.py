"""Continuous-batching server for partitioning jobs on one GPU.

Requests (one molecule and scheme each) arrive over time. The server keeps
one context (device, stream, HBM budget) and runs a loop:

1. admit waiting requests in arrival order while the job fits the HBM budget
   (``hp_job_create`` refuses a job that would exceed it; the request then
   waits for memory to free up);
2. advance every live job with ``hp_step_n`` (shared kernel launches for all
   live jobs of a scheme, one host wait per step): gLISA jobs by two solver
   iterations queued back to back, the other schemes by one outer iteration;
3. retire finished jobs: copy their results out, free their device memory,
   record their latency (completion minus arrival).

Inputs, densities and parameters of admitted jobs stay resident on the device
until the job retires. Because every reduction runs in a fixed order inside
one job's own tiles, a job's result is bit-identical whether it runs alone or
in any mix of other jobs.

There is no reference counterpart: horton-part runs one molecule at a time
(``scripts/program.py:120-131`` loops over input files serially).
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .basis import ExpBasisFuncHelper
from .mbis import get_initial_mbis_propars, get_nshell

__all__ = ["Request", "PartitionServer", "request_from_molecule"]


@dataclass
class Request:
    """One partitioning request."""

    rid: int
    scheme: str
    arrays: dict
    options: dict
    arrival: float = 0.0
    admitted: float | None = None
    finished: float | None = None
    result: dict | None = None
    error: str | None = None
    niter: int = 0
    evals: float = 0.0
    job: object = field(default=None, repr=False)

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


def request_from_molecule(rid, scheme, mol, precision="fp64", threshold=1e-8, solver="default",
                          basis="gauss", maxiter=None, polish=True):
    """Build a request for ``mol`` (a :class:`~horton_part_gb300.synthetic.Molecule`).

    ``polish`` (mixed precision): finish near the threshold in float-float
    (MBIS) or FP64 (basis schemes)."""
    arrays = dict(coordinates=mol.coordinates, pseudo_numbers=mol.pseudo_numbers,
                  points=mol.grid.points, weights=mol.grid.weights, density=mol.density)
    opts = dict(precision=precision, threshold=threshold, solver=solver, grid_type=3,
                polish=bool(polish))
    if scheme == "mbis":
        nsh = [int(get_nshell(z)) for z in mol.numbers]
        arrays["shell_offsets"] = np.concatenate([[0], np.cumsum(nsh)]).astype(np.int32)
        arrays["initial_propars"] = np.concatenate([get_initial_mbis_propars(z) for z in mol.numbers])
        opts.update(inner_threshold=threshold, inner_maxiter=2000, maxiter=maxiter or 500)
    else:
        h = ExpBasisFuncHelper.from_function_type(basis) if isinstance(basis, str) else basis
        nsh = [h.get_nshell(z) for z in mol.numbers]
        arrays["shell_offsets"] = np.concatenate([[0], np.cumsum(nsh)]).astype(np.int32)
        parts = []
        for z, zp in zip(mol.numbers, mol.pseudo_numbers):
            ini = np.array(h.get_initial(z), dtype=float)
            ini[ini < 1e-4] = 1e-4
            parts.append(ini / ini.sum() * zp)
        arrays["initial_propars"] = np.concatenate(parts)
        arrays["shell_orders"] = np.concatenate([h.get_order(z) for z in mol.numbers])
        arrays["shell_exponents"] = np.concatenate([h.get_exponent(z) for z in mol.numbers])
        opts.update(inner_threshold=threshold, maxiter=maxiter or (100 if scheme == "glisa" else 500))
        if scheme == "lisa":
            opts["inner_maxiter"] = 100000
    return Request(rid, scheme, arrays, opts)


class PartitionServer:
    """Admit, step and retire partitioning jobs on one GPU."""

    def __init__(self, context=None, device=0, hbm_budget=150 * 10**9, max_live=4096):
        self.ctx = context or _lib.Context(device, hbm_budget=int(hbm_budget))
        self.max_live = max_live
        self.waiting: list[Request] = []
        self.live: list[Request] = []
        self.done: list[Request] = []
        self.steps = 0

    def submit(self, req: Request, now=None):
        req.arrival = time.perf_counter() if now is None else now
        self.waiting.append(req)

    def _admit(self):
        still = []
        for i, req in enumerate(self.waiting):
            if len(self.live) >= self.max_live:
                still.extend(self.waiting[i:])
                break
            try:
                req.job = _lib.Job(self.ctx, req.scheme, **req.arrays, **req.options)
            except MemoryError:
                # does not fit the budget now; keep the arrival order
                still.extend(self.waiting[i:])
                break
            except Exception as exc:  # invalid request: finish with an error
                req.error = str(exc)
                req.finished = time.perf_counter()
                self.done.append(req)
                continue
            req.admitted = time.perf_counter()
            self.live.append(req)
        self.waiting = still

    def _retire(self):
        keep = []
        for req in self.live:
            info = req.job.info()
            if info.done:
                req.niter = int(info.niter)
                req.evals = float(info.point_atom_evals)
                if info.status == 0:
                    req.result = req.job.results(promoldens=False, histories=False)
                else:
                    req.error = f"status {info.status}"
                req.job.close()
                req.job = None
                req.finished = time.perf_counter()
                self.done.append(req)
            else:
                keep.append(req)
        self.live = keep

    def step(self):
        """One server step: admit, advance all live jobs, retire."""
        self._admit()
        if self.live:
            try:
                # gLISA jobs take two solver iterations per step (one host
                # round trip); the other schemes one
                self.ctx.step([r.job for r in self.live], 2)
            except _lib.HPError:
                pass  # per-job failures are recorded in the job status
            self.steps += 1
        self._retire()
        return len(self.live) + len(self.waiting)

    def run_stream(self, requests, arrival_times, time_limit=None):
        """Serve ``requests`` arriving at ``arrival_times`` (seconds from now)."""
        t0 = time.perf_counter()
        order = np.argsort(arrival_times)
        pending = [(float(arrival_times[i]), requests[i]) for i in order]
        k = 0
        while k < len(pending) or self.live or self.waiting:
            now = time.perf_counter() - t0
            while k < len(pending) and pending[k][0] <= now:
                self.submit(pending[k][1], now=t0 + pending[k][0])
                k += 1
            if not self.live and not self.waiting and k < len(pending):
                time.sleep(max(0.0, min(0.01, pending[k][0] - now)))
                continue
            self.step()
            if time_limit is not None and time.perf_counter() - t0 > time_limit:
                break
        return time.perf_counter() - t0

    def stats(self, wall):
        lat = np.array([r.latency for r in self.done if r.error is None and r.latency is not None])
        ok = len(lat)
        return {
            "jobs_done": ok,
            "jobs_failed": sum(1 for r in self.done if r.error is not None),
            "jobs_per_s": ok / wall if wall > 0 else 0.0,
            "p50_latency_s": float(np.percentile(lat, 50)) if ok else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if ok else None,
            "point_atom_evals_per_s": sum(r.evals for r in self.done) / wall if wall > 0 else 0.0,
            "server_steps": self.steps,
        }

    def close(self):
        for req in self.live:
            if req.job is not None:
                req.job.close()
        self.ctx.close()
