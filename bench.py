"""Benchmark of the partitioning loop on one GB300 (or N independent replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload glisa-c6h10n2o2|mbis-h2o] [--precision fp64|mixed]

Default workload: gLISA (exact Newton) on a 20-atom C6H10N2O2 chain,
100 radial x Lebedev-302 points per atom (604,000 points), 6 s-Gaussians per
H and 9 per C/N/O with exponents geometric in [0.05, 300] (150 shells),
threshold 1e-8. One step = one complete partitioning job (every solver
iteration until convergence) on inputs already resident in HBM; the basis
matrix G (150 x 604,000 FP64 = 725 MB) is larger than L2, so no L2 flush is
added between steps.

Metric: pro-atom evaluations (point x atom) per second, counted in the
reference's convention (each solver iteration evaluates every pro-atom on
every grid point three times: promolecule and the two sides of the change).

Output: one JSON line (rank 0). Under torchrun every rank runs its own
replica of the job (no collective on the data path); value = sum over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MBIS/gLISA point·atom evals/s"
UNIT = "point·atom evals/s"


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

def workload(name):
    from horton_part_gb300 import synthetic

    if name in ("glisa-c6h10n2o2", "gisa-c6h10n2o2"):
        mol = synthetic.chain_molecule({6: 6, 1: 10, 7: 2, 8: 2}, 100, 302, seed=2024)
        helper = synthetic.geometric_gaussian_basis({1: 6, 6: 9, 7: 9, 8: 9}, 0.05, 300.0)
        if name.startswith("gisa"):
            return dict(name=name, scheme="gisa", solver="quadprog", mol=mol, helper=helper,
                        threshold=1e-8, maxiter=500)
        return dict(name=name, scheme="glisa", solver="newton", mol=mol, helper=helper,
                    threshold=1e-8, maxiter=100)
    if name == "mbis-h2o":
        mol = synthetic.water(75, 110)
        return dict(name=name, scheme="mbis", solver="default", mol=mol, helper=None,
                    threshold=1e-8, maxiter=500)
    raise ValueError(name)


def job_arrays(w):
    mol = w["mol"]
    if w["scheme"] == "mbis":
        from horton_part_gb300.mbis import get_initial_mbis_propars, get_nshell

        nsh = [int(get_nshell(z)) for z in mol.numbers]
        off = np.concatenate([[0], np.cumsum(nsh)]).astype(np.int32)
        init = np.concatenate([get_initial_mbis_propars(z) for z in mol.numbers])
        return off, init, None, None
    h = w["helper"]
    off = np.concatenate([[0], np.cumsum([h.get_nshell(z) for z in mol.numbers])]).astype(np.int32)
    parts = []
    for z, zp in zip(mol.numbers, mol.pseudo_numbers):
        ini = np.array(h.get_initial(z), dtype=float)
        ini[ini < 1e-4] = 1e-4
        parts.append(ini / ini.sum() * zp)
    init = np.concatenate(parts)
    orders = np.concatenate([h.get_order(z) for z in mol.numbers])
    exps = np.concatenate([h.get_exponent(z) for z in mol.numbers])
    return off, init, orders, exps


def make_job(ctx, w, precision, pinned=None):
    from horton_part_gb300 import _lib

    mol = w["mol"]
    off, init, orders, exps = job_arrays(w)
    pts, wts, rho = (mol.grid.points, mol.grid.weights, mol.density) if pinned is None else pinned
    extra = {"inner_maxiter": 2000} if w["scheme"] == "mbis" else {}
    return _lib.Job(ctx, w["scheme"], mol.coordinates, mol.pseudo_numbers, pts, wts, rho, off,
                    init, shell_orders=orders, shell_exponents=exps, solver=w["solver"],
                    precision=precision, grid_type=3, threshold=w["threshold"],
                    inner_threshold=w["threshold"], maxiter=w["maxiter"], **extra)


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU (oracle) timing
# ---------------------------------------------------------------------------

def cpu_sample(w, iterations):
    """Time the FP64 NumPy oracle on the same input; returns (evals/s, sample text, threads)."""
    from oracle import hp_oracle as O

    mol = w["mol"]
    args = (mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid.points, mol.grid.weights,
            mol.density)
    threads = os.cpu_count() or 1
    if w["scheme"] == "glisa":
        h = w["helper"]
        orders = [h.get_order(z) for z in mol.numbers]
        exps = [h.get_exponent(z) for z in mol.numbers]
        inits = [h.get_initial(z) for z in mol.numbers]
        t0 = time.perf_counter()
        try:
            res = O.glisa(*args, orders, exps, inits, threshold=w["threshold"], solver="newton",
                          maxiter=iterations)
            nit = res["niter"]
        except O.OracleError:
            nit = iterations
        dt = time.perf_counter() - t0
        evals = 3.0 * mol.natom * mol.npoint * nit + mol.natom * mol.npoint
        return evals / dt, f"oracle gLISA newton, {nit} solver iterations incl. basis set-up, {dt:.1f} s", threads
    if w["scheme"] == "gisa":
        h = w["helper"]
        t0 = time.perf_counter()
        res = O.basis_scheme("gisa", *args, [h.get_order(z) for z in mol.numbers],
                             [h.get_exponent(z) for z in mol.numbers],
                             [h.get_initial(z) for z in mol.numbers], threshold=w["threshold"],
                             maxiter=iterations)
        dt = time.perf_counter() - t0
        evals = 4.0 * mol.natom * mol.npoint * res["niter"]
        return (evals / dt, f"oracle GISA, {res['niter']} outer iterations incl. basis set-up, "
                f"{dt:.1f} s", threads)
    t0 = time.perf_counter()
    res = O.mbis(*args, threshold=w["threshold"], maxiter=iterations, inner_threshold=w["threshold"])
    dt = time.perf_counter() - t0
    inner = sum(sum(x) for x in res["inner_iterations"])
    evals = mol.npoint * (3.0 * mol.natom * res["niter"] + inner)
    return evals / dt, f"oracle MBIS, {res['niter']} outer iterations, {dt:.1f} s", 1


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def dist_env():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), int(
        os.environ.get("LOCAL_RANK", "0"))


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    w = workload(args.workload)
    rates = []
    for _ in range(args.warmup):
        cpu_sample(w, 1)
    t0 = time.perf_counter()
    samples = []
    for _ in range(args.steps):
        r, sample, threads = cpu_sample(w, 1 if w["scheme"] == "glisa" else 3)
        rates.append(r)
        samples.append(sample)
    dt = time.perf_counter() - t0
    value = statistics.median(rates)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_of(w, args, "fp64"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": samples[0]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_of(w, args, precision):
    mol = w["mol"]
    return {"workload": w["name"], "natom": int(mol.natom), "npoint": int(mol.npoint),
            "nshell": int(sum(w["helper"].get_nshell(z) for z in mol.numbers)) if w["helper"] else None,
            "solver": w["solver"], "threshold": w["threshold"], "precision": precision,
            "l2": "inputs larger than L2 (basis matrix 725 MB)" if w["scheme"] == "glisa"
            else "L2-resident small case", "parallelism": f"replicas{args.gpus}"}


def run_ours(args):
    import torch

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from horton_part_gb300 import _lib
    from horton_part_gb300.build import build

    build()
    w = workload(args.workload)
    mol = w["mol"]
    stream = torch.cuda.current_stream()
    ctx = _lib.Context(torch.cuda.current_device(), stream=stream.cuda_stream)
    job = make_job(ctx, w, args.precision)
    for _ in range(args.warmup):
        job.reset()
        job.run()
    info = job.info()
    evals_per_job = info.point_atom_evals
    niter = info.niter

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    ctx.profile(True)
    barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            job.reset()
            job.run()
        end.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = start.elapsed_time(end)
    hess_ms, hess_n = ctx.profile_get("glisa_hess")
    fam_ms = {f: ctx.profile_get(f) for f in _lib.KERNEL_FAMILIES}
    launches = ctx.launch_count()
    ctx.profile(False)
    ms_max = ms
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_max = float(t.item())
    value = evals_per_job * args.steps * world / (ms_max / 1000.0)

    # end to end through the C ABI: host inputs (pinned), job create (H2D),
    # run, charges back (D2H), destroy
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    pinned = (pin(mol.grid.points), pin(mol.grid.weights), pin(mol.density))
    e2e_steps = max(1, min(args.steps, 3))
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        j2 = make_job(ctx, w, args.precision, pinned=pinned)
        j2.run()
        q = j2.results(promoldens=False, histories=False)["charges"]
        j2.close()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_value = evals_per_job * world / e2e_s
    h2d = int(mol.npoint * 5 * 8 + mol.natom * 4 * 8)
    d2h = int(q.nbytes + job.nparam * 8)

    fams = {k: {"ms": round(v[0], 3), "launches": v[1]} for k, v in fam_ms.items() if v[1]}
    roofline = None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    if w["scheme"] != "glisa":
        # dominant kernel family and its algorithmic bytes per launch
        A, N = float(mol.natom), float(mol.npoint)
        model = {  # bytes that the pass must move at least once
            "promol": 8 * N * (3 + 2 + 1) + 8 * A * N * 3,   # xyz, w, rho, promol; rho_a w/r/w
            "inner": 8 * N * (3 + 1) + 8 * A * N,            # xyz, w; rho_a read
            "change": 8 * N * (3 + 1),                       # xyz, w
        }
        fam = max(model, key=lambda f: fam_ms[f][0])
        f_ms, f_n = fam_ms[fam]
        if f_n:
            per_launch_s = f_ms / f_n / 1000.0
            achieved = model[fam] / per_launch_s / 1e9
            roofline = {"kernel": fam, "bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                        "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                        "peak_source": "measured" if peaks else "fallback",
                        "ms_per_launch": per_launch_s * 1000.0}
    if w["scheme"] == "glisa" and hess_n:
        nshell = config_of(w, args, args.precision)["nshell"]
        per_launch_s = hess_ms / hess_n / 1000.0
        alg_bytes = (nshell + 1) * mol.npoint * 8.0  # G and w rho/rho0^2 once
        achieved = alg_bytes / per_launch_s / 1e9
        roofline = {"kernel": "k_glisa_hess", "bound": "hbm", "achieved": achieved,
                    "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                    "traffic": None, "peak_source": "measured" if peaks else "fallback",
                    "ms_per_launch": per_launch_s * 1000.0,
                    "note": "FP64 CUDA-core Hessian; FP64 issue rate, not HBM, limits it"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic",
        "config": config_of(w, args, args.precision), "niter_per_job": int(niter),
        "point_atom_evals_per_job": evals_per_job, "kernel_ms": fams,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_s},
        "roofline": roofline, "clocks": clocks.summary(),
        "gpu_launches": int(launches),
    }
    if args.precision == "mixed":
        # error of the mixed-precision result against the FP64 path on the
        # same input (the FP64 path matches the reference to 1e-8 e in tests)
        jm = make_job(ctx, w, "mixed")
        jm.run()
        rm, im = jm.results(promoldens=False, histories=False), jm.info()
        jm.close()
        jd = make_job(ctx, w, "fp64")
        jd.run()
        rd = jd.results(promoldens=False, histories=False)
        jd.close()
        off = np.asarray(job_arrays(w)[0])
        per = 2 if w["scheme"] == "mbis" else 1
        dp = 0.0
        for a in range(len(off) - 1):
            sl = slice(per * off[a], per * off[a + 1])
            for k in ((slice(0, None, 2), slice(1, None, 2)) if per == 2 else (slice(None),)):
                ref = rd["propars"][sl][k]
                dp = max(dp, float(np.abs(rm["propars"][sl][k] - ref).max() / np.abs(ref).max()))
        line["accuracy_vs_fp64"] = {
            "max_abs_dq_e": float(np.abs(rm["charges"] - rd["charges"]).max()),
            "max_scaled_dparam": dp, "polish_iterations": int(im.polish_iterations),
            "niter_mixed": int(im.niter)}
    if rank == 0 and world == 1 and not args.no_cpu:
        r, sample, threads = cpu_sample(w, 2 if w["scheme"] == "glisa" else 3)
        line["cpu_baseline"] = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    job.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="gisa-c6h10n2o2")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
