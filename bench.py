"""Benchmark of the partitioning loop on one GB300 (or N independent replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload glisa-c6h10n2o2|gisa-c6h10n2o2|mbis-h2o|mbis-chain60|
                                mbis-batch<N>|serve]
                    [--precision auto|fp64|mixed] [--no-polish] [--no-cpu] [--no-check]

Default workload: gLISA with non-negative populations (the reference's cvxopt
default, served by projected Newton) on a 20-atom C6H10N2O2 chain, 100 radial
x Lebedev-302 points per atom (604,000 points), 6 s-Gaussians per H and 9 per
C/N/O with exponents geometric in [0.05, 300] (150 shells), threshold 1e-8;
precision "auto" = the Hessian on the tensor cores with FP64 refinement. One
step = one complete partitioning job (every solver iteration until
convergence) on inputs already resident in HBM; the basis matrix G
(150 x 604,000 FP64 = 725 MB) is larger than L2, so no L2 flush is added
between steps.

Batched workloads (mbis-batch<N>: N molecules of 3-60 atoms, 75 x
Lebedev-194 per atom): a step is one outer iteration of every live job (one
pass of the loop over the whole batch, shared launches); the batch converges
over hundreds of such steps, so W warm-up and K timed steps are the first
W + K iterations from the initial parameters.

Metric: pro-atom evaluations (point x atom) per second, counted in the
reference's convention (gLISA: each solver iteration evaluates every pro-atom
on every grid point three times: promolecule and the two sides of the change;
MBIS/aLISA add one per inner iteration).

Output: one JSON line (rank 0). Under torchrun every rank runs its own
replica of the job (no collective on the data path); value = sum over ranks.
"""

from __future__ import annotations

import os

# The CPU baseline of a single job runs the NumPy oracle on one core, as the
# reference's single-job path runs (its NumPy element-wise work is single
# threaded); BLAS must not fan out over the host's cores. Set before NumPy loads.
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
os.environ.setdefault("MKL_NUM_THREADS", "1")

import argparse  # noqa: E402
import json  # noqa: E402
import statistics  # noqa: E402
import subprocess  # noqa: E402
import sys  # noqa: E402
import threading  # noqa: E402
import time  # noqa: E402
import warnings  # noqa: E402

import numpy as np  # noqa: E402

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
        # the reference's default gLISA solver (cvxopt: populations >= 0) is
        # served by projected Newton; exact Newton is singular on this basis
        return dict(name=name, scheme="glisa", solver="pnewton", mol=mol, helper=helper,
                    threshold=1e-8, maxiter=100)
    if name == "mbis-h2o":
        mol = synthetic.water(75, 110)
        return dict(name=name, scheme="mbis", solver="default", mol=mol, helper=None,
                    threshold=1e-8, maxiter=500)
    if name.startswith("alisa-peptide"):
        # 200-atom peptide-like chain (H:C:N:O:S 100:64:18:16:2), 150 radial x
        # Lebedev-590 per atom (17.7M points), 6 s-Gaussians per H, 9 per
        # C/N/O, 10 per S, exponents geometric in [0.05, 500] (1,502 shells);
        # aLISA sc. A step is one outer iteration whose inner sc loop runs at
        # most 50 iterations per atom: the throughput of the loop (the full
        # job needs thousands of inner iterations per outer iteration).
        # "alisa-peptide<A>": the same construction with about A atoms on
        # 75 x Lebedev-194 grids.
        natom = int(name[len("alisa-peptide"):] or 200)
        base = {1: 100, 6: 64, 7: 18, 8: 16, 16: 2}
        counts = {z: max(1, round(n * natom / 200)) for z, n in base.items()}
        nrad, nang = (150, 590) if natom >= 200 else (75, 194)
        mol = synthetic.peptide_molecule(counts=counts, nrad=nrad, nang=nang, seed=4)
        helper = synthetic.geometric_gaussian_basis({1: 6, 6: 9, 7: 9, 8: 9, 16: 10}, 0.05, 500.0)
        return dict(name=name, scheme="lisa", solver="sc", mol=mol, helper=helper,
                    threshold=1e-6, maxiter=500, inner_maxiter=50, per_iteration=True)
    if name == "mbis-chain60":
        # the largest molecule of the batched-MBIS mix: 60 atoms, 75 x Lebedev-194
        mols = synthetic.batch_molecules(natoms=[60], nrad=75, nang=194, seed=3)
        return dict(name=name, scheme="mbis", solver="default", mol=mols[0], helper=None,
                    threshold=1e-8, maxiter=500)
    if name.startswith("mbis-batch"):
        # 512 molecules, 3-60 atoms (H:C:N:O 10:6:1:1), 75 radial x Lebedev-194
        nmol = int(name[len("mbis-batch"):] or 512)
        mols = synthetic.batch_molecules(nmol=nmol, amin=3, amax=60, nrad=75, nang=194, seed=3)
        return dict(name=name, scheme="mbis", solver="default", mol=mols[0], mols=mols,
                    helper=None, threshold=1e-8, maxiter=500)
    raise ValueError(name)


def job_arrays(w, mol=None):
    mol = mol if mol is not None else w["mol"]
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


def make_job(ctx, w, precision, pinned=None, mol=None):
    from horton_part_gb300 import _lib

    mol = mol if mol is not None else w["mol"]
    off, init, orders, exps = job_arrays(w, mol)
    pts, wts, rho = (mol.grid.points, mol.grid.weights, mol.density) if pinned is None else pinned
    extra = {"inner_maxiter": 2000} if w["scheme"] == "mbis" else {}
    if "inner_maxiter" in w:
        extra["inner_maxiter"] = w["inner_maxiter"]
    return _lib.Job(ctx, w["scheme"], mol.coordinates, mol.pseudo_numbers, pts, wts, rho, off,
                    init, shell_orders=orders, shell_exponents=exps, solver=w["solver"],
                    precision=precision, grid_type=3, threshold=w["threshold"],
                    inner_threshold=w["threshold"], maxiter=w["maxiter"], polish=POLISH, **extra)


POLISH = True

# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu
# capture of the same workload (ncu --set full; the summaries in profiles/
# give the commands). Keyed by (workload, precision, kernel family).
NCU_TRAFFIC = {
    ("glisa-c6h10n2o2", "mixed", "k_glisa_hess_tc1"): 364.90e6 + 3.19e6,
    ("glisa-c6h10n2o2", "mixed", "k_glisa_fused_ff<1>"): 324.64e6 + 7.57e6,
    ("glisa-c6h10n2o2", "mixed", "k_glisa_trials_fused"): 329.22e6 + 27.24e6,
    ("mbis-chain60", "mixed", "inner"): 125.81e6 + 3.46e6,
}


def measure_tf32_peak(n=8192, reps=10):
    """Best-of-`reps` TF32 GEMM rate of cuBLAS (TFLOP/s, 2 n^3 per product),
    timed with CUDA events: the denominator of the tensor-core Hessian's
    roofline (no TF32 figure is recorded beside the HBM and BF16 peaks)."""
    import torch

    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        a = torch.randn(n, n, device="cuda", dtype=torch.float32)
        b = torch.randn(n, n, device="cuda", dtype=torch.float32)
        c = torch.empty(n, n, device="cuda", dtype=torch.float32)
        for _ in range(3):
            torch.matmul(a, b, out=c)
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1000.0)
        del a, b, c
        return 2.0 * n ** 3 / best / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old


def measure_fp64_peak(n=4096, reps=5):
    """Best-of-`reps` FP64 GEMM rate of cuBLAS (TFLOP/s): the denominator of
    the FP64 density kernel's roofline (no FP64 figure is recorded beside the
    HBM and BF16 peaks)."""
    import torch

    a = torch.randn(n, n, device="cuda", dtype=torch.float64)
    b = torch.randn(n, n, device="cuda", dtype=torch.float64)
    c = torch.empty(n, n, device="cuda", dtype=torch.float64)
    for _ in range(2):
        torch.matmul(a, b, out=c)
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1000.0)
    del a, b, c
    return 2.0 * n ** 3 / best / 1e12


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
    """Time the FP64 NumPy oracle on the same input on one host core; returns
    (evals/s, sample text, threads).

    gLISA: the oracle's projected Newton (the optimum of the reference's
    default cvxopt problem; cvxopt is not installed), the solver family the
    GPU runs, for ``iterations`` solver iterations including the basis set-up,
    counted like the GPU (three pro-atom passes per iteration)."""
    from oracle import hp_oracle as O

    mol = w["mol"]
    args = (mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid.points, mol.grid.weights,
            mol.density)
    threads = 1
    if w["scheme"] == "glisa":
        h = w["helper"]
        orders = [h.get_order(z) for z in mol.numbers]
        exps = [h.get_exponent(z) for z in mol.numbers]
        inits = [h.get_initial(z) for z in mol.numbers]
        t0 = time.perf_counter()
        res = O.glisa_nonneg(*args, orders, exps, inits, maxiter=iterations,
                             raise_on_maxiter=False)
        nit = res["niter"]
        dt = time.perf_counter() - t0
        evals = 3.0 * mol.natom * mol.npoint * nit
        return (evals / dt, f"oracle gLISA projected Newton (cvxopt problem), {nit} solver "
                f"iterations incl. basis set-up, {dt:.1f} s, 1 thread", threads)
    if w["scheme"] == "lisa":
        # one atom's inner sc iterations over the whole grid (the reference
        # solves the atoms one after another, alisa.py:1304-1335 -> 193-291)
        h = w["helper"]
        a = int(np.argmax(mol.numbers))
        r = np.linalg.norm(mol.grid.points - mol.coordinates[a], axis=1)
        t0 = time.perf_counter()
        bs = O.basis_functions(h.get_order(mol.numbers[a]), h.get_exponent(mol.numbers[a]), r)
        ini = np.array(h.get_initial(mol.numbers[a]), dtype=float)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            O.lisa_solver_sc(bs, mol.density * 0.5, ini / ini.sum() * mol.pseudo_numbers[a],
                             mol.grid.weights, 1e-30, max_niter_inner=iterations)
        dt = time.perf_counter() - t0
        evals = float(mol.npoint) * iterations
        return (evals / dt, f"oracle aLISA sc: {iterations} inner iterations of one atom over all "
                f"{mol.npoint} points incl. its basis, {dt:.1f} s, 1 thread", threads)
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
                f"{dt:.1f} s, 1 thread", threads)
    t0 = time.perf_counter()
    res = O.mbis(*args, threshold=w["threshold"], maxiter=iterations, inner_threshold=w["threshold"])
    dt = time.perf_counter() - t0
    inner = sum(sum(x) for x in res["inner_iterations"])
    evals = mol.npoint * (3.0 * mol.natom * res["niter"] + inner)
    return evals / dt, f"oracle MBIS, {res['niter']} outer iterations, {dt:.1f} s, 1 thread", 1


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def run_reference(args):
    from horton_part_gb300 import replicas

    world, rank, _ = replicas.env()
    if rank != 0:
        return
    # the serving mix has no CPU server; its CPU sample is the MBIS H2O job
    w = workload("mbis-h2o" if args.workload == "serve" else args.workload)
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
    mols = w.get("mols", [w["mol"]])
    mol = mols[0]
    natom = sum(m.natom for m in mols)
    npoint = sum(m.npoint for m in mols)
    # bytes streamed per pass: the basis matrix G (S x N, float-float planes or
    # FP64) for gLISA, rho_a (A x N values) for the other schemes
    if w["scheme"] == "glisa":
        resident = sum(sum(w["helper"].get_nshell(z) for z in m.numbers) * m.npoint
                       for m in mols) * 8
        what = "of G"
    else:
        resident = sum(m.natom * m.npoint for m in mols) * (4 if precision == "mixed" else 8)
        what = "of rho_a"
    cfg = {"workload": w["name"], "molecules": len(mols), "natom": int(natom),
           "npoint": int(npoint),
           "nshell": int(sum(w["helper"].get_nshell(z) for z in mol.numbers)) if w["helper"] else None,
           "solver": w["solver"], "threshold": w["threshold"], "precision": precision,
           "polish": POLISH if precision == "mixed" else None,
           "l2": ("inputs larger than L2 (%.0f MB %s per pass)" % (resident / 1e6, what))
           if resident > 129e6 else "inputs smaller than L2 (%.0f MB)" % (resident / 1e6),
           "parallelism": f"replicas{args.gpus}"}
    return cfg


def run_ours(args):
    import torch

    from horton_part_gb300 import replicas

    # one process per GPU, each running its own replica of the job: no
    # collective on the data path, only the barrier and max-over-ranks timing
    world, rank, local = replicas.init("nccl")
    torch.cuda.set_device(local if world > 1 else 0)
    from horton_part_gb300 import _lib
    from horton_part_gb300.build import build

    build()
    w = workload(args.workload)
    mol = w["mol"]
    mols = w.get("mols", [mol])
    stream = torch.cuda.current_stream()
    ctx = _lib.Context(torch.cuda.current_device(), stream=stream.cuda_stream)
    jobs = [make_job(ctx, w, args.precision, mol=m) for m in mols]
    job = jobs[0]

    # A step: for one molecule, one complete job (every iteration to
    # convergence); for a batch of molecules, one outer iteration of every
    # live job (the batch converges over hundreds of such steps).
    batched = len(mols) > 1 or bool(w.get("per_iteration"))

    def run_all(js):
        for j in js:
            j.reset()
        if len(js) == 1:
            js[0].run()  # hp_job_run: gLISA queues several iterations per round trip
        else:
            while ctx.step(js) > 0:
                pass

    def one_step(js):
        if batched:
            ctx.step(js)
        else:
            run_all(js)

    def snapshot(js):
        return [(i.point_atom_evals, i.niter, i.inner_iterations, i.point_atom_evals_skipped)
                for i in (j.info() for j in js)]

    if batched:
        for j in jobs:
            j.reset()
    for _ in range(args.warmup):
        one_step(jobs)
    before = snapshot(jobs)
    barrier = replicas.barrier

    ctx.profile(False)  # no per-family events in the timed region; resets the launch counter
    barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            one_step(jobs)
        end.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = start.elapsed_time(end)
    launches = ctx.launch_count()
    after = snapshot(jobs)
    if batched:
        evals_timed = sum(a[0] - b[0] for a, b in zip(after, before))
        skipped_timed = sum(a[3] - b[3] for a, b in zip(after, before))
    else:
        evals_timed = args.steps * sum(a[0] for a in after)
        skipped_timed = args.steps * sum(a[3] for a in after)
    niter = max(a[1] for a in after)
    # one more step with CUDA events around each kernel family (on the
    # launching stream) for the per-family times and the roofline
    ctx.profile(True)
    one_step(jobs)
    hess_ms, hess_n = ctx.profile_get("glisa_hess")
    fam_ms = {f: ctx.profile_get(f) for f in _lib.KERNEL_FAMILIES}
    ctx.profile(False)
    prof = snapshot(jobs)
    if batched:  # work of the profiled step: the differences
        d_iter = [p[1] - a[1] for p, a in zip(prof, after)]
        d_inner = [p[2] - a[2] for p, a in zip(prof, after)]
    else:
        d_iter = [p[1] for p in prof]
        d_inner = [p[2] for p in prof]
    ms_max = replicas.reduce_max(ms)
    value = evals_timed * world / (ms_max / 1000.0)
    evals_per_step = evals_timed / args.steps

    # end to end through the C ABI: host inputs (pinned), job creation (H2D),
    # the same work as one step (a batch: creation, warm-up and timed
    # iterations), charges and parameters back (D2H), destroy
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    pinned = [(pin(m.grid.points), pin(m.grid.weights), pin(m.density)) for m in mols]
    e2e_steps = 1 if batched else max(1, min(args.steps, 3))
    if batched:
        for j in jobs:  # the resident copies make room for the end-to-end jobs
            j.close()
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_jobs = [make_job(ctx, w, args.precision, pinned=pp, mol=m) for pp, m in zip(pinned, mols)]
        if batched:
            for _ in range(args.warmup + args.steps):
                ctx.step(e2e_jobs)
        elif len(e2e_jobs) == 1:
            e2e_jobs[0].run()
        else:
            while ctx.step(e2e_jobs) > 0:
                pass
        e2e_evals = sum(j2.info().point_atom_evals for j2 in e2e_jobs)
        q = [j2.results(promoldens=False, histories=False) for j2 in e2e_jobs]
        for j2 in e2e_jobs:
            j2.close()
    torch.cuda.synchronize()
    e2e_s = replicas.reduce_max((time.perf_counter() - t0) / e2e_steps)
    e2e_value = e2e_evals * world / e2e_s
    h2d = int(sum(m.npoint * 5 * 8 + m.natom * 4 * 8 for m in mols))
    d2h = int(sum(r["charges"].nbytes + r["propars"].nbytes for r in q))
    if batched:
        jobs = [make_job(ctx, w, args.precision, mol=mols[0])]
        job = jobs[0]

    fams = {k: {"ms": round(v[0], 3), "launches": v[1]} for k, v in fam_ms.items() if v[1]}
    roofline = None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    if w["scheme"] != "glisa":
        # Dominant kernel family and its algorithmic bytes per launch, from the
        # work of the profiled step: every per-point array once per pass (all
        # atoms of a point share it) plus every per-(atom, point) array once.
        # Per point: coordinates 24 B (FP64, or float hi/lo pairs), w and rho
        # one value each; per pair: rho_a (and the pro-atom) one value. Value
        # size: mixed 4 B (FP32), ff and fp64 8 B (float pair or double).
        val = 4.0 if args.precision == "mixed" else 8.0
        pt = 24.0
        an_pass = sum(m.natom * m.npoint * d for m, d in zip(mols, d_iter))  # per outer pass
        pt_pass = sum(m.npoint * d for m, d in zip(mols, d_iter))
        inner_evals = float(sum(m.npoint * d for m, d in zip(mols, d_inner)))
        # the per-atom cutoff skips (atom, tile) pairs: count performed work
        d_all = sum(p[0] - a[0] for p, a in zip(prof, after)) if batched else sum(p[0] for p in prof)
        d_skip = sum(p[3] - a[3] for p, a in zip(prof, after)) if batched else sum(p[3] for p in prof)
        performed = 1.0 - d_skip / d_all if d_all > 0 else 1.0
        inner_evals *= performed
        if w["scheme"] == "gisa":
            inner_evals = an_pass
        per_step = {  # (point-atom evals, algorithmic bytes) of the profiled step
            # promolecule + at_weights: points (xyz, w, rho, promol), pro-atom
            # written, read back and rho_a written
            "promol": (an_pass, pt_pass * (pt + 3 * val) + an_pass * 3 * val),
            # inner iterations: points (xyz, w) per launch, rho_a per pair
            "inner": (inner_evals, None),
            # outer change: points (xyz, w)
            "change": (an_pass, pt_pass * (pt + val)),
        }
        fam = max(per_step, key=lambda f: fam_ms[f][0])
        f_ms, f_n = fam_ms[fam]
        if f_n:
            evals, step_bytes = per_step[fam]
            per_launch_s = f_ms / f_n / 1000.0
            if step_bytes is None:  # inner: points once per launch plus rho_a per evaluation
                n_pts = float(sum(m.npoint for m in mols))
                alg_bytes = n_pts * (pt + val) + evals / f_n * val
            else:
                alg_bytes = step_bytes / f_n
            achieved = alg_bytes / per_launch_s / 1e9
            roofline = {"kernel": fam, "bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                        "unit": "GB/s", "frac": achieved / hbm_peak,
                        "traffic": NCU_TRAFFIC.get((w["name"], args.precision, fam)),
                        "peak_source": "measured" if peaks else "fallback",
                        "ms_per_launch": per_launch_s * 1000.0,
                        "algorithmic_bytes_per_launch": alg_bytes,
                        "point_atom_evals_per_launch": evals / f_n}
    job_bound = None
    if w["scheme"] == "glisa":
        nshell = config_of(w, args, args.precision)["nshell"]
        g_active = float(job.info().g_active_values)
        fused = args.precision == "mixed" and nshell <= 192 and g_active > 0
        if fused:
            # The two passes over G of a tensor-core gLISA iteration; the
            # roofline line is the one with more time in the profiled step.
            # Bytes: G's two float planes in the tiles' active rows only (8
            # bytes per value; the other rows are identically zero on their
            # tile and never read) plus the per-point arrays.
            cands = {}
            pro_ms, pro_n = fam_ms["glisa_pro"]
            if pro_n:
                # promolecule + gradient + change + tensor-core Hessian: w rho
                # and rho as float pairs (16 B) and w (8 B) in, rho0 and
                # w rho / rho0^2 as float pairs (16 B) out
                p_s = pro_ms / pro_n / 1000.0
                alg = 8.0 * g_active + mol.npoint * (16.0 + 8.0 + 16.0)
                ach = alg / p_s / 1e9
                hflop = 2.0 * nshell * nshell * mol.npoint
                cands["pro"] = (pro_ms, {
                    "kernel": "k_glisa_fused_ff<1>", "bound": "hbm", "achieved": ach,
                    "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
                    "traffic": NCU_TRAFFIC.get((w["name"], args.precision, "k_glisa_fused_ff<1>")),
                    "peak_source": "measured" if peaks else "fallback",
                    "ms_per_launch": p_s * 1000.0, "algorithmic_bytes_per_launch": alg,
                    "active_fraction_of_G": g_active / (nshell * mol.npoint),
                    "hessian_tflops_in_pass": hflop / p_s / 1e12,
                    "hessian_flop_per_launch": hflop,
                    "note": "one pass over G per iteration forms rho0, the gradient, the "
                            "change (compensated FP32 sums) and the Hessian (tcgen05 TF32 "
                            "MMAs on the staged sub-tiles)"})
            tr_ms, tr_n = fam_ms.get("glisa_trials", (0.0, 0))
            if tr_n:
                # trial pass: u = G^T delta and eight trial objectives; rho0
                # pair (8 B) and w rho / rho pairs (16 B) in
                t_s = tr_ms / tr_n / 1000.0
                alg = 8.0 * g_active + mol.npoint * (8.0 + 16.0)
                ach = alg / t_s / 1e9
                cands["trials"] = (tr_ms, {
                    "kernel": "k_glisa_trials_fused", "bound": "hbm", "achieved": ach,
                    "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
                    "traffic": NCU_TRAFFIC.get((w["name"], args.precision, "k_glisa_trials_fused")),
                    "peak_source": "measured" if peaks else "fallback",
                    "ms_per_launch": t_s * 1000.0, "algorithmic_bytes_per_launch": alg,
                    "note": "family time: also the trial set-up and pick (one block per job)"})
            if cands:
                fam = max(cands, key=lambda k: cands[k][0])
                roofline = cands[fam][1]
                others = {k: v[1] for k, v in cands.items() if k != fam}
                if others:
                    roofline["other_kernels"] = {v["kernel"]: {
                        "achieved": v["achieved"], "unit": v["unit"], "frac": v["frac"],
                        "ms_per_launch": v["ms_per_launch"]} for v in others.values()}
            # job-level bound: the bytes of G every solver iteration reads at
            # least (two passes over the active rows of both planes) at the
            # copy peak, against the measured time per job
            per_iter = 2 * 8.0 * g_active
            bound_ms = per_iter * niter / (hbm_peak * 1e9) * 1e3
            job_bound = {"g_bytes_per_iteration": per_iter, "iterations": int(niter),
                         "hbm_bound_ms": bound_ms, "frac_of_job": bound_ms / (ms / args.steps)}
        elif hess_n and hess_ms > 0:
            per_launch_s = hess_ms / hess_n / 1000.0
            if args.precision == "mixed":
                flops = 2.0 * nshell * nshell * mol.npoint
                achieved = flops / per_launch_s / 1e12
                tf32 = measure_tf32_peak()
                hk = "k_glisa_hess_tc1" if nshell <= 256 else "k_glisa_hess_tc"
                roofline = {
                    "kernel": hk, "bound": "tensor", "achieved": achieved,
                    "peak": tf32, "unit": "TFLOP/s", "frac": achieved / tf32,
                    "traffic": NCU_TRAFFIC.get((w["name"], args.precision, hk)),
                    "peak_source": "measured: cuBLAS TF32 GEMM 8192^3, this run",
                    "ms_per_launch": per_launch_s * 1000.0, "algorithmic_flop_per_launch": flops}
            else:
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
        "point_atom_evals_per_step": evals_per_step,
        "point_atom_evals_performed_per_step": (evals_timed - skipped_timed) / args.steps,
        "kernel_ms_one_profiled_step": fams,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_s},
        "roofline": roofline, "job_hbm_bound": job_bound, "clocks": clocks.summary(),
        "gpu_launches": int(launches),
    }
    if args.precision == "mixed" and not args.no_check and not w.get("per_iteration"):
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
        if w["scheme"] == "glisa":
            line["accuracy_vs_fp64"]["newton_fp64_factors"] = int(im.f64_factors)
        fixture = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                               "glisa_nonneg_c6h10n2o2_100x302.npz")
        if w["name"] == "glisa-c6h10n2o2" and os.path.exists(fixture):
            # the optimum of the reference's cvxopt problem on this input, certified
            # by its KKT residuals (tests/golden/make_glisa_nonneg.py)
            with np.load(fixture) as f:
                opt = f["charges"]
            line["accuracy_vs_certified_optimum"] = {
                "max_abs_dq_e_mixed": float(np.abs(rm["charges"] - opt).max()),
                "max_abs_dq_e_fp64": float(np.abs(rd["charges"] - opt).max())}
    if rank == 0 and world == 1 and args.workload == "glisa-c6h10n2o2" and not args.no_extras:
        line.update(extra_sections(ctx, args, w))
    if rank == 0 and world == 1 and not args.no_cpu:
        r, sample, threads = cpu_sample(w, 2 if w["scheme"] == "glisa" else 3)
        line["cpu_baseline"] = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    job.close()
    ctx.close()
    replicas.finalize()


def density_section(ctx, mol):
    """The density generator (part-gen's density step) on the molecule's
    grid: a split-valence-plus-d basis on every atom (14 functions per heavy
    atom, 5 per H) and a closed-shell density matrix, FP64. Device-resident
    points timed with CUDA events (3 evaluations after 2 warm-ups), the
    host-array call timed end to end, the oracle timed on 20,000 points on
    one core, and the GPU result checked against the oracle there."""
    import torch

    from horton_part_gb300 import synthetic
    from horton_part_gb300.density import DensityPlan
    from oracle import hp_density as H

    from horton_part_gb300 import _lib

    shells = synthetic.contracted_basis(mol.numbers, mol.coordinates)
    nb = sum(s.nfunc for s in shells)
    D = synthetic.density_matrix(nb, int(round(float(np.sum(mol.numbers)) / 2)))
    pts_h = np.ascontiguousarray(mol.grid.points)
    n = len(pts_h)
    pts = torch.tensor(pts_h, device="cuda")
    out = torch.empty((1, n), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    # a context on a stream of its own, so that the events below are recorded
    # on the stream the kernel runs on
    stream = torch.cuda.Stream()
    dctx = _lib.Context(torch.cuda.current_device(), stream=stream.cuda_stream)
    plan = DensityPlan(shells, D, context=dctx)
    for _ in range(2):
        plan.evaluate_device(pts, out)
    torch.cuda.synchronize()
    st0 = plan.stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    e0.record(stream)
    for _ in range(reps):
        plan.evaluate_device(pts, out)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    st1 = plan.stats()
    fma = (st1["fma_per_matrix"] - st0["fma_per_matrix"]) / reps
    values = (st1["basis_values"] - st0["basis_values"]) / reps
    t0 = time.perf_counter()
    host = plan.evaluate(pts_h)[0]
    e2e_s = time.perf_counter() - t0
    sample = np.random.default_rng(9).choice(n, 20000, replace=False)
    t0 = time.perf_counter()
    ref = H.density(D, shells, pts_h[sample])
    cpu_s = time.perf_counter() - t0
    plan.close()
    dctx.close()
    peak = measure_fp64_peak()
    achieved = 2.0 * fma / (ms / 1e3) / 1e12
    return {
        "workload": f"density-{mol.natom}atoms", "npoint": n, "nbasis": nb, "nshell": len(shells),
        "dtype": "f64", "ms_per_evaluation": ms, "points_per_s": n / (ms / 1e3),
        "e2e": {"seconds": e2e_s, "points_per_s": n / e2e_s, "h2d_bytes": 24 * n, "d2h_bytes": 8 * n},
        "screening": {"basis_values_fraction": values / (nb * n),
                      "contraction_fma": fma, "dense_fma": nb * (nb + 1) / 2 * n},
        "roofline": {"kernel": "k_density", "bound": "fp64", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak,
                     "peak_source": "measured: cuBLAS FP64 GEMM 4096^3, this run",
                     "note": "contraction FMA (2 FLOP each) only; the exps of the basis values "
                             "are extra FP64 work"},
        "cpu_baseline": {"points_per_s": len(sample) / cpu_s, "cores": 1, "kind": "port",
                         "sample": f"oracle density (NumPy einsum) on {len(sample)} points, "
                                   f"{cpu_s:.1f} s, 1 thread"},
        "err_vs_oracle": {
            "max_abs_over_max_rho": float(np.max(np.abs(host[sample] - ref)) / np.max(np.abs(ref))),
            "max_rel_where_rho_above_1e-8_max": float(np.max(
                (np.abs(host[sample] - ref) / np.abs(ref))[np.abs(ref) > 1e-8 * np.max(np.abs(ref))]))},
    }


def extra_sections(ctx, args, workload_main=None):
    """Bounded measurements of the metric's other workloads, added to the
    default line: the batched MBIS step (config 3's generator, 32 molecules
    of 3-60 atoms, 75 x Lebedev-194 per atom; three outer iterations of every
    job with shared launches, timed with CUDA events) and the continuous-
    batching server (12 requests, 70 % MBIS / 30 % gLISA, 3-60 atoms:
    closed-loop capacity, then Poisson arrivals at 70 % of it with p50/p99
    latency), and the density generator on the main workload's molecule and
    grid (density_section). Each takes a few tens of seconds."""
    import torch

    from horton_part_gb300 import _lib, synthetic
    from horton_part_gb300.serve import PartitionServer, request_from_molecule

    out = {}
    stream = torch.cuda.current_stream()
    w = {"scheme": "mbis", "solver": "default", "threshold": 1e-8, "maxiter": 500, "helper": None}
    mols = synthetic.batch_molecules(nmol=32, amin=3, amax=60, nrad=75, nang=194, seed=3)
    jobs = [make_job(ctx, w, "mixed", mol=m) for m in mols]
    for _ in range(2):  # warm-up: the first outer iterations
        ctx.step(jobs)
    before = [j.info() for j in jobs]
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    nsteps = 3
    for _ in range(nsteps):
        ctx.step(jobs)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    after = [j.info() for j in jobs]
    evals = sum(a.point_atom_evals - b.point_atom_evals for a, b in zip(after, before))
    skipped = sum(a.point_atom_evals_skipped - b.point_atom_evals_skipped for a, b in zip(after, before))
    for j in jobs:
        j.close()
    out["batch"] = {"workload": "mbis-batch32", "molecules": len(mols),
                    "natom": int(sum(m.natom for m in mols)),
                    "npoint": int(sum(m.npoint for m in mols)), "precision": "mixed",
                    "steps": nsteps, "ms_per_step": ms / nsteps,
                    "point_atom_evals_per_s": evals / (ms / 1000.0),
                    "performed_fraction": 1.0 - skipped / evals if evals else None}
    # serving: 12 requests from the serving mix's generator, atoms 3-60
    rng = np.random.default_rng(17)
    nreq = 12
    is_mbis = rng.random(nreq) < 0.7
    natoms = np.rint(np.exp(rng.uniform(np.log(3.0), np.log(60.0), nreq))).astype(int)
    mb = iter(synthetic.batch_molecules(natoms=natoms[is_mbis], nrad=75, nang=194, seed=17))
    gl = iter(synthetic.batch_molecules(natoms=natoms[~is_mbis], nrad=100, nang=302, seed=18))
    pool = [("mbis", next(mb), "default") if is_mbis[i] else ("glisa", next(gl), "pnewton")
            for i in range(nreq)]

    def serve(arrivals):
        srv = PartitionServer(hbm_budget=150 * 10**9)
        reqs = [request_from_molecule(i, sch, m, precision="mixed", threshold=1e-8, solver=sv)
                for i, (sch, m, sv) in enumerate(pool)]
        wall = srv.run_stream(reqs, arrivals)
        st = srv.stats(wall)
        srv.close()
        return st

    cap = serve(np.zeros(nreq))
    lam = 0.7 * cap["jobs_per_s"]
    arr = np.cumsum(np.random.default_rng(19).exponential(1.0 / lam, nreq))
    load = serve(arr)
    out["serving"] = {"requests": nreq, "mbis": int(is_mbis.sum()), "glisa": int((~is_mbis).sum()),
                      "natom_total": int(natoms.sum()), "precision": "mixed",
                      "capacity_jobs_per_s": cap["jobs_per_s"],
                      "poisson_arrival_rate_jobs_per_s": lam, "poisson": load,
                      "note": "every request enters from host arrays and returns its results"}
    if workload_main is not None:
        out["density"] = density_section(ctx, workload_main["mol"])
    return out


def serve_requests(nreq, seed, precision):
    """Seeded request mix of the serving workload: 70 % MBIS on 75 x Lebedev-194
    grids, 30 % gLISA (projected Newton, default Gaussian basis) on 100 x
    Lebedev-302 grids, atom counts log-uniform in [3, 150], threshold 1e-8."""
    from horton_part_gb300 import synthetic
    from horton_part_gb300.serve import request_from_molecule

    rng = np.random.default_rng(seed)
    is_mbis = rng.random(nreq) < 0.7
    natoms = np.rint(np.exp(rng.uniform(np.log(3.0), np.log(150.0), nreq))).astype(int)
    mb = iter(synthetic.batch_molecules(natoms=natoms[is_mbis], nrad=75, nang=194, seed=seed))
    gl = iter(synthetic.batch_molecules(natoms=natoms[~is_mbis], nrad=100, nang=302,
                                        seed=seed + 1))
    return [("mbis", next(mb), "default") if is_mbis[i] else ("glisa", next(gl), "pnewton")
            for i in range(nreq)]


def run_serve(args):
    """Continuous-batching server under Poisson arrivals: the closed-loop
    capacity first (every request queued at t = 0), then arrival rates at
    50 % and 80 % of it, each reporting jobs/s and p50/p99 latency. Every
    request enters from host arrays (job creation copies them in) and its
    charges and parameters come back to the host, so the served rate is an
    end-to-end figure."""
    import torch

    from horton_part_gb300 import _lib
    from horton_part_gb300.build import build
    from horton_part_gb300.serve import PartitionServer, request_from_molecule

    torch.cuda.set_device(0)
    build()
    pool = serve_requests(args.serve_jobs, 5, args.precision)
    h2d = sum(m.npoint * 5 * 8 + m.natom * 4 * 8 for _, m, _ in pool)

    def requests(precision=args.precision):
        return [request_from_molecule(i, s, m, precision=precision, threshold=1e-8, solver=sv,
                                      polish=POLISH)
                for i, (s, m, sv) in enumerate(pool)]

    def serve(arrivals, precision=args.precision):
        srv = PartitionServer(hbm_budget=150 * 10**9)
        reqs = requests(precision)
        with ClockSampler(torch.cuda.current_device()) as clocks:
            wall = srv.run_stream(reqs, arrivals)
        st = srv.stats(wall)
        launches = srv.ctx.launch_count()
        srv.close()
        return reqs, st, wall, clocks.summary(), launches

    # warm-up: the smallest MBIS and gLISA requests once
    small = sorted(range(len(pool)), key=lambda i: pool[i][1].npoint)
    warm = [i for i in small if pool[i][0] == "mbis"][:1] + [i for i in small if pool[i][0] == "glisa"][:1]
    for _ in range(max(1, args.warmup // 3)):
        srv = PartitionServer(hbm_budget=150 * 10**9)
        srv.run_stream([requests()[i] for i in warm], np.zeros(len(warm)))
        srv.close()

    reqs, cap, wall0, clocks, launches = serve(np.zeros(len(pool)))
    capacity = cap["jobs_per_s"]
    rates = []
    rng = np.random.default_rng(11)
    for frac in (0.5, 0.8):
        lam = frac * capacity
        arr = np.cumsum(rng.exponential(1.0 / lam, len(pool)))
        _, st, wall, _, _ = serve(arr)
        rates.append({"arrival_rate_jobs_per_s": lam, "load": frac, **st, "wall_s": wall})

    # accuracy: the served (mixed-precision) charges of the smallest requests
    # against the FP64 path run alone
    check = [i for i in small if pool[i][0] == "mbis"][:3] + [i for i in small if pool[i][0] == "glisa"][:1]
    dq = 0.0
    ctx = _lib.Context(0)
    for i in check:
        s, m, sv = pool[i]
        r = request_from_molecule(i, s, m, precision="fp64", threshold=1e-8, solver=sv)
        j = _lib.Job(ctx, r.scheme, **r.arrays, **r.options)
        j.run()
        ref = j.results(promoldens=False, histories=False)["charges"]
        j.close()
        got = reqs[i].result["charges"] if reqs[i].result is not None else None
        if got is not None:
            dq = max(dq, float(np.abs(got - ref).max()))
    ctx.close()

    evals = sum(r.evals for r in reqs)
    value = evals / wall0
    d2h = sum(r.result["charges"].nbytes + r.result["propars"].nbytes
              for r in reqs if r.result is not None)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": 1,
        "warmup": args.warmup, "ms_per_step": wall0 * 1000.0, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": "serve", "requests": len(pool),
                   "mbis": sum(1 for p in pool if p[0] == "mbis"),
                   "glisa": sum(1 for p in pool if p[0] == "glisa"),
                   "natom_total": int(sum(p[1].natom for p in pool)),
                   "npoint_total": int(sum(p[1].npoint for p in pool)),
                   "precision": args.precision, "hbm_budget_gb": 150, "threshold": 1e-8,
                   "l2": "inputs larger than L2", "parallelism": "replicas1"},
        "serving": {"capacity_jobs_per_s": capacity, "closed_loop": cap, "poisson": rates,
                    "max_abs_dq_vs_fp64_e": dq, "dq_checked_requests": len(check)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "note": "every request enters from host arrays and returns its results"},
        "clocks": clocks, "gpu_launches": int(launches),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="glisa-c6h10n2o2")
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed", "ff"],
                    help="auto: MBIS mixed (FP32 bulk, float-float finish); gLISA mixed "
                         "(tensor-core Hessian, FP64 refinement); GISA FP64 with the basis "
                         "matrix resident. ff: MBIS in float-float throughout")
    ap.add_argument("--no-polish", action="store_true",
                    help="mixed precision: stay in FP32 to the threshold (no finish phase)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the bounded batch and serving sections of the default workload")
    ap.add_argument("--no-check", action="store_true",
                    help="skip the mixed-precision accuracy run against the FP64 path")
    ap.add_argument("--serve-jobs", type=int, default=32,
                    help="serving workload: number of requests in the stream")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.precision == "auto":
        # MBIS: FP32 bulk with an FP64 finish; gLISA: tensor-core Hessian with
        # FP64 refinement; GISA: FP64 with the basis matrix resident
        args.precision = "fp64" if args.workload.startswith("gisa") else "mixed"
    global POLISH
    POLISH = not args.no_polish
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "serve":
        run_serve(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
