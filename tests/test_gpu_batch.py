"""Batched stepping: several jobs of uneven size advanced together by
hp_step give bit-identical results to each job run alone (fixed per-job
tiles and fixed reduction orders make every reduction independent of the
batch it runs in)."""

import numpy as np
import pytest

from horton_part_gb300 import _lib, synthetic
from horton_part_gb300.mbis import get_initial_mbis_propars, get_nshell

pytestmark = pytest.mark.gpu


def mbis_job(ctx, mol, **kw):
    nsh = [int(get_nshell(z)) for z in mol.numbers]
    off = np.concatenate([[0], np.cumsum(nsh)]).astype(np.int32)
    init = np.concatenate([get_initial_mbis_propars(z) for z in mol.numbers])
    return _lib.Job(ctx, "mbis", mol.coordinates, mol.pseudo_numbers, mol.grid.points,
                    mol.grid.weights, mol.density, off, init, threshold=1e-8, maxiter=500,
                    inner_threshold=1e-8, inner_maxiter=2000, **kw)


def molecules():
    return [synthetic.water(nrad=40, nang=110),
            synthetic.chain_molecule({6: 1, 8: 1, 1: 3}, 30, 50, seed=11),
            synthetic.chain_molecule({6: 2, 7: 1, 1: 5}, 25, 50, seed=5)]


def test_batch_equals_alone(gpu_context):
    ctx = gpu_context
    mols = molecules()
    alone = []
    for m in mols:
        j = mbis_job(ctx, m)
        j.run()
        alone.append(j.results())
        j.close()
    jobs = [mbis_job(ctx, m) for m in mols]
    steps = 0
    while ctx.step(jobs) > 0:
        steps += 1
        assert steps < 1000
    for j, a in zip(jobs, alone):
        r = j.results()
        assert np.array_equal(r["charges"], a["charges"])
        assert np.array_equal(r["propars"], a["propars"])
        assert np.array_equal(r["history_changes"], a["history_changes"])
        j.close()


def test_jobs_join_a_running_batch(gpu_context):
    """A job admitted while others are mid-run gets the same result as alone."""
    ctx = gpu_context
    mols = molecules()
    ref = mbis_job(ctx, mols[2])
    ref.run()
    want = ref.results()
    ref.close()
    jobs = [mbis_job(ctx, mols[0]), mbis_job(ctx, mols[1])]
    for _ in range(5):
        ctx.step(jobs)
    late = mbis_job(ctx, mols[2])
    jobs.append(late)
    while ctx.step(jobs) > 0:
        pass
    got = late.results()
    assert np.array_equal(got["charges"], want["charges"])
    for j in jobs:
        j.close()


@pytest.mark.parametrize("solver,precision", [("pnewton", "mixed"), ("newton", "fp64"),
                                              ("sc", "fp64")])
def test_queued_glisa_iterations_equal_one_per_round_trip(solver, precision, gpu_context):
    """hp_step_n queues several gLISA iterations per host round trip; the
    device stops each job at the iteration that finishes it, so a batch
    advanced 8 iterations at a time ends bit-identical (results, iteration
    counts, histories) to one iteration per hp_step."""
    from horton_part_gb300.serve import request_from_molecule

    ctx = gpu_context
    mols = [synthetic.water(nrad=30, nang=50),
            synthetic.chain_molecule({6: 1, 8: 1, 1: 3}, 25, 50, seed=11)]
    reqs = [request_from_molecule(i, "glisa", m, precision=precision, solver=solver,
                                  maxiter=5000 if solver == "sc" else None)
            for i, m in enumerate(mols)]
    results = []
    for chunk in (1, 8):
        jobs = [_lib.Job(ctx, "glisa", **r.arrays, **r.options) for r in reqs]
        calls = 0
        while ctx.step(jobs, chunk) > 0:
            calls += 1
            assert calls < 6000
        results.append([(j.results(), j.info()) for j in jobs])
        for j in jobs:
            j.close()
    for (r1, i1), (r8, i8) in zip(*results):
        assert i1.niter == i8.niter and i1.converged == i8.converged == 1
        for key in ("charges", "propars", "history_changes", "history_entropies"):
            assert np.array_equal(r1[key], r8[key]), key
