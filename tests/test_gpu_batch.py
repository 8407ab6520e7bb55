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
