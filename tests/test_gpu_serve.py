"""Continuous batching: requests that arrive while others run are admitted as
memory frees up, advance together, and give the same result as alone.

Every reduction of a job runs in a fixed order over that job's own tiles, so
"the same" here is bit-identical (tolerance 0).
"""

import numpy as np
import pytest

from horton_part_gb300 import _lib, synthetic
from horton_part_gb300.serve import PartitionServer, request_from_molecule

pytestmark = pytest.mark.gpu


def _molecules():
    return [
        ("mbis", synthetic.water(nrad=30, nang=50)),
        ("glisa", synthetic.water(nrad=30, nang=50)),
        ("mbis", synthetic.chain_molecule({6: 1, 8: 1, 1: 3}, 25, 50, seed=11)),
        ("glisa", synthetic.chain_molecule({6: 1, 8: 1, 1: 3}, 25, 50, seed=11)),
        ("mbis", synthetic.chain_molecule({6: 2, 7: 1, 1: 5}, 20, 50, seed=5)),
        ("mbis", synthetic.chain_molecule({6: 3, 1: 4}, 20, 50, seed=9)),
    ]


def _request(i, scheme, mol, precision):
    """MBIS in the given precision; gLISA with the FP64 Newton solver, or in the
    mixed form of the serving workload (projected Newton with the tensor-core
    Hessian and float-float G) when the precision is mixed."""
    if scheme != "glisa":
        return request_from_molecule(i, scheme, mol, precision=precision, solver="default")
    if precision == "mixed":
        return request_from_molecule(i, scheme, mol, precision="mixed", solver="pnewton")
    return request_from_molecule(i, scheme, mol, precision="fp64", solver="newton")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_served_results_equal_alone(precision, gpu_context):
    mols = _molecules()
    alone = []
    ctx = _lib.Context(0)
    for i, (scheme, mol) in enumerate(mols):
        req = _request(i, scheme, mol, precision)
        job = _lib.Job(ctx, scheme, **req.arrays, **req.options)
        job.run()
        alone.append(job.results(promoldens=False, histories=False))
        job.close()
    ctx.close()

    server = PartitionServer(hbm_budget=8 * 10**9)
    reqs = [_request(i, s, m, precision) for i, (s, m) in enumerate(mols)]
    arrivals = np.array([0.0, 0.0, 0.02, 0.05, 0.05, 0.1])  # some arrive mid-run
    wall = server.run_stream(reqs, arrivals, time_limit=300)
    stats = server.stats(wall)
    server.close()
    assert stats["jobs_done"] == len(mols) and stats["jobs_failed"] == 0
    assert stats["p99_latency_s"] >= stats["p50_latency_s"] > 0
    for req in reqs:
        got, want = req.result, alone[req.rid]
        assert np.array_equal(got["charges"], want["charges"]), req.rid
        assert np.array_equal(got["propars"], want["propars"]), req.rid


def test_admission_waits_for_memory(gpu_context):
    """With a budget that holds about two jobs, the rest wait and still finish."""
    mols = _molecules()[:4]
    reqs = [_request(i, s, m, "fp64") for i, (s, m) in enumerate(mols)]
    probe = _lib.Context(0)
    job = _lib.Job(probe, reqs[3].scheme, **reqs[3].arrays, **reqs[3].options)
    need = job.info().device_bytes
    job.close()
    probe.close()
    server = PartitionServer(hbm_budget=int(2.2 * need))
    wall = server.run_stream(reqs, np.zeros(len(reqs)), time_limit=300)
    stats = server.stats(wall)
    server.close()
    assert stats["jobs_done"] == len(reqs)
    assert max(r.admitted - r.arrival for r in reqs) > 0  # someone waited for memory
