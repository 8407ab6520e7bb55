"""Multi-rank host logic of the replicas path on CPU (gloo, world size 2):
job sharding, barrier and the max / sum reductions the benchmark uses for
its timed region."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")

from horton_part_gb300 import replicas  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    w, r, _ = replicas.init("gloo")
    jobs = replicas.shard(range(11), r, w)
    replicas.barrier()
    out[rank] = (w, r, jobs, replicas.reduce_max(10.0 * (r + 1)), replicas.reduce_sum(len(jobs)))
    replicas.finalize()


def test_shard_covers_every_job_once():
    for world in (1, 2, 3, 8):
        parts = [replicas.shard(range(21), r, world) for r in range(world)]
        flat = sorted(x for p in parts for x in p)
        assert flat == list(range(21))
        assert max(map(len, parts)) - min(map(len, parts)) <= 1


def test_single_process_reductions_are_identity():
    assert replicas.reduce_max(3.5) == 3.5
    assert replicas.reduce_sum(2.0) == 2.0


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0][2] == [0, 2, 4, 6, 8, 10] and res[1][2] == [1, 3, 5, 7, 9]
    assert res[0][3] == res[1][3] == 20.0          # max over ranks
    assert res[0][4] == res[1][4] == 11.0          # every job counted once
