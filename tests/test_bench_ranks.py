"""CPU: the multi-process bookkeeping of bench.py (one process per GPU,
replicas of the transform with no collective on the data path) with two
gloo ranks: rank / world from the launcher's environment, the slowest rank's
time, the whole-job value, and the reference arm's rank-0-only rule."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    w, r, local = bench.dist_setup(None)
    dist.init_process_group("gloo", rank=r, world_size=w)
    ms = bench.max_over_ranks(10.0 + 5.0 * r, w)  # rank 1 is the slow one
    value = bench.job_value(4096, 65536, w, ms / 4)
    dist.barrier()
    dist.destroy_process_group()
    out.put((r, w, local, ms, value))


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[3] == 15.0 for r in res)  # max over ranks, the same on both
    import bench  # noqa: E402  (imported after the ranks: the parent needs no process group)
    assert res[0][4] == pytest.approx(bench.job_value(4096, 65536, 2, 15.0 / 4))
    assert res[0][4] == pytest.approx(2 * bench.job_value(4096, 65536, 1, 15.0 / 4))


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        n = 4096
        steps = 1
        warmup = 1
    assert bench.run_reference(A()) is None  # returns before any work or output
