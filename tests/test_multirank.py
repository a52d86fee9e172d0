"""The N > 1 path of bench.py on the CPU: two gloo ranks, each timing its
own replica; the job's time is the slowest rank's and the value counts the
work of both ranks (weak scaling, replicas)."""

import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, lr, w = bench.dist_env()
    assert (r, lr, w) == (rank, rank, world)
    ms = 1.0 + 2.0 * rank  # rank 1 is slower
    out[rank] = bench.max_over_ranks(ms, world, "cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_rank():
    port = 29500 + os.getpid() % 1000
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert out[0] == 3.0 and out[1] == 3.0
