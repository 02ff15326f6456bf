"""The multi-GPU form is replicas: each rank steps its own batch and the bench
takes the slowest rank's timed region. Checked here with two gloo ranks on the
CPU (no GPU): every rank sees the maximum, and the whole-job rate counts all
ranks' cell-updates over it."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(1.0 + rank)          # rank 1 is the slower
    dist.barrier()
    out[rank] = (t, bench.whole_job_rate(1000, 10, world, t))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.0
    assert res[0][1] == res[1][1] == 1000 * 10 * 2 / 2.0
