"""Multi-GPU here is replicas only: independent slices per rank, no data-path
collective; the job's rate is all ranks' slices over the slowest rank's time.
This checks bench.py's rank aggregation with two gloo ranks on the CPU."""
import os
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    seconds = bench.reduce_max(1.0 + rank * 0.5)  # rank 1 is the slowest
    rate = bench.whole_job_rate(4, seconds, world)
    q.put((rank, seconds, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [1.5, 1.5]
    assert all(abs(o[2] - 8 / 1.5) < 1e-12 for o in out)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_max(2.5) == 2.5
    assert bench.whole_job_rate(3, 1.5, 1) == 2.0
