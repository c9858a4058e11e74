"""Multi-GPU path of bench.py is replicas only: each rank runs its own volume and
the job time is the slowest rank's.  Checked with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 10.0 * (rank + 1)                     # rank 1 is the slow one
    worst = bench.max_over_ranks(ms)
    value = bench.job_throughput(world, 1_000_000, 4, worst)
    q.put((rank, worst, value))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_value():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, worst, value in res:
        assert worst == pytest.approx(20.0)
        # two replicas x 1e6 voxels x 4 steps in 20 ms
        assert value == pytest.approx(2 * 1e6 * 4 / 0.020 / 1e9)


def test_single_process_is_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
