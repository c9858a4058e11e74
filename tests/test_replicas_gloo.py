"""Multi-GPU path is replicas only: each rank runs its own volume (or its share of a
batch) and the job time is the slowest rank's.  Checked with gloo ranks on the CPU:
the max-over-ranks timing, the whole-job throughput, and the host side of a rank's
work (the seeded workload each replica builds, and the batch partition every rank
computes on its own)."""
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


def _partition_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import numpy as np
    import torch
    import bench
    from pyvoxeldosimetry_gb300.batch import partition_volumes
    rng = np.random.default_rng(3)        # the bench's seeded uneven batch shapes
    shapes = [(int(rng.integers(96, 321)), int(rng.integers(96, 321)), int(rng.integers(96, 257)))
              for _ in range(64)]
    mine = partition_volumes(shapes, world)[rank]
    # every rank's view of every rank's share, gathered: the assignment must agree
    objs = [None] * world
    dist.all_gather_object(objs, (rank, mine, partition_volumes(shapes, world)))
    # the replica workload's host side: the seeded phantom and its byte model are the same on every rank
    wl = bench.WORKLOADS["sphere128_y90"]
    act, rho = bench.make_inputs(wl)
    digest = torch.tensor([float(act.astype(np.float64).sum()),
                           float(bench.byte_model(wl["shape"], (15, 15, 15), 1, False)["_per_step"])],
                          dtype=torch.float64)
    ref = digest.clone()
    dist.broadcast(ref, 0)
    q.put((rank, objs, bool(torch.equal(digest, ref)), [shapes[i] for i in mine]))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_batch_partition_and_replica_workload(world):
    import numpy as np
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_partition_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
        assert p.exitcode == 0
    res = sorted((q.get(timeout=10) for _ in range(world)), key=lambda x: x[0])
    shares = [r[1][r[0]][1] for r in res]
    assert sorted(i for sh in shares for i in sh) == list(range(64))          # disjoint and complete
    for _, objs, same_workload, _ in res:
        assert same_workload
        for _, mine, full in objs:
            assert full == res[0][1][0][2]                                       # every rank computed the same split
    loads = [sum(int(np.prod(s)) for s in r[3]) for r in res]
    assert max(loads) <= 1.05 * min(loads)                                     # balanced to 5 %


def test_partition_edge_cases():
    from pyvoxeldosimetry_gb300.batch import partition_volumes
    assert partition_volumes([], 2) == [[], []]
    assert partition_volumes([(2, 2, 2)], 3) == [[0], [], []]
    assert partition_volumes([(4, 4, 4), (2, 2, 2), (2, 2, 2), (2, 2, 2)], 2) == [[0], [1, 2, 3]]
    with pytest.raises(ValueError):
        partition_volumes([(2, 2, 2)], 0)
