"""Host-side logic of the N-replica benchmark, on CPU with gloo (world size 2).

bench.py runs one independent replica per GPU (the step does not shard); the
job time is the max over ranks and the value is the whole-job throughput.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    w, r, lr = bench.dist_setup()
    ms = 10.0 * (rank + 1)  # rank 1 is the slower replica
    t = bench.max_over_ranks(ms, "cpu")
    v = bench.replica_value(w, 5, t)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, w, r, t, v))


def test_replica_aggregation_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, w, r, t, v in out:
        assert w == 2 and r == rank
        assert t == pytest.approx(20.0)
        assert v == pytest.approx(2 * 2048 * 2048 * 5 / 0.020 / 1e6)
