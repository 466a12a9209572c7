"""The N > 1 path of bench.py: independent replicas, the rate aggregated as the units of all
ranks over the slowest rank's time, over a world_size-2 gloo group on CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = [10.0, 25.0][rank]
    units = [1000, 1000][rank]
    value, ms_max = bench.aggregate(units, ms, steps=4, dist=dist)
    dist.barrier()
    q.put((rank, value, ms_max))
    dist.destroy_process_group()


def test_two_replicas_aggregate_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms_max in out:
        assert ms_max == 25.0
        assert value == pytest.approx(2000 * 4 / 0.025)
