"""The bench's multi-process (replica) aggregation on CPU with gloo, world size 2."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 10.0 + 5.0 * rank  # rank 1 is the slower replica
    t, units = bench.aggregate_over_ranks(dist, local_ms, 1000 * (rank + 1))
    out.put((rank, t, units))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_gloo_two_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t, units in got:
        assert t == 15.0 and units == 3000  # max time over ranks, units summed
    import bench
    assert bench.aggregate_over_ranks(None, 7.0, 42) == (7.0, 42)
