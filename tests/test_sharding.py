"""Batches spread over ranks (one GPU per rank), tested on the CPU.

Checks:
* The largest-first assignment partitions the scenes.
* It keeps every rank within the 4/3 balance bound.
* Its shards reassemble the batch exactly.
* A two-rank gloo run in which each rank steps only its own scenes (with the
  CPU oracle standing in for the GPU) gives every scene the bits of a
  one-process run: scenes do not interact, so the path needs no
  communication.
* Only the timing is combined, by max over ranks, with units summed over
  ranks.
"""
import os
import socket
import sys

import numpy as np
import pytest

from simplefluid_gb300 import SPHParameters, assign_scenes, batch_cubes, shard_batch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("nranks", [1, 2, 3, 4, 8])
def test_assignment_partitions_and_balances(nranks):
    counts = np.random.default_rng(nranks).integers(2000, 65536, size=256)
    parts = assign_scenes(counts, nranks)
    assert len(parts) == nranks
    allp = np.sort(np.concatenate(parts))
    assert np.array_equal(allp, np.arange(256))
    loads = np.array([counts[p].sum() for p in parts])
    best = max(counts.sum() / nranks, counts.max())
    assert loads.max() <= 4.0 / 3.0 * best


def test_more_ranks_than_scenes():
    parts = assign_scenes([5, 3], 4)
    assert sorted(len(p) for p in parts) == [0, 0, 1, 1]


def test_shards_reassemble_the_batch(lib):
    base = SPHParameters(particleRadius=0.01, kernelRadius=0.04)
    params, counts, pos = batch_cubes(3, 9, base)
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    seen = {}
    for r in range(3):
        p, c, x, mine = shard_batch(params, counts, pos, r, 3)
        o = np.concatenate([[0], np.cumsum(c)]).astype(np.int64)
        for k, s in enumerate(mine):
            assert p[k].viscosity == params[s].viscosity
            assert np.array_equal(x[o[k]:o[k + 1]], pos[off[s]:off[s + 1]])
            seen[int(s)] = r
    assert sorted(seen) == list(range(9))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _scene_steps(params_c, x, steps):
    from oracle import oracle as O
    st = O.State(x)
    st.step(params_c, steps)
    return st.original_order()[0]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import time

    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    base = SPHParameters(particleRadius=0.02, kernelRadius=0.08)
    params, counts, pos = batch_cubes(11, 5, base)
    p, c, x, mine = shard_batch(params, counts, pos, rank, world)
    o = np.concatenate([[0], np.cumsum(c)]).astype(np.int64)
    t0 = time.perf_counter()
    res = {int(s): _scene_steps(p[k], x[o[k]:o[k + 1]], 2) for k, s in enumerate(mine)}
    t, units = bench.aggregate_over_ranks(dist, time.perf_counter() - t0, int(c.sum()) * 2)
    out.put((rank, res, t, units))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_batch_gloo_two_ranks(oracle):
    torch = pytest.importorskip("torch")
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=300) for _ in range(2)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    base = SPHParameters(particleRadius=0.02, kernelRadius=0.08)
    params, counts, pos = batch_cubes(11, 5, base)
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    merged = {}
    for rank, res, t, units in got:
        assert units == int(counts.sum()) * 2  # all ranks' updates
        merged.update(res)
    assert sorted(merged) == list(range(5))
    assert got[0][2] == got[1][2]  # the same (slowest) time on every rank
    for s in range(5):
        ref = _scene_steps(params[s], pos[off[s]:off[s + 1]], 2)
        assert np.array_equal(merged[s].view(np.uint32), ref.view(np.uint32))
