"""Independent scenes of a batch spread over ranks, one GPU per rank.

Scenes never interact, so a batch shards with no data-path communication:
each rank steps its own scenes and only the timing is combined.  The
assignment is greedy largest-first by particle count (LPT), which keeps the
most loaded rank within 4/3 of the best possible balance.
"""
from __future__ import annotations

import numpy as np


def assign_scenes(counts, nranks: int) -> list:
    """Scene indices of each rank (ascending within a rank)."""
    counts = np.asarray(counts, np.int64)
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    order = np.argsort(-counts, kind="stable")
    loads = np.zeros(nranks, np.int64)
    parts = [[] for _ in range(nranks)]
    for s in order:
        r = int(np.argmin(loads))  # the first least-loaded rank
        parts[r].append(int(s))
        loads[r] += counts[s]
    return [np.array(sorted(p), np.int64) for p in parts]


def shard_batch(params, counts, pos, rank: int, nranks: int, vel=None):
    """This rank's part of a batch: (per-scene params, counts, positions[,
    velocities]) in scene order, and the global scene indices."""
    counts = np.asarray(counts, np.int64)
    off = np.concatenate([[0], np.cumsum(counts)])
    mine = assign_scenes(counts, nranks)[rank]
    sel = np.concatenate([np.arange(off[s], off[s + 1]) for s in mine]) if len(mine) else np.zeros(0, np.int64)
    p_mine = (type(params[0]) * len(mine))(*[params[s] for s in mine]) if len(mine) else None
    out = (p_mine, counts[mine].astype(np.uint32), np.ascontiguousarray(pos[sel]))
    if vel is not None:
        out = out + (np.ascontiguousarray(vel[sel]),)
    return out + (mine,)
