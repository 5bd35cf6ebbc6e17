"""Event sharding across ranks and the per-step gradient reduction.

Events are independent in the reference (the event id is packed into the
pixel id, detsim_jax.py:241-242), so a batch splits by whole events with no
data exchange; a fit step then sums its [loss, gradient] vector across ranks
once.  ``shard_events`` assigns events greedily by segment count (largest
first, to the least-loaded rank) and relabels each shard's events to the
local namespace 0..k-1 the reference requires (detsim_jax.py:117-152).
"""

from __future__ import annotations

import numpy as np


def shard_events(tracks, fields, rank: int, world: int):
    """Rows of ``tracks`` owned by ``rank``, event ids relabelled 0..k-1.

    Returns (rows, global_event_ids).  Padding rows (eventID -1) are dropped.
    """
    col = tuple(fields).index("eventID")
    ev = np.asarray(tracks[:, col]).astype(np.int64)
    valid = ev >= 0
    ids, counts = np.unique(ev[valid], return_counts=True)
    load = np.zeros(world, np.int64)
    owner = {}
    for i in np.argsort(-counts, kind="stable"):
        r = int(np.argmin(load))
        owner[int(ids[i])] = r
        load[r] += counts[i]
    mine = np.array(sorted(e for e, r in owner.items() if r == rank), dtype=np.int64)
    keep = valid & np.isin(ev, mine)
    rows = np.array(tracks[keep], copy=True)
    rows[:, col] = np.searchsorted(mine, ev[keep]).astype(rows.dtype)
    return rows, mine


def allreduce_result(result, group=None):
    """Sum a [loss, grad...] tensor over the ranks of ``group`` in place."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(result, op=dist.ReduceOp.SUM, group=group)
    return result
