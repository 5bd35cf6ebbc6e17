"""Multi-rank host logic on CPU: event sharding and the per-step gradient
all-reduce, with world_size 2 over gloo (127.0.0.1)."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from larndsim_gb300 import parallel, workloads


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shards_cover_every_event_once():
    tracks, fields = workloads.batched_events(seed=3, n_events=9, min_segments=50, max_segments=400)
    tracks = workloads.pad_tracks(tracks, fields, tracks.shape[0] + 13)
    world = 3
    col = fields.index("eventID")
    seen, total = [], 0
    for r in range(world):
        rows, mine = parallel.shard_events(tracks, fields, r, world)
        assert set(np.unique(rows[:, col]).astype(int)) == set(range(len(mine)))
        seen += mine.tolist()
        total += rows.shape[0]
    assert sorted(seen) == list(range(9))
    assert total == int((tracks[:, col] >= 0).sum())


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    tracks, fields = workloads.batched_events(seed=4, n_events=5, min_segments=30, max_segments=100)
    rows, mine = parallel.shard_events(tracks, fields, rank, world)
    # a stand-in per-shard result: [loss, 8 grads] linear in the shard's rows
    res = torch.tensor([rows.shape[0]] + [float(rows[:, fields.index("dE")].sum())] * 8, dtype=torch.float64)
    parallel.allreduce_result(res)
    q.put((rank, res.numpy()))
    torch.distributed.destroy_process_group()


def test_gloo_world2_allreduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    tracks, fields = workloads.batched_events(seed=4, n_events=5, min_segments=30, max_segments=100)
    expect = np.array([tracks.shape[0]] + [float(tracks[:, fields.index("dE")].sum())] * 8)
    for r in (0, 1):
        np.testing.assert_allclose(out[r], expect, rtol=1e-6)


def test_allreduce_is_identity_without_group():
    t = torch.ones(9)
    assert parallel.allreduce_result(t) is t and float(t.sum()) == 9
