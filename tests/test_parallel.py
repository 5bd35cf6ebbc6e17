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


def _oracle_loss_grad(tracks, fields):
    """The float64 oracle's SSE-ADC loss and gradient of one set of events:
    target at nominal parameters, prediction at perturbed ones (the fit
    step's [loss, 8 gradients] vector)."""
    from larndsim_gb300 import consts
    from oracle import grad64 as G
    from oracle import reference_np as R
    p = consts.Params(number_pix_neighbors=1, RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0,
                      long_diff_template=consts.jax_linspace_f32(0.001, 10, 10))
    tmpl = R.load_lut_templates(workloads.synthetic_response(seed=0, nx=15, ny=15), p)
    w, u = R.simulate_wfs(p, tmpl, tracks, fields, history={})
    o = R.simulate_stochastic(p, w, u)
    v = u >= 0
    pp = p.replace(Ab=0.83, eField=0.52, lifetime=2000.0, tran_diff=9e-6)
    fr = G.Frozen(pp, tmpl, tracks, fields, u[v], o["grid_adcs"][v])
    th = G.theta_dict(pp)
    g = G.adjoint64(fr, th)
    return np.array([G.loss64(fr, th)] + [g[k] for k in G.GRAD_PARAMS])


def _oracle_events():
    parts, fields = [], None
    for e in range(4):
        t, fields = workloads.muon_event(seed=90 + e, n_tracks=2, event_id=e)
        parts.append(t)
    return np.concatenate(parts), fields


def _oracle_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    tracks, fields = _oracle_events()
    rows, mine = parallel.shard_events(tracks, fields, rank, world)
    res = torch.from_numpy(_oracle_loss_grad(rows, fields))
    parallel.allreduce_result(res)
    q.put((rank, res.numpy(), mine.tolist()))
    torch.distributed.destroy_process_group()


def test_gloo_world2_shard_oracle_results_sum_to_the_batch():
    """Each rank computes the oracle's loss and gradient on its own event
    shard; the all-reduced vector equals the whole batch's."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_oracle_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        r, v, mine = q.get(timeout=300)
        out[r] = (v, mine)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(out[0][1] + out[1][1]) == [0, 1, 2, 3] and out[0][1] and out[1][1]
    tracks, fields = _oracle_events()
    whole = _oracle_loss_grad(tracks, fields)
    assert whole[0] > 0 and np.abs(whole[1:]).max() > 0
    for r in (0, 1):
        np.testing.assert_allclose(out[r][0], whole, rtol=1e-9, atol=1e-12 * np.abs(whole).max())


def test_allreduce_is_identity_without_group():
    t = torch.ones(9)
    assert parallel.allreduce_result(t) is t and float(t.sum()) == 9
