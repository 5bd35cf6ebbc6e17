"""Size-independent properties of the batched path (events are independent
in the reference: the event id is packed into the pixel id,
detsim_jax.py:241-242):

* the waveform rows of one event in a batch are bit-identical to the rows
  of the same event simulated alone;
* the loss and gradient of a batch equal the sums over event shards (the
  multi-GPU decomposition), and a large shower event runs end to end with a
  deterministic, finite result.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_common import small_params

pytestmark = pytest.mark.gpu


def _batch(seed=21):
    from larndsim_gb300 import workloads
    parts, fields = [], None
    for e, kind in enumerate(("muon", "shower", "muon", "shower")):
        if kind == "muon":
            t, fields = workloads.muon_event(seed=seed + e, n_tracks=3, event_id=e)
        else:
            t, fields = workloads.shower_event(seed=seed + e, n_segments=400, event_id=e)
        parts.append(t)
    return np.concatenate(parts), fields


def test_batch_rows_equal_single_event_rows(cuda):
    from larndsim_gb300 import sim, workloads
    from oracle import reference_np as R
    p = small_params(n_neighbors=2)
    resp = workloads.synthetic_response(seed=0, nx=25, ny=25)
    tmpl = torch.from_numpy(R.load_lut_templates(resp, p)).cuda()
    tracks, fields = _batch()
    col = fields.index("eventID")
    sim.reset_size_history()
    wfs, unique = sim.simulate_wfs(p, tmpl, tracks, fields)
    wfs, unique = wfs.cpu().numpy(), unique.cpu().numpy()
    ev_b = np.where(unique >= 0, R.id2pixel(p, np.maximum(unique, 0))[3], -9)
    checked = 0
    for e in range(4):
        one = tracks[tracks[:, col] == e].copy()
        one[:, col] = 0
        sim.reset_size_history()
        w1, u1 = sim.simulate_wfs(p, tmpl, one, fields)
        w1, u1 = w1.cpu().numpy(), u1.cpu().numpy()
        rows_b = wfs[(ev_b == e)]
        rows_1 = w1[u1 >= 0]
        assert rows_b.shape == rows_1.shape and rows_1.shape[0] > 10
        np.testing.assert_array_equal(rows_b, rows_1)
        checked += rows_1.shape[0]
    assert checked == int((unique >= 0).sum())


def _loss_grad(p, tmpl, tracks, fields):
    from larndsim_gb300 import grad
    chain = grad.LUTChain(p, tmpl, tracks, fields)
    target = chain.target(p)
    pp = p.replace(Ab=0.83, kb=0.05, eField=0.52, lifetime=2000.0, long_diff=5e-6, tran_diff=9e-6, lArDensity=1.39)
    loss, g = chain.loss_and_grad(pp, target)
    return loss, np.array([g[k] for k in grad.GRAD_PARAMS], dtype=np.float64)


def test_event_shards_sum_to_the_batch(cuda):
    from larndsim_gb300 import parallel, workloads
    from oracle import reference_np as R
    p = small_params(n_neighbors=2)
    resp = workloads.synthetic_response(seed=0, nx=25, ny=25)
    tmpl = torch.from_numpy(R.load_lut_templates(resp, p)).cuda()
    tracks, fields = _batch(seed=40)
    loss, g = _loss_grad(p, tmpl, tracks, fields)
    loss_s, g_s = 0.0, np.zeros_like(g)
    for rank in range(2):
        rows, mine = parallel.shard_events(tracks, fields, rank, 2)
        assert len(mine) == 2
        l, gg = _loss_grad(p, tmpl, rows, fields)
        loss_s += l
        g_s += gg
    assert loss > 0
    assert abs(loss_s - loss) <= 1e-6 * loss
    np.testing.assert_allclose(g_s, g, rtol=1e-5, atol=1e-6 * np.abs(g).max())


def test_large_shower_event_runs_deterministically(cuda):
    from larndsim_gb300 import consts, grad, sim, workloads
    p = consts.Params(number_pix_neighbors=4, RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0)
    tmpl, p = sim.load_lut(workloads.synthetic_response(seed=0), p)
    tracks, fields = workloads.large_shower_event(seed=1, n_segments=100_000, n_subtracks=10)
    chain = grad.LUTChain(p, tmpl, tracks, fields)
    target = chain.target(p)
    pp = p.replace(eField=0.52, tran_diff=9e-6)
    a = chain.loss_and_grad(pp, target)
    b = chain.loss_and_grad(pp, target)
    assert a == b
    assert a[0] > 0 and np.isfinite(a[0]) and all(np.isfinite(v) for v in a[1].values())
    assert chain._stage.n_valid > 1000


def test_launch_shapes_do_not_change_results(cuda):
    """Every launch shape the autotuner may pick gives bit-identical loss
    and gradient."""
    from larndsim_gb300 import grad, tune, workloads
    from oracle import reference_np as R
    p = small_params(n_neighbors=2)
    tmpl = torch.from_numpy(R.load_lut_templates(workloads.synthetic_response(seed=0, nx=25, ny=25), p)).cuda()
    tracks, fields = _batch(seed=60)
    chain = grad.LUTChain(p, tmpl, tracks, fields)
    target = chain.target(p)
    pp = p.replace(eField=0.52, lifetime=2000.0, tran_diff=9e-6)
    results = set()
    try:
        for cfg in tune.DEFAULT_CANDIDATES:
            tune.set_tuning(cfg)
            loss, g = chain.loss_and_grad(pp, target)
            results.add((loss,) + tuple(g.values()))
        cfg, times = tune.autotune(lambda: chain.loss_and_grad_device(pp, target), reps=1, warmup=0)
        assert set(times) == {tuple(c[k] for k in tune.FIELDS) for c in tune.DEFAULT_CANDIDATES}
        assert cfg in tune.DEFAULT_CANDIDATES
    finally:
        tune.set_tuning(None)
    assert len(results) == 1


def test_parametrised_batch_rows_equal_single_event_rows(cuda):
    """Parametrised mode (number_pix_neighbors = 0, Monte-Carlo diffusion
    draws supplied per segment): the same batch invariance."""
    from larndsim_gb300 import sim
    from oracle import reference_np as R
    p = small_params(n_neighbors=0, mc_diff=True)
    tracks, fields = _batch(seed=80)
    col = fields.index("eventID")
    offsets = np.random.default_rng(3).standard_normal((tracks.shape[0], 3)).astype(np.float32)
    sim.reset_size_history()
    wfs, unique = sim.simulate_parametrized_wfs(p, tracks, fields, offsets=torch.from_numpy(offsets).cuda())
    wfs, unique = wfs.cpu().numpy(), unique.cpu().numpy()
    ev_b = np.where(unique >= 0, R.id2pixel(p, np.maximum(unique, 0))[3], -9)
    for e in range(4):
        m = tracks[:, col] == e
        one = tracks[m].copy()
        one[:, col] = 0
        sim.reset_size_history()
        w1, u1 = sim.simulate_parametrized_wfs(p, one, fields, offsets=torch.from_numpy(offsets[m]).cuda())
        w1, u1 = w1.cpu().numpy(), u1.cpu().numpy()
        rows_1 = w1[u1 >= 0]
        assert rows_1.shape[0] > 10
        np.testing.assert_array_equal(wfs[ev_b == e], rows_1)
