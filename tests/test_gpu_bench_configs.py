"""Parity on the measured configurations themselves, not only on small cases.

* Batched forward (64 events, segment counts log-uniform in [1k, 50k],
  n = 4, L = 150, the full 100x45x45x1950 template bank): the whole batch
  runs through the CUDA path in one call, exactly as the benchmark step
  does; the four smallest events and one of the largest are then simulated
  alone by the oracle (events are independent: the event id is only packed
  into the pixel id, detsim_jax.py:241-242) and compared row for row:
  unique pixels identical, waveforms within 1e-5 of each row's largest
  value, front-end crossing ticks identical except near-threshold
  crossings (fraction reported and bounded), ADCs within 1e-5 where the
  ticks agree.
* Gradient (a 5k-segment event at n = 4 on the full bank, prediction at
  parameters perturbed by N(0, 5 %)): the CUDA loss gradient against the
  float64 vector-Jacobian product of the frozen-decision oracle at the
  GPU's own residuals, 1e-4 relative per parameter (fit_params.py:704-731).
* Large event (500k segments around 40 sub-tracks): clusters of 5x5
  pixels sampled over the event, each compared with the oracle run on only
  the segments that can reach it (a pixel receives charge only from
  segments whose principal pixel lies within max(n, 1) pixels of it,
  sim_jax.py:427-450).
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_common import ADC_RTOL, WFS_RTOL, compare_fee, compare_wfs

pytestmark = pytest.mark.gpu

MAX_TICK_MISMATCH = 5e-3     # fraction of hit slots whose crossing tick may differ (near-threshold crossings)


@pytest.fixture(scope="module")
def bank(cuda):
    """n = 4, L = 150 nominal parameters and the full template bank, built
    on the GPU (its builder is compared with the oracle's load_lut in the
    forward tests) with a host copy for the oracle."""
    from larndsim_gb300 import consts, sim, workloads
    p = consts.Params(number_pix_neighbors=4, signal_length=150, RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0)
    tmpl_gpu, p = sim.load_lut(workloads.synthetic_response(seed=0), p)
    return p, tmpl_gpu, tmpl_gpu.cpu().numpy()


def _rows_of_event(p, wfs, unique, event):
    """Valid rows of one event of a batch, with their pixel ids re-packed
    for event 0 (the id an event simulated alone gets)."""
    from oracle import reference_np as R
    u = unique.cpu().numpy()
    px, py, plane, ev = R.id2pixel(p, np.maximum(u, 0))
    sel = (u >= 0) & (ev == event)
    idx = torch.from_numpy(np.nonzero(sel)[0]).to(wfs.device)
    return wfs.index_select(0, idx).cpu().numpy(), R.pixel2id(p, px[sel], py[sel], plane[sel], 0)


def _fee_grids(p, rows):
    from larndsim_gb300 import sim
    from oracle import reference_np as R
    integral, ticks = sim.get_adc_values(p, torch.from_numpy(rows).cuda())
    return R.digitize(p, integral.cpu().numpy()), ticks.cpu().numpy()


def test_batched_benchmark_events_match_oracle(bank):
    from larndsim_gb300 import sim, workloads
    from oracle import reference_np as R
    p, tmpl_gpu, tmpl = bank
    tracks, fields = workloads.batched_events(seed=0)
    col = fields.index("eventID")
    ev = tracks[:, col].astype(np.int64)
    counts = np.bincount(ev)
    assert counts.size == 64 and tracks.shape[0] > 700_000
    sim.reset_size_history()
    wfs, unique = sim.simulate_wfs(p, tmpl_gpu, tracks, fields)
    order = np.argsort(counts, kind="stable")
    chosen = list(order[:4]) + [int(order[-4])]          # the four smallest and one of the largest
    slots = mism = 0
    worst_w = worst_a = 0.0
    for e in chosen:
        rows_g, pids_g = _rows_of_event(p, wfs, unique, e)
        one = tracks[ev == e].copy()
        one[:, col] = 0
        wo, uo = R.simulate_wfs(p, tmpl, one, fields, history={})
        v = uo >= 0
        assert np.array_equal(pids_g, uo[v]), f"event {e}: unique pixels differ"
        assert pids_g.size > 100
        err = compare_wfs(rows_g, pids_g, wo[v], uo[v])
        assert err < WFS_RTOL, (e, err)
        adc_g, ticks_g = _fee_grids(p, rows_g)
        integral_o, ticks_o = R.get_adc_values(p, wo[v])
        frac, aerr = compare_fee(adc_g, ticks_g, R.digitize(p, integral_o), ticks_o)
        assert frac <= MAX_TICK_MISMATCH and aerr < ADC_RTOL, (e, frac, aerr)
        slots += ticks_g.size
        mism += int(round(frac * ticks_g.size))
        worst_w, worst_a = max(worst_w, err), max(worst_a, aerr)
    print(f"\nbatched benchmark events {chosen} ({int(counts[chosen].sum())} segments): waveforms within "
          f"{worst_w:.2e} of the row scale, ADC within {worst_a:.2e}, crossing ticks differing on "
          f"{mism} of {slots} hit slots ({mism / slots:.2e})")


def test_gradient_5k_segment_event_full_bank_vs_fp64(bank):
    from larndsim_gb300 import grad, workloads
    from oracle import grad64 as G
    p, tmpl_gpu, tmpl = bank
    tracks = workloads.mixed_event(np.random.default_rng(7), 5000, 0)
    fields = workloads.SEGMENT_FIELDS
    chain = grad.LUTChain(p, tmpl_gpu, tracks, fields)
    target = chain.target(p)
    rng = np.random.default_rng(1234)
    pp = p.replace(**{k: float(getattr(p, k)) * (1.0 + 0.05 * rng.standard_normal()) for k in grad.GRAD_PARAMS})
    loss, g = chain.loss_and_grad(pp, target)
    fr = G.Frozen(pp, tmpl, tracks, fields, target.pids.cpu().numpy(), target.adc.cpu().numpy())
    th = G.theta_dict(pp)
    adc, ticks, pids = chain.adc(pp)
    assert np.array_equal(pids.cpu().numpy(), fr.unique[fr.valid])
    assert pids.numel() > 500
    acc = ~fr.cond[fr.valid]
    assert np.array_equal(ticks.cpu().numpy()[acc], fr.idx[fr.valid][acc].astype(np.float32))
    L64 = G.loss64(fr, th)
    assert abs(loss - L64) <= 1e-3 * L64 + 1e-3
    assert g["vdrift"] == 0.0
    resid = 2.0 * (adc.cpu().numpy().astype(np.float64) - fr.tgt)
    g_ref = G.adjoint64(fr, th, g_adc=resid)
    sens = max(abs(g_ref[k] * th[k]) for k in g_ref)
    worst = 0.0
    for k in g_ref:
        err = abs(g[k] - g_ref[k])
        ok = err <= 1e-4 * abs(g_ref[k]) or err * abs(th[k]) <= 1e-6 * sens
        assert ok, (k, g[k], g_ref[k])
        if g_ref[k] != 0.0:
            worst = max(worst, err / abs(g_ref[k]))
    print(f"\n5k-segment gradient, {pids.numel()} pixels: largest relative deviation from the float64 "
          f"adjoint {worst:.2e}")


def test_large_event_sampled_pixels_match_oracle(bank):
    from larndsim_gb300 import sim, workloads
    from oracle import reference_np as R
    p, tmpl_gpu, tmpl = bank
    tracks, fields = workloads.large_shower_event(seed=0, n_segments=500_000, n_subtracks=40)
    sim.reset_size_history()
    wfs, unique = sim.simulate_wfs(p, tmpl_gpu, tracks, fields)
    u = unique.cpu().numpy()
    valid = np.nonzero(u >= 0)[0]
    assert valid.size > 10_000
    sh = R.shift_tracks(p, tracks, fields)
    xs, ys = sh[:, fields.index("x")], sh[:, fields.index("y")]
    assert np.all(np.sign(sh[:, fields.index("z")]) == np.sign(sh[0, fields.index("z")])), "one TPC"
    px, py, plane, _ = R.id2pixel(p, u[valid])
    cx, cy = R.get_pixel_coordinates(p, px, py, plane).T
    pitch = float(p.pixel_pitch)
    reach = (int(p.number_pix_neighbors) + 2) * pitch + 2.5 * pitch      # block half-width + neighbourhood
    rng = np.random.default_rng(11)
    n_clusters = checked = segs = 0
    worst = 0.0
    for i in rng.permutation(valid.size)[:200]:
        if n_clusters == 12:
            break
        x0, y0 = cx[i], cy[i]
        sel = (np.abs(xs - x0) <= reach) & (np.abs(ys - y0) <= reach)
        if sel.sum() > 8000:
            continue                     # keep the oracle's share of the test bounded
        block = (np.abs(px - px[i]) <= 2) & (np.abs(py - py[i]) <= 2)
        wo, uo = R.simulate_wfs(p, tmpl, tracks[sel], fields, history={})
        pos = np.searchsorted(uo, u[valid][block])
        assert np.all(uo[np.minimum(pos, uo.size - 1)] == u[valid][block]), "block pixel missing from the oracle"
        opx, opy, _, _ = R.id2pixel(p, np.maximum(uo, 0))
        in_block = (uo >= 0) & (np.abs(opx - px[i]) <= 2) & (np.abs(opy - py[i]) <= 2)
        assert int(in_block.sum()) == int(block.sum()), "the oracle has block pixels the GPU has not"
        rows_g = wfs.index_select(0, torch.from_numpy(valid[block]).to(wfs.device)).cpu().numpy()
        err = compare_wfs(rows_g, u[valid][block], wo[pos], uo[pos])
        assert err < WFS_RTOL, (i, err)
        worst = max(worst, err)
        n_clusters += 1
        checked += int(block.sum())
        segs += int(sel.sum())
    assert n_clusters >= 8 and checked >= 200
    print(f"\nlarge event, {valid.size} pixels: {checked} pixels in {n_clusters} 5x5 clusters ({segs} segments "
          f"through the oracle) within {worst:.2e} of the row scale")
