"""Probabilistic front end (lsim_fee_prob: the beam search of
get_adc_values_average_noise_vmap, fee_jax.py:386-461, and the reductions
of get_average_hit_values, :463-480) against the oracle, which restates it
in float32 numpy.

Tolerances: charges (the expected charge of a hit read at each tick) are
differences of cumulative sums, compared relative to each row's largest
|charge|; probabilities exp(log_prob) are compared absolutely; log
probabilities are compared in absolute log units above -5 and relative to
|log_prob| down to -20: below that float32 cancellation in
log(Phi(a) - Phi(b)) dominates both implementations (observed: 6e-5 above
-5, relative 1.7e-3 down to -20, probabilities within 1e-5).
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_common import small_params

pytestmark = pytest.mark.gpu

CHARGE_RTOL = 1e-5
PROB_ATOL = 5e-5
LOGP_ATOL = 5e-4       # for log_prob > -5
LOGP_RTOL = 5e-3       # relative to |log_prob|, for log_prob > -20
RED_ATOL = 1e-4        # lambda; expected tick and ADC relative 1e-3


@pytest.fixture(scope="module")
def case():
    from larndsim_gb300 import workloads
    from oracle import reference_np as R
    p = small_params(n_neighbors=1, RESET_NOISE_CHARGE=900)
    tmpl = R.load_lut_templates(workloads.synthetic_response(seed=0, nx=25, ny=25), p)
    tracks, fields = workloads.muon_event(seed=7, n_tracks=4)
    w, u = R.simulate_wfs(p, tmpl, tracks, fields, history={})
    w = np.concatenate([np.zeros((3, w.shape[1]), np.float32), w[u >= 0][:40]])
    lo, qo = R.get_adc_values_average_noise(p, w)
    return p, w, lo, qo


def test_beam_search_matches_oracle(cuda, case):
    from larndsim_gb300 import sim
    p, w, lo, qo = case
    lg, qg = sim.get_adc_values_average_noise_vmap(p, torch.from_numpy(w).cuda())
    lg, qg = lg.cpu().numpy(), qg.cpu().numpy()
    assert lg.shape == lo.shape == (w.shape[0], int(p.MAX_ADC_VALUES), w.shape[1] - 1)
    scale = np.maximum(np.abs(qo).max(axis=2, keepdims=True), 1.0)
    assert (np.abs(qg - qo) / scale).max() <= CHARGE_RTOL
    assert np.abs(np.exp(lg.astype(np.float64)) - np.exp(lo.astype(np.float64))).max() <= PROB_ATOL
    m = lo > -5
    assert m.sum() > 500
    assert np.abs(lg - lo)[m].max() <= LOGP_ATOL
    m = lo > -20
    assert m.sum() > 2000
    assert (np.abs(lg - lo)[m] / np.abs(lo[m]).clip(min=1.0)).max() <= LOGP_RTOL


def test_global_stop_blanks_the_same_steps(cuda, case):
    """Steps after the batch's last active one hold -1000 and 0 exactly."""
    from larndsim_gb300 import sim
    p, w, lo, qo = case
    lg, qg = sim.get_adc_values_average_noise_vmap(p, torch.from_numpy(w).cuda())
    lg, qg = lg.cpu().numpy(), qg.cpu().numpy()
    dead_o = np.all(lo == -1000, axis=(0, 2)) & np.all(qo == 0, axis=(0, 2))
    dead_g = np.all(lg == -1000, axis=(0, 2)) & np.all(qg == 0, axis=(0, 2))
    np.testing.assert_array_equal(dead_g, dead_o)
    assert dead_o.any() and not dead_o[0]


def test_fused_reductions_match(cuda, case):
    from larndsim_gb300 import sim
    from oracle import reference_np as R
    p, w, lo, qo = case
    eto, eao, lamo = R.get_average_hit_values(np.exp(lo), R.digitize(p, qo))
    etg, eag, lamg = (t.cpu().numpy() for t in sim.average_hit_values(p, torch.from_numpy(w).cuda()))
    assert np.abs(lamg - lamo).max() <= RED_ATOL
    on = lamo > 1e-3
    assert on.sum() > 20
    assert (np.abs(etg - eto)[on] / np.maximum(np.abs(eto[on]), 1)).max() <= 1e-3
    assert (np.abs(eag - eao)[on] / np.maximum(np.abs(eao[on]), 1)).max() <= 1e-3
    # fused and unfused GPU paths agree
    lg, qg = sim.get_adc_values_average_noise_vmap(p, torch.from_numpy(w).cuda())
    from larndsim_gb300.fee import digitize
    et2, ea2, lam2 = sim.get_average_hit_values(torch.exp(lg), digitize(p, qg))
    np.testing.assert_allclose(lam2.cpu().numpy(), lamg, rtol=1e-4, atol=1e-6)


def test_pixel_coordinates_and_strategy(cuda):
    from larndsim_gb300 import sim, strategies, workloads
    from oracle import reference_np as R
    p = small_params(n_neighbors=1, RESET_NOISE_CHARGE=900)
    ids = np.array([-1, 0, 5, 139, 140 * 280 - 1, 140 * 280, 140 * 280 * 2 + 77, 140 * 280 * 2 * 3 + 1234],
                   dtype=np.int32)
    x, y, plane, event = (t.cpu().numpy() for t in sim.pixel_coordinates(p, ids))
    px, py, pl, ev = R.id2pixel(p, ids)
    # the fused form XLA compiles get_pixel_coordinates to (pinned by the
    # reference's committed outputs): fma(p, pitch, border) + pitch / 2
    b = np.asarray(p.tpc_borders, np.float32)
    f32 = np.float32
    for got, pix, ax in ((x, px, 0), (y, py, 1)):
        exp = ((pix.astype(np.float64) * f32(p.pixel_pitch) + b[pl, ax, 0]).astype(f32) + f32(p.pixel_pitch / 2))
        np.testing.assert_array_equal(got.view(np.uint32), exp.astype(f32).view(np.uint32))
    np.testing.assert_array_equal(event, ev)
    np.testing.assert_array_equal(plane, pl)
    tmpl, p = sim.load_lut(workloads.synthetic_response(seed=0, nx=25, ny=25), p)
    tracks, fields = workloads.muon_event(seed=2, n_tracks=1)
    out = strategies.LUTProbabilisticSimulation(tmpl).predict(p, tracks, fields, None)
    n = out["unique_pixels"].shape[0]
    assert n % 128 == 0 and out["adcs_distrib"].shape == (n, int(p.MAX_ADC_VALUES), out["wfs"].shape[1] - 1)
    assert out["hit_prob"].shape == out["adcs_distrib"].shape and out["pixel_plane"].shape == (n,)
    assert torch.isfinite(out["hit_prob"]).all()
