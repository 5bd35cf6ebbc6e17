"""LUT-mode forward parity: simulate_wfs / simulate_stochastic on the GPU vs
the CPU oracle (reference sim_jax.py:689-769), on seeded inputs."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_common import ADC_RTOL, WFS_RTOL, compare_fee, compare_wfs, small_params

pytestmark = pytest.mark.gpu


def _run(params, tmpl, tracks, fields):
    from larndsim_gb300 import sim
    from oracle import reference_np as R
    sim.reset_size_history()
    wfs, unique = sim.simulate_wfs(params, torch.from_numpy(tmpl).cuda(), tracks, fields)
    wfs_o, unique_o = R.simulate_wfs(params, tmpl, tracks, fields, history={})
    return wfs.cpu().numpy(), unique.cpu().numpy(), wfs_o, unique_o


@pytest.fixture(scope="module")
def small_lut():
    from larndsim_gb300 import workloads
    from oracle import reference_np as R
    p = small_params()
    resp = workloads.synthetic_response(seed=0, nx=15, ny=15)
    return p, R.load_lut_templates(resp, p)


def test_muon_waveforms_small(cuda, small_lut):
    from larndsim_gb300 import workloads
    p, tmpl = small_lut
    tracks, fields = workloads.muon_event(seed=1)
    w, u, wo, uo = _run(p, tmpl, tracks, fields)
    assert (u >= 0).sum() > 100
    assert compare_wfs(w, u, wo, uo) < WFS_RTOL
    assert np.all(w[u < 0] == 0)


def test_fee_on_same_waveforms(cuda, small_lut):
    from larndsim_gb300 import sim, workloads
    from oracle import reference_np as R
    p, tmpl = small_lut
    tracks, fields = workloads.muon_event(seed=2)
    w, u, wo, uo = _run(p, tmpl, tracks, fields)
    integral, ticks = sim.get_adc_values(p, torch.from_numpy(w).cuda())
    ai, ti = R.get_adc_values(p, w)
    frac, err = compare_fee(integral.cpu().numpy(), ticks.cpu().numpy(), ai, ti, p)
    assert frac < 0.005, frac
    assert err < ADC_RTOL, err
    # raw integrals: within a few float32 ulps of the row's cumulative charge
    same = np.cumprod(ticks.cpu().numpy() == ti, axis=1).astype(bool)
    cmax = np.abs(np.cumsum(w * np.float32(p.t_sampling), axis=1)).max(axis=1, keepdims=True)
    assert np.all(np.abs(integral.cpu().numpy() - ai)[same] <= (4e-6 * cmax + 1e-3).repeat(ai.shape[1], 1)[same])
    assert (ti < 1998).sum() > 50        # the case has real hits


def test_stochastic_outputs(cuda, small_lut):
    from larndsim_gb300 import sim, workloads
    from oracle import reference_np as R
    p, tmpl = small_lut
    tracks, fields = workloads.muon_event(seed=4)
    sim.reset_size_history()
    wfs, unique = sim.simulate_wfs(p, torch.from_numpy(tmpl).cuda(), tracks, fields)
    (adcs, x, y, z, ticks, hp, ev, pix), (ag, tg) = sim.simulate_stochastic(p, wfs, unique, 0, return_grids=True)
    ref = R.simulate_stochastic(p, wfs.cpu().numpy(), unique.cpu().numpy())
    frac, err = compare_fee(ag.cpu().numpy(), tg.cpu().numpy(), ref["grid_adcs"], ref["grid_ticks"])
    assert frac < 0.005 and err < ADC_RTOL
    if frac == 0:
        assert adcs.shape[0] == ref["nb_valid"]
        np.testing.assert_array_equal(pix.cpu().numpy(), ref["pixels"])
        np.testing.assert_array_equal(ev.cpu().numpy(), ref["event"])
        np.testing.assert_array_equal(ticks.cpu().numpy(), ref["ticks"])
        np.testing.assert_allclose(adcs.cpu().numpy(), ref["adcs"], rtol=ADC_RTOL)
        # pixel centres / hit z: fused forms agree with the oracle's plain
        # forms to within 2 ulp
        np.testing.assert_allclose(x.cpu().numpy(), ref["pixel_x"], rtol=3e-7, atol=3e-6)
        np.testing.assert_allclose(y.cpu().numpy(), ref["pixel_y"], rtol=3e-7, atol=3e-6)
        np.testing.assert_allclose(z.cpu().numpy(), ref["pixel_z"], rtol=3e-7, atol=3e-6)
        assert np.all(hp.cpu().numpy() == 1)


def test_edge_cases_padding_outside_and_events(cuda, small_lut):
    """eventID -1 padding rows, segments outside every TPC, segments just
    outside the pixel plane (principal pixel -1 with bins on pixel 0),
    several events, and a non-zero shift."""
    from larndsim_gb300 import workloads
    p, tmpl = small_lut
    a, fields = workloads.muon_event(seed=5, n_tracks=4, event_id=0)
    b, _ = workloads.muon_event(seed=6, n_tracks=3, event_id=1)
    col = {f: i for i, f in enumerate(fields)}
    edge = a[:6].copy()
    bx0 = np.float32(p.tpc_borders[0, 0, 0])
    for k, dx in enumerate([-0.019, -0.01, -0.001, 0.0005, 0.01, 0.03]):
        edge[k, col["x"]] = bx0 + np.float32(dx)
        edge[k, col["x_start"]] = edge[k, col["x"]]
        edge[k, col["x_end"]] = edge[k, col["x"]]
    out = a[:5].copy()
    out[:, col["z"]] = 0.0          # between the two TPCs: mask false
    tracks = np.concatenate([a, b, edge, out])
    tracks = workloads.pad_tracks(tracks, fields, tracks.shape[0] + 40)
    p2 = p.replace(shift_z=0.05, shift_x=-0.03)
    w, u, wo, uo = _run(p2, tmpl, tracks, fields)
    assert (u < -1).any() and (u == -1).any()
    assert compare_wfs(w, u, wo, uo) < WFS_RTOL


def test_empty_and_single_segment(cuda, small_lut):
    from larndsim_gb300 import workloads
    p, tmpl = small_lut
    tracks, fields = workloads.muon_event(seed=7, n_tracks=1)
    w, u, wo, uo = _run(p, tmpl, tracks[:1], fields)
    assert compare_wfs(w, u, wo, uo) < WFS_RTOL
    w, u, wo, uo = _run(p, tmpl, tracks[:0], fields)
    assert np.array_equal(u, uo) and w.shape == wo.shape


def test_no_neighbours_main_bins_spill(cuda):
    """number_pix_neighbors = 0: no neighbour parts, but a segment's main
    bins still land on the adjacent simulated pixels (dense shower)."""
    from larndsim_gb300 import workloads
    from oracle import reference_np as R
    p = small_params(n_neighbors=0)
    tmpl = R.load_lut_templates(workloads.synthetic_response(seed=0, nx=5, ny=5), p)
    tracks, fields = workloads.shower_event(seed=8, n_segments=600)
    w, u, wo, uo = _run(p, tmpl, tracks, fields)
    assert (u >= 0).sum() > 100
    assert compare_wfs(w, u, wo, uo) < WFS_RTOL


def test_recombination_models(cuda, small_lut):
    from larndsim_gb300 import consts, workloads
    p, tmpl = small_lut
    tracks, fields = workloads.shower_event(seed=8, n_segments=600)
    for mode in (consts.RecombinationMode.BOX, consts.RecombinationMode.ELLIPSOID):
        w, u, wo, uo = _run(p.replace(recombination_mode=mode), tmpl, tracks, fields)
        assert compare_wfs(w, u, wo, uo) < WFS_RTOL


def test_noise_with_supplied_normals(cuda, small_lut):
    from larndsim_gb300 import sim, workloads
    from oracle import reference_np as R
    p, tmpl = small_lut
    p = p.replace(RESET_NOISE_CHARGE=900, UNCORRELATED_NOISE_CHARGE=500)
    tracks, fields = workloads.muon_event(seed=9)
    w, u, wo, uo = _run(p, tmpl, tracks, fields)
    rng = np.random.default_rng(0)
    normals = rng.standard_normal((w.shape[0], 1 + 3 * p.MAX_ADC_VALUES)).astype(np.float32)
    integral, ticks = sim.get_adc_values(p, torch.from_numpy(w).cuda(), normals=normals)
    ai, ti = R.get_adc_values(p, w, normals)
    frac, err = compare_fee(integral.cpu().numpy(), ticks.cpu().numpy(), ai, ti, p)
    assert frac < 0.005 and err < ADC_RTOL


def test_c1_full_lut_n4(cuda):
    """c1: 12 muons, 45x45x1950 LUT, 100 templates built on the GPU, n=4."""
    from larndsim_gb300 import consts, sim, workloads
    from oracle import reference_np as R
    p = consts.Params(number_pix_neighbors=4, RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0)
    resp = workloads.synthetic_response(seed=0)
    tmpl_gpu, p = sim.load_lut(resp, p)
    tmpl = tmpl_gpu.cpu().numpy()
    # the template bank builder agrees with the oracle's load_lut on sampled rows
    sub = R.load_lut_templates(resp[:3, :2], p)
    np.testing.assert_allclose(tmpl[:, :3, :2], sub, rtol=2e-5, atol=2e-6 * np.abs(sub).max())
    tracks, fields = workloads.muon_event(seed=11)
    sim.reset_size_history()
    wfs, unique = sim.simulate_wfs(p, tmpl_gpu, tracks, fields)
    wo, uo = R.simulate_wfs(p, tmpl, tracks, fields, history={})
    assert compare_wfs(wfs.cpu().numpy(), unique.cpu().numpy(), wo, uo) < WFS_RTOL
