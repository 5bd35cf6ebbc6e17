"""Gradient of the parametrised mode (lsim_param_wfs_vjp through
sim.param_wfs_fn): a cotangent on the waveform rows pulled back to the 8
parameters, against the complex-step derivative of the float64 oracle
(oracle/grad64.py param_waveforms64) with the float32 forward's discrete
decisions frozen (pixels, t0 ticks, min(a, 1) branch), which is what
jax.grad of simulate_parametrized computes with the offsets held fixed.

Tolerance: 2e-3 relative on each parameter, or 1e-5 of the largest
|dL/dtheta * theta| (the float32 EMG expressions cancel in their window
differences)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_common import small_params

pytestmark = pytest.mark.gpu
RTOL = 2e-3


def _case(seed, n_tracks, shower=0):
    from larndsim_gb300 import workloads
    tracks, fields = workloads.muon_event(seed=seed, n_tracks=n_tracks)
    if shower:
        sh, _ = workloads.shower_event(seed=seed + 50, n_segments=shower)
        tracks = np.concatenate([tracks, sh])
    nrm = np.random.default_rng(seed).standard_normal((tracks.shape[0], 3)).astype(np.float32)
    return tracks, fields, nrm


@pytest.mark.parametrize("seed,n_tracks,shower", [(4, 2, 0), (6, 1, 300)])
def test_param_wfs_vjp_matches_complex_step(cuda, seed, n_tracks, shower):
    from larndsim_gb300 import grad, sim
    from oracle import grad64 as G
    p = small_params(n_neighbors=0, mc_diff=True)
    pp = p.replace(Ab=0.83, kb=0.05, eField=0.52, lifetime=2000.0, long_diff=5e-6, tran_diff=9e-6,
                   lArDensity=1.39)
    tracks, fields, nrm = _case(seed, n_tracks, shower)
    theta = grad.theta_of(pp).requires_grad_(True)
    wfs, unique = sim.param_wfs_fn(theta, pp, tracks, fields, nrm)
    rng = np.random.default_rng(seed + 1)
    c = torch.from_numpy(rng.standard_normal(tuple(wfs.shape)).astype(np.float32)).cuda()
    (wfs * c).sum().backward()
    g_gpu = dict(zip(grad.GRAD_PARAMS, theta.grad.cpu().numpy().tolist()))
    th = G.theta_dict(pp)
    W, fr, valid = G.param_waveforms64(pp, tracks, fields, nrm, th)
    u = unique.cpu().numpy()
    assert np.array_equal(valid, u[u >= 0])
    # the forward itself
    w = wfs.detach().cpu().numpy()[u >= 0]
    sc = np.abs(W).max(axis=1, keepdims=True)
    assert float((np.abs(w - W) / np.where(sc > 0, sc, 1)).max()) < 2e-4
    cv = c.cpu().numpy().astype(np.float64)[u >= 0]
    sens, g_cs = 0.0, {}
    for k in G.GRAD_PARAMS:
        tc = {q: complex(v) for q, v in th.items()}
        tc[k] += 1e-30j
        g_cs[k] = float((G.param_waveforms64(pp, tracks, fields, nrm, tc, fr)[0] * cv).sum().imag / 1e-30)
        sens = max(sens, abs(g_cs[k] * th[k]))
    assert abs(g_cs["eField"]) > 0 and g_gpu["vdrift"] == 0.0
    for k in G.GRAD_PARAMS:
        err = abs(g_gpu[k] - g_cs[k])
        assert err <= RTOL * abs(g_cs[k]) or err * abs(th[k]) <= 1e-5 * sens, (k, g_gpu[k], g_cs[k])


def test_param_adc_chain_is_differentiable(cuda):
    """param_wfs_fn -> fee_adc: the ADC-level gradient of the parametrised
    mode (params_loss_parametrized's path) runs and is finite; a loss
    against a target at other charge-scale parameters (lifetime, Ab: the
    electron positions, hence the pixels, stay put) has non-zero gradients."""
    from larndsim_gb300 import grad, sim
    p = small_params(n_neighbors=0, mc_diff=True)
    tracks, fields, nrm = _case(8, 3)
    with torch.no_grad():
        w0, u0 = sim.param_wfs_fn(grad.theta_of(p), p, tracks, fields, nrm)
        a0, _ = sim.fee_adc(p, w0[u0 >= 0])
    pp = p.replace(lifetime=2100.0, Ab=0.82)
    theta = grad.theta_of(pp).requires_grad_(True)
    wfs, unique = sim.param_wfs_fn(theta, pp, tracks, fields, nrm)
    assert torch.equal(unique, u0)
    adc, _ = sim.fee_adc(pp, wfs[unique >= 0])
    loss = ((adc - a0) ** 2).sum()
    loss.backward()
    g = theta.grad.cpu().numpy()
    assert np.all(np.isfinite(g)) and float(loss.detach()) > 0
    assert g[grad.GRAD_PARAMS.index("lifetime")] != 0.0 and g[grad.GRAD_PARAMS.index("Ab")] != 0.0
