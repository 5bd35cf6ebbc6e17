"""Edge cases of the gradient paths and the next-row kernels: padding rows
(eventID -1, the reference's TracksDataset padding, optimize/dataio.py:340-355)
and an event id with no segments in a gradient batch; all-zero and empty
waveform sets through the probabilistic front end and its adjoint; a loss
whose reference set lacks one of the predicted events; padding rows through
the parametrised-mode adjoint."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_common import small_params

pytestmark = pytest.mark.gpu


def test_lut_gradient_with_padding_rows_and_a_missing_event(cuda):
    from larndsim_gb300 import grad, sim, workloads
    p = small_params(n_neighbors=1)
    tmpl, p = sim.load_lut(workloads.synthetic_response(seed=0, nx=15, ny=15), p)
    a, fields = workloads.muon_event(seed=1, n_tracks=2, event_id=0)
    b, _ = workloads.muon_event(seed=2, n_tracks=2, event_id=2)          # event 1 has no segments
    tracks = workloads.pad_tracks(np.concatenate([a, b]), fields, a.shape[0] + b.shape[0] + 25)
    chain = grad.LUTChain(p, tmpl, tracks, fields, n_events=3)
    target = chain.target(p)
    loss0, g0 = chain.loss_and_grad(p, target)
    assert loss0 == 0.0 and all(v == 0.0 for v in g0.values())
    loss, g = chain.loss_and_grad(p.replace(eField=0.52, lifetime=2000.0), target)
    assert loss > 0 and all(np.isfinite(v) for v in g.values())
    # the padding rows change nothing
    chain2 = grad.LUTChain(p, tmpl, np.concatenate([a, b]), fields, n_events=3)
    loss2, g2 = chain2.loss_and_grad(p.replace(eField=0.52, lifetime=2000.0), chain2.target(p))
    # (the per-segment partial sums are chunked by row count, so compare to rounding)
    assert abs(loss2 - loss) <= 1e-6 * loss
    np.testing.assert_allclose([g2[k] for k in g], [g[k] for k in g], rtol=1e-6, atol=0)


def test_probabilistic_front_end_on_zero_and_empty_rows(cuda):
    from larndsim_gb300 import sim
    p = small_params(n_neighbors=1, RESET_NOISE_CHARGE=900)
    H = int(p.MAX_ADC_VALUES)
    zero = torch.zeros((5, 2000), device="cuda", requires_grad=True)
    et, ea, lam = sim.average_hit_values(p, zero)
    assert torch.isfinite(et).all() and torch.isfinite(ea).all() and torch.isfinite(lam).all()
    assert float(lam.detach().max()) < 1e-3                            # nothing crosses the threshold
    (et.sum() + ea.sum() + lam.sum()).backward()
    assert torch.isfinite(zero.grad).all()
    empty = torch.zeros((0, 2000), device="cuda")
    lp, ch = sim.get_adc_values_average_noise_vmap(p, empty)
    assert lp.shape == (0, H, 1999) and ch.shape == (0, H, 1999)
    e2 = sim.average_hit_values(p, empty)
    assert all(t.shape == (0, H) for t in e2)


def test_loss_with_an_event_missing_from_the_reference(cuda):
    from larndsim_gb300 import consts, losses
    from oracle import losses_np as L
    rng = np.random.default_rng(4)
    n, m = 300, 200
    ev = np.sort(rng.integers(0, 3, n)).astype(np.int32)
    rev = np.sort(rng.choice([0, 2], m)).astype(np.int32)                # no reference hits in event 1
    x, y, z = (rng.normal(0, 2, n).astype(np.float32) for _ in range(3))
    rx, ry, rz = (rng.normal(0, 2, m).astype(np.float32) for _ in range(3))
    Q = rng.uniform(5, 40, n).astype(np.float32)
    rQ = rng.uniform(5, 40, m).astype(np.float32)
    one, rone = np.ones(n, np.float32), np.ones(m, np.float32)
    p = consts.Params()
    l1, _ = losses.mse_adc(p, Q, x, y, z, None, one, ev, rQ, rx, ry, rz, None, rone, rev)
    r1 = L.mse_adc(Q, x, y, z, one, ev, rQ, rx, ry, rz, rone, rev)[0]
    assert abs(float(l1) - r1) <= 1e-5 * abs(r1)
    l2, _ = losses.nll_loss(p, Q, x, y, z, None, one, ev, rQ, rx, ry, rz, None, rone, rev)
    r2 = L.nll_loss(Q, x, y, z, one, ev, rQ, rx, ry, rz, rone, rev)[0]
    assert abs(float(l2) - r2) <= 1e-5 * abs(r2)
    from larndsim_gb300 import sim
    sim.reset_size_history()
    l3, _ = losses.chamfer_3d(p, Q, x, y, z, None, None, ev, rQ, rx, ry, rz, None, None, rev)
    sizes = sim.get_size_history()["chamfer_3d"][0]
    r3 = L.chamfer_3d(Q, x, y, z, ev, rQ, rx, ry, rz, rev, pad_to=(sizes[1], sizes[0]))[0]
    assert abs(float(l3) - r3) <= 1e-5 * abs(r3)


def test_param_gradient_with_padding_rows(cuda):
    from larndsim_gb300 import grad, sim, workloads
    p = small_params(n_neighbors=0, mc_diff=True)
    tracks, fields = workloads.muon_event(seed=5, n_tracks=2)
    nrm = np.random.default_rng(5).standard_normal((tracks.shape[0], 3)).astype(np.float32)
    padded = workloads.pad_tracks(tracks, fields, tracks.shape[0] + 30)
    nrm_p = np.concatenate([nrm, np.zeros((30, 3), np.float32)])
    pp = p.replace(lifetime=2000.0)
    out = []
    for tr, nr in ((tracks, nrm), (padded, nrm_p)):
        theta = grad.theta_of(pp).requires_grad_(True)
        sim.reset_size_history()
        wfs, unique = sim.param_wfs_fn(theta, pp, tr, fields, nr)
        (wfs[unique >= 0] ** 2).sum().backward()
        out.append(theta.grad.cpu().numpy())
    assert np.all(np.isfinite(out[0])) and np.abs(out[0]).max() > 0
    np.testing.assert_array_equal(out[0], out[1])
