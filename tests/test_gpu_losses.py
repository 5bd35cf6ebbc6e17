"""Hit-level fit loss mse_adc (lsim_mse_adc; losses_jax.py:13-79) against
the float64 oracle, and its gradient through the LUT chain
(params_loss, losses_jax.py:385-398, differentiated as fit_params.py:731
does).

Tolerances: the loss within 1e-5 relative (float32 kernel values summed
per row in float32, totals in float64); the weight and z gradients within
1e-4 of the largest component."""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _hits(rng, n, n_events, spread=3.0):
    ev = np.sort(rng.integers(0, n_events, n)).astype(np.int32)
    cx = rng.uniform(-20, 20, n_events)[ev]
    return ((cx + rng.normal(0, spread, n)).astype(np.float32), rng.normal(0, spread, n).astype(np.float32),
            rng.normal(0, spread, n).astype(np.float32), ev)


@pytest.mark.parametrize("shuffle", [False, True])
def test_mse_adc_matches_oracle(cuda, shuffle):
    from larndsim_gb300 import consts, losses
    from oracle import losses_np as L
    rng = np.random.default_rng(5)
    x, y, z, ev = _hits(rng, 700, 4)
    rx, ry, rz, rev = _hits(rng, 600, 4)
    Q = rng.uniform(5, 80, 700).astype(np.float32)
    hp = (rng.uniform(0, 1, 700) > 0.1).astype(np.float32)
    rQ = rng.uniform(5, 80, 600).astype(np.float32)
    rhp = np.ones(600, np.float32)
    if shuffle:
        i, j = rng.permutation(700), rng.permutation(600)
        x, y, z, ev, Q, hp = x[i], y[i], z[i], ev[i], Q[i], hp[i]
        rx, ry, rz, rev, rQ, rhp = rx[j], ry[j], rz[j], rev[j], rQ[j], rhp[j]
    p = consts.Params()
    tQ = torch.from_numpy(Q).cuda().requires_grad_(True)
    tz = torch.from_numpy(z).cuda().requires_grad_(True)
    loss, aux = losses.mse_adc(p, tQ, x, y, tz, None, hp, ev, rQ, rx, ry, rz, None, rhp, rev, sigma=1.5,
                               lambda_Q=0.5)
    loss.backward()
    ref, m, c = L.mse_adc(Q, x, y, z, hp, ev, rQ, rx, ry, rz, rhp, rev, sigma=1.5, lambda_Q=0.5)
    assert abs(float(loss.detach()) - ref) <= 1e-5 * abs(ref)
    assert abs(float(aux["mmd_loss_term"]) - m) <= 1e-5 * abs(ref)
    gw, gz = L.mse_adc_grad(Q.astype(np.float64) * hp, x, y, z, ev, rQ.astype(np.float64) * rhp, rx, ry, rz, rev,
                            sigma=1.5, lambda_Q=0.5)
    gq = gw * hp
    np.testing.assert_allclose(tQ.grad.cpu().numpy(), gq, atol=1e-4 * np.abs(gq).max(), rtol=0)
    np.testing.assert_allclose(tz.grad.cpu().numpy(), gz, atol=1e-4 * np.abs(gz).max(), rtol=0)


def test_mse_adc_events_are_independent(cuda):
    """Hits of different events never interact: a set against itself gives
    0, against the same hits moved to other events the sum of both self terms."""
    from larndsim_gb300 import consts, losses
    rng = np.random.default_rng(9)
    x, y, z, ev = _hits(rng, 400, 3)
    Q = rng.uniform(5, 80, 400).astype(np.float32)
    one = np.ones(400, np.float32)
    p = consts.Params()
    # against itself shifted by one event id: no pair interacts across sets
    loss, aux = losses.mse_adc(p, Q, x, y, z, None, one, ev, Q, x, y, z, None, one, ev + 10, lambda_Q=0.0)
    # MMD with disjoint supports = A/sw^2 + C/sv^2 with A = C
    loss_self, _ = losses.mse_adc(p, Q, x, y, z, None, one, ev, Q, x, y, z, None, one, ev, lambda_Q=0.0)
    assert abs(float(loss_self)) <= 1e-5 * float(loss)
    assert float(loss) > 0


def test_params_loss_gradient(cuda):
    """dL/dtheta through mse_adc, the hit z and the LUT adjoint: (1) equals
    the explicit composition (the kernel's weight and z gradients pulled
    back by the LUT vector-Jacobian product and by z(eField)); (2) matches
    float64 central differences of the same loss built on the oracle with
    the crossing ticks frozen, the semantics jax.grad gives it (ticks carry
    no gradient)."""
    from larndsim_gb300 import grad, losses
    from oracle import grad64 as G, losses_np as L, reference_np as R
    from gpu_common import small_params
    from larndsim_gb300 import workloads
    p = small_params(n_neighbors=1)
    tmpl = R.load_lut_templates(workloads.synthetic_response(seed=0, nx=15, ny=15), p)
    tracks, fields = workloads.muon_event(seed=3, n_tracks=3)
    chain = grad.LUTChain(p, torch.from_numpy(tmpl).cuda(), tracks, fields)
    with torch.no_grad():
        ref = tuple(t.detach() for t in grad.predicted_hits(grad.theta_of(p, device="cuda"), chain, p))
    pp = p.replace(Ab=0.83, kb=0.05, eField=0.52, lifetime=2000.0, long_diff=5e-6, tran_diff=9e-6,
                   lArDensity=1.39)
    loss, aux, theta = grad.params_loss(pp, chain, ref, sigma=1.0)
    loss.backward()
    g = dict(zip(grad.GRAD_PARAMS, theta.grad.cpu().numpy().tolist()))
    # (1) explicit composition
    th = grad.theta_of(pp, device="cuda").requires_grad_(True)
    Q, x, y, z, t, hp, ev = grad.predicted_hits(th, chain, pp)
    Qd = Q.detach().requires_grad_(True)
    zd = z.detach().requires_grad_(True)
    l2, _ = losses.mse_adc(pp, Qd, x, y, zd, t, hp, ev, *ref)
    l2.backward()
    assert abs(float(l2.detach()) - float(loss.detach())) <= 1e-6 * abs(float(loss.detach()))
    g_explicit = torch.autograd.grad((Q * Qd.grad).sum() + (z * zd.grad).sum(), th)[0].cpu().numpy()
    g_vec = np.array([g[k] for k in grad.GRAD_PARAMS])
    np.testing.assert_allclose(g_vec, g_explicit, rtol=1e-5, atol=1e-6 * np.abs(g_vec).max())
    # (2) frozen-decision float64 loss on the oracle
    adc_g, ticks_g, pids_g = chain.adc(pp)
    fr = G.Frozen(pp, tmpl, tracks, fields, pids_g.cpu().numpy(), adc_g.cpu().numpy())
    assert np.array_equal(fr.unique[fr.valid], pids_g.cpu().numpy())
    H = adc_g.shape[1]
    tk = ticks_g.cpu().numpy().reshape(-1)
    keep = tk < (int(pp.time_interval[1] / pp.t_sampling) - 3)
    xg, yg, plane, evg = (a.cpu().numpy() for a in grad.sim.pixel_coordinates(pp, pids_g))
    rep = lambda a: np.repeat(a, H)[keep]   # noqa: E731
    b = np.asarray(pp.tpc_borders, np.float64)[rep(plane)]
    za, sgn = b[:, 2, 0], np.sign(b[:, 2, 1] - b[:, 2, 0])
    tkk = tk[keep].astype(np.float64)
    rq, rx, ry, rz, _, rhp, rev = (a.cpu().numpy() for a in ref)
    bset = L.stacked(rx, ry, rz, rev)
    v = rq.astype(np.float64) * rhp
    a32 = L.stacked(rep(xg), rep(yg), np.zeros(keep.sum(), np.float32), rep(evg))
    k_q = (pp.V_REF - pp.V_CM) / pp.ADC_COUNTS / pp.GAIN * 1e-3
    q_off = (pp.V_CM - pp.V_PEDESTAL) / pp.GAIN * 1e-3

    def loss64(thd):
        adc = G.adc64(fr, thd)[fr.valid].reshape(-1)[keep]
        w = adc * k_q + q_off
        a = a32.copy()
        a[:, 2] = za + tkk * pp.t_sampling * G.vdrift64(pp, thd["eField"]) * sgn
        m = L.mmd(a, bset, w, v, 1.0)
        return m + ((w.sum() - v.sum()) / (v.sum() + 1e-6)) ** 2

    th0 = G.theta_dict(pp)
    sens = 0.0
    fd = {}
    for k in G.GRAD_PARAMS:
        h = 1e-5 * abs(th0[k])
        tp, tm = dict(th0), dict(th0)
        tp[k] += h
        tm[k] -= h
        fd[k] = (loss64(tp) - loss64(tm)) / (2 * h)
        sens = max(sens, abs(fd[k] * th0[k]))
    for k in G.GRAD_PARAMS:
        err = abs(g[k] - fd[k])
        assert err <= 2e-3 * abs(fd[k]) or err * abs(th0[k]) <= 1e-4 * sens, (k, g[k], fd[k])


def test_nll_loss_matches_oracle(cuda):
    from larndsim_gb300 import consts, losses
    from oracle import losses_np as L
    rng = np.random.default_rng(12)
    x, y, z, ev = _hits(rng, 500, 4, spread=1.5)
    rx, ry, rz, rev = _hits(rng, 450, 4, spread=1.5)
    Q = rng.uniform(5, 40, 500).astype(np.float32)
    rQ = rng.uniform(5, 40, 450).astype(np.float32)
    hp = rng.uniform(0.1, 1.0, 500).astype(np.float32)
    rhp = (rng.uniform(0, 1, 450) > 0.2).astype(np.float32)
    tQ = torch.from_numpy(Q).cuda().requires_grad_(True)
    tz = torch.from_numpy(z).cuda().requires_grad_(True)
    thp = torch.from_numpy(hp).cuda().requires_grad_(True)
    loss, _ = losses.nll_loss(consts.Params(), tQ, x, y, tz, None, thp, ev, rQ, rx, ry, rz, None, rhp, rev,
                              adc_norm=10.0, sigma=1.0)
    loss.backward()
    ref, gq, gz, ghp = L.nll_loss(Q, x, y, z, hp, ev, rQ, rx, ry, rz, rhp, rev, adc_norm=10.0, sigma=1.0)
    assert abs(float(loss.detach()) - ref) <= 1e-5 * abs(ref)
    for got, exp in ((tQ.grad, gq), (tz.grad, gz), (thp.grad, ghp)):
        np.testing.assert_allclose(got.cpu().numpy(), exp, atol=1e-4 * np.abs(exp).max(), rtol=0)


@pytest.mark.parametrize("n_events", [1, 4])
def test_chamfer_3d_matches_oracle(cuda, n_events):
    """Including the reference's zero padding (pad_size buckets) and the
    float32 rounding of x + event * 1e9."""
    from larndsim_gb300 import consts, losses, sim
    from oracle import losses_np as L
    rng = np.random.default_rng(20 + n_events)
    x, y, z, ev = _hits(rng, 600, n_events)
    rx, ry, rz, rev = _hits(rng, 520, n_events)
    Q = rng.uniform(5, 40, 600).astype(np.float32)
    rQ = rng.uniform(5, 40, 520).astype(np.float32)
    sim.reset_size_history()
    tQ = torch.from_numpy(Q).cuda().requires_grad_(True)
    tz = torch.from_numpy(z).cuda().requires_grad_(True)
    loss, _ = losses.chamfer_3d(consts.Params(), tQ, x, y, tz, None, None, ev, rQ, rx, ry, rz, None, None, rev)
    loss.backward()
    sizes = sim.get_size_history()["chamfer_3d"][0]
    ref, gq, gz = L.chamfer_3d(Q, x, y, z, ev, rQ, rx, ry, rz, rev, adc_norm=10.0, pad_to=(sizes[1], sizes[0]))
    assert abs(float(loss.detach()) - ref) <= 1e-5 * abs(ref)
    np.testing.assert_allclose(tQ.grad.cpu().numpy(), gq, atol=1e-4 * np.abs(gq).max(), rtol=0)
    np.testing.assert_allclose(tz.grad.cpu().numpy(), gz, atol=1e-4 * np.abs(gz).max(), rtol=0)
