"""Adjoint parity: the GPU forward+backward of the LUT chain against the
float64 pathwise gradient of the frozen-decision loss (oracle/grad64.py:
reverse-mode adjoint, checked against complex-step derivatives and central
finite differences) -- the gradient jax.value_and_grad computes
(fit_params.py:731).  Tolerance: 1e-4 relative per parameter.

The loss gradient is sum 2 (ADC - target) dADC/dtheta; close to the target
the residuals are a few % of the ADC, so float32 rounding of the forward
ADC (~3e-6 relative) moves the residuals by ~1e-4.  The loss test therefore
compares against the float64 vector-Jacobian product at the GPU's own
residuals, and the end-to-end finite-difference test uses a 20 % parameter
offset where residuals dominate rounding."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_common import small_params

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-4


def _setup(n_neighbors=1, seed=3, n_tracks=3, shower=0):
    from larndsim_gb300 import grad, workloads
    from oracle import reference_np as R
    p = small_params(n_neighbors=n_neighbors)
    nx = 10 * n_neighbors + 5
    resp = workloads.synthetic_response(seed=0, nx=nx, ny=nx)
    tmpl = R.load_lut_templates(resp, p)
    tracks, fields = workloads.muon_event(seed=seed, n_tracks=n_tracks)
    if shower:
        sh, _ = workloads.shower_event(seed=seed + 100, n_segments=shower)
        tracks = np.concatenate([tracks, sh])
    chain = grad.LUTChain(p, torch.from_numpy(tmpl).cuda(), tracks, fields)
    target = chain.target(p)
    return p, tmpl, tracks, fields, chain, target


def _perturbed(p):
    return p.replace(Ab=0.83, kb=0.05, eField=0.52, lifetime=2000.0, long_diff=5e-6, tran_diff=9e-6,
                     lArDensity=1.39)


def _check(g_gpu, g_fd, theta):
    names = list(g_fd)
    sens = max(abs(g_fd[k] * theta[k]) for k in names)
    for k in names:
        err = abs(g_gpu[k] - g_fd[k])
        ok = err <= GRAD_RTOL * abs(g_fd[k]) or err * abs(theta[k]) <= GRAD_RTOL * sens * 1e-2
        assert ok, (k, g_gpu[k], g_fd[k])


@pytest.mark.parametrize("case", [dict(n_neighbors=1), dict(n_neighbors=2, seed=5, n_tracks=2, shower=300),
                                  dict(n_neighbors=0, seed=6, n_tracks=2, shower=300),
                                  dict(n_neighbors=4, seed=7, n_tracks=2, shower=200)])
def test_loss_and_grad_vs_fp64_adjoint(cuda, case):
    from oracle import grad64 as G
    p, tmpl, tracks, fields, chain, target = _setup(**case)
    pp = _perturbed(p)
    loss, g = chain.loss_and_grad(pp, target)
    fr = G.Frozen(pp, tmpl, tracks, fields, target.pids.cpu().numpy(), target.adc.cpu().numpy())
    th = G.theta_dict(pp)
    # the GPU forward takes the same discrete decisions as the oracle's
    adc, ticks, pids = chain.adc(pp)
    assert np.array_equal(pids.cpu().numpy(), fr.unique[fr.valid])
    acc = ~fr.cond[fr.valid]
    assert np.array_equal(ticks.cpu().numpy()[acc], fr.idx[fr.valid][acc].astype(np.float32))
    L64 = G.loss64(fr, th)
    assert abs(loss - L64) <= 1e-3 * L64 + 1e-3
    assert g["vdrift"] == 0.0
    resid = 2.0 * (adc.cpu().numpy().astype(np.float64) - fr.tgt)
    g_ref = G.adjoint64(fr, th, g_adc=resid)
    _check(g, g_ref, th)


def test_fp64_adjoint_matches_complex_step_and_fd(cuda):
    """The oracle's reverse mode equals its complex-step and FD gradients."""
    from oracle import grad64 as G
    p, tmpl, tracks, fields, chain, target = _setup()
    pp = _perturbed(p)
    fr = G.Frozen(pp, tmpl, tracks, fields, target.pids.cpu().numpy(), target.adc.cpu().numpy())
    th = G.theta_dict(pp)
    adj, cs, fd = G.adjoint64(fr, th), G.complex_step_gradient(fr, th), G.fd_gradient(fr, th, 1e-6)
    for k in G.GRAD_PARAMS:
        assert abs(adj[k] - cs[k]) <= 1e-9 * abs(cs[k]) + 1e-12
        assert abs(adj[k] - fd[k]) <= 1e-5 * abs(cs[k]) + 1e-9


def test_loss_gradient_vs_fd_far_from_target(cuda):
    """End to end: GPU loss gradient vs FP64 central differences at a 20 %
    offset, where the residuals are large compared with float32 rounding."""
    from oracle import grad64 as G
    p, tmpl, tracks, fields, chain, target = _setup()
    pp = p.replace(Ab=0.8 * 1.2, kb=0.0486 * 0.8, eField=0.6, lifetime=1800.0, long_diff=6e-6, tran_diff=1.1e-5,
                   lArDensity=1.38 * 1.02)
    loss, g = chain.loss_and_grad(pp, target)
    fr = G.Frozen(pp, tmpl, tracks, fields, target.pids.cpu().numpy(), target.adc.cpu().numpy())
    th = G.theta_dict(pp)
    _check(g, G.complex_step_gradient(fr, th), th)


def test_autograd_function_matches_fd(cuda):
    """torch.autograd path with an arbitrary cotangent on the ADC grid."""
    from larndsim_gb300 import grad
    from oracle import grad64 as G
    p, tmpl, tracks, fields, chain, target = _setup()
    pp = _perturbed(p)
    theta = grad.theta_of(pp).requires_grad_(True)
    adc, ticks, pids = grad.adc_fn(theta, chain, pp)
    rng = np.random.default_rng(1)
    c = torch.from_numpy(rng.standard_normal(tuple(adc.shape)).astype(np.float32)).cuda()
    (adc * c).sum().backward()
    g_gpu = dict(zip(grad.GRAD_PARAMS, theta.grad.cpu().numpy().tolist()))
    fr = G.Frozen(pp, tmpl, tracks, fields, target.pids.cpu().numpy(), target.adc.cpu().numpy())
    cc = c.cpu().numpy().astype(np.float64)
    th = G.theta_dict(pp)

    def lin(t):
        return float((G.adc64(fr, t)[fr.valid] * cc).sum())

    g_fd = {}
    for k in G.GRAD_PARAMS:
        h = 1e-4 * abs(th[k])
        tp, tm = dict(th), dict(th)
        tp[k] += h
        tm[k] -= h
        g_fd[k] = (lin(tp) - lin(tm)) / (2 * h)
    _check(g_gpu, g_fd, th)


def test_gradient_is_deterministic(cuda):
    p, tmpl, tracks, fields, chain, target = _setup()
    pp = _perturbed(p)
    a = chain.loss_and_grad(pp, target)
    b = chain.loss_and_grad(pp, target)
    assert a == b


def test_loss_zero_at_target_params(cuda):
    p, tmpl, tracks, fields, chain, target = _setup()
    loss, g = chain.loss_and_grad(p, target)
    assert loss == 0.0
    assert all(v == 0.0 for v in g.values())


def test_stored_waveform_variant_matches_recompute(cuda):
    """The store-the-waveforms adjoint gives the recomputing adjoint's
    loss and gradient bit for bit."""
    p, tmpl, tracks, fields, chain, target = _setup(n_neighbors=2, seed=5, n_tracks=2, shower=300)
    pp = _perturbed(p)
    a = chain.loss_and_grad(pp, target)
    loss, g, wfs = chain.loss_and_grad_stored(pp, target)
    assert wfs.shape[0] == chain._stage.n_valid
    assert (loss, g) == a


@pytest.mark.parametrize("case", [dict(n_neighbors=1), dict(n_neighbors=2, seed=5, n_tracks=2, shower=300),
                                  dict(n_neighbors=1, seed=11, n_tracks=2, recomb="BOX"),
                                  dict(n_neighbors=1, seed=12, n_tracks=2, recomb="ELLIPSOID")])
def test_wfs_vjp_matches_complex_step(cuda, case):
    """lsim_lut_wfs_vjp through grad.wfs_fn (jax.vjp of simulate_wfs): an
    arbitrary cotangent on the waveform rows pulled back to the 8
    parameters, against the complex-step derivative of the float64
    waveforms of the oracle (decisions frozen)."""
    from larndsim_gb300 import consts, grad
    from oracle import grad64 as G
    case = dict(case)
    recomb = case.pop("recomb", None)
    p, tmpl, tracks, fields, chain, target = _setup(**case)
    pp = _perturbed(p)
    if recomb is not None:   # Box models: eField and lArDensity enter through csi
        pp = pp.replace(recombination_mode=getattr(consts.RecombinationMode, recomb))
        target = chain.target(pp)
    theta = grad.theta_of(pp).requires_grad_(True)
    wfs, unique = grad.wfs_fn(theta, chain, pp)
    rng = np.random.default_rng(4)
    c = torch.from_numpy(rng.standard_normal(tuple(wfs.shape)).astype(np.float32)).cuda()
    (wfs * c).sum().backward()
    g_gpu = dict(zip(grad.GRAD_PARAMS, theta.grad.cpu().numpy().tolist()))
    fr = G.Frozen(pp, tmpl, tracks, fields, target.pids.cpu().numpy(), target.adc.cpu().numpy())
    u = unique.cpu().numpy()
    assert np.array_equal(fr.unique[fr.valid], u[u >= 0])
    cv = c.cpu().numpy().astype(np.float64)[u >= 0]
    th = G.theta_dict(pp)
    g_cs = {}
    for k in G.GRAD_PARAMS:
        tc = {q: complex(v) for q, v in th.items()}
        tc[k] += 1e-30j
        g_cs[k] = float((G.waveforms64(fr, tc)[fr.valid] * cv).sum().imag / 1e-30)
    _check(g_gpu, g_cs, th)


def test_fee_vjp_matches_fp64_front_end_adjoint(cuda):
    """lsim_fee_vjp through sim.fee_adc: dL/dwfs for a random ADC cotangent,
    against the float64 reverse-mode adjoint of the front end with its
    decisions frozen (oracle fee_adjoint64)."""
    from larndsim_gb300 import sim
    from oracle import grad64 as G
    p, tmpl, tracks, fields, chain, target = _setup(n_neighbors=2, seed=5, n_tracks=2, shower=300)
    pp = _perturbed(p)
    wfs, unique = chain.wfs(pp)
    w = wfs[unique >= 0].contiguous().requires_grad_(True)
    adc, ticks = sim.fee_adc(pp, w)
    rng = np.random.default_rng(8)
    g_adc = rng.standard_normal(tuple(adc.shape)).astype(np.float32)
    (adc * torch.from_numpy(g_adc).cuda()).sum().backward()
    fr = G.Frozen.__new__(G.Frozen)
    fr.params = pp
    fr._fee_decisions(w.detach().cpu().numpy())
    # rows whose hit ticks agree on both sides (cumulative sums in another
    # order can move a crossing that sits on the threshold by one tick)
    T = w.shape[1]
    same = np.all(ticks.cpu().numpy() == np.where(fr.cond, T - 2, fr.idx).astype(np.float32), axis=1)
    assert same.mean() > 0.99 and same.sum() > 50
    ref = G.fee_adjoint64(fr, g_adc.astype(np.float64))[same]
    got = w.grad.cpu().numpy()[same]
    assert np.abs(ref).max() > 0
    np.testing.assert_allclose(got, ref, atol=1e-5 * np.abs(ref).max(), rtol=0)


def test_modular_chain_equals_fused_gradient(cuda):
    """wfs_fn -> fee_adc in torch autograd (waveforms materialised, two
    vector-Jacobian products) gives the gradient the fused lsim_lut_grad
    computes without storing waveforms, for the same ADC cotangent."""
    from larndsim_gb300 import grad, sim
    p, tmpl, tracks, fields, chain, target = _setup(n_neighbors=1, seed=9, n_tracks=3, shower=200)
    pp = _perturbed(p)
    theta = grad.theta_of(pp).requires_grad_(True)
    wfs, unique = grad.wfs_fn(theta, chain, pp)
    adc, _ = sim.fee_adc(pp, wfs[unique >= 0])
    rng = np.random.default_rng(2)
    c = torch.from_numpy(rng.standard_normal(tuple(adc.shape)).astype(np.float32)).cuda()
    (adc * c).sum().backward()
    g_mod = dict(zip(grad.GRAD_PARAMS, theta.grad.cpu().numpy().tolist()))
    g_fused = dict(zip(grad.GRAD_PARAMS, chain.vjp(pp, c).cpu().numpy().tolist()))
    _check(g_mod, g_fused, {k: float(getattr(pp, k)) for k in grad.GRAD_PARAMS})
