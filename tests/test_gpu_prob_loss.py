"""CUDA likelihood losses on the probabilistic front end's distributions
(lsim_prob_llhd, lsim_llhd_loss, lsim_occurrence_indices) against the
oracle (oracle/prob_loss_np.py, itself pinned to the reference's own source)
and against the reference-source golden values.

Tolerances: the per-hit terms are float32 in the reference's order and the
sums are accumulated in double, so the loss agrees with the oracle's
float64 sum of the same float32 terms to 1e-6 relative; gradients to 1e-5
relative of the largest entry (float32 coefficient products)."""

import sys
from pathlib import Path

import numpy as np
import pytest
import torch

from larndsim_gb300 import consts, losses, strategies
from oracle import prob_loss_np as PL

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

from make_prob_loss_golden import llhd_inputs, prob_loss_inputs  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def params():
    return consts.Params()


def _strategy_call(params, sim, lp, ad, tp, tt, ta, dev, sigma=500.0, grad=True):
    lp_t = torch.from_numpy(lp).to(dev).requires_grad_(grad)
    ad_t = torch.from_numpy(ad).to(dev).requires_grad_(grad)
    pred = {"unique_pixels": torch.from_numpy(sim).to(dev), "hit_prob": lp_t, "adcs_distrib": ad_t}
    tgt = {"pixel_id": tp, "ticks": tt, "adcs": ta}
    loss, aux = strategies.ProbabilisticLossStrategy(sigma_charge=sigma).compute(params, pred, tgt)
    g = None
    if grad:
        loss.backward()
        g = (lp_t.grad.cpu().numpy(), ad_t.grad.cpu().numpy())
    return float(loss.detach()), {k: float(v) for k, v in aux.items()}, g


def _check(params, args, dev, sigma=500.0):
    cst = PL.adc_charge_consts(params)
    loss, aux, (g_lp, g_ad) = _strategy_call(params, *args, dev, sigma=sigma)
    lo, auxo = PL.prob_llhd(*args, cst, sigma_charge=sigma)
    assert abs(loss - lo) <= 1e-6 * max(abs(lo), 1e-30), (loss, lo)
    for k in auxo:
        assert abs(aux[k] - auxo[k]) <= 1e-6 * max(abs(auxo[k]), 1.0), (k, aux[k], auxo[k])
    go_lp, go_ad = PL.prob_llhd_grad(*args, cst, sigma_charge=sigma)
    for a, b in ((g_lp, go_lp), (g_ad, go_ad)):
        assert np.array_equal(a != 0, b != 0)
        assert np.abs(a - b).max() <= 1e-5 * max(np.abs(b).max(), 1e-30)
    return loss


def test_strategy_matches_oracle_and_reference(cuda, params):
    gold = np.load(GOLDEN / "prob_loss_ref.npz")
    loss = _check(params, prob_loss_inputs(), cuda)
    assert abs(loss - float(gold["prob/loss32"])) <= 1e-6 * loss


def test_strategy_edge_cases(cuda, params):
    rng = np.random.default_rng(5)
    sim = np.concatenate([np.full(3, -1, np.int32), np.arange(10, 400, 7, dtype=np.int32)])
    P, H, T = sim.shape[0], 4, 50
    lp = rng.uniform(-30, 0, (P, H, T)).astype(np.float32)
    lp[:, :, 7] = np.log(np.float32(1e-10))            # exact ties with the clamp
    ad = rng.uniform(0, 255, (P, H, T)).astype(np.float32)
    # runs longer than H (clamped row), unsorted ids, absent ids, pads, ticks
    # outside [0, T) both ways, ticks on the tie column
    tp = np.array([17] * 7 + [10, 400, 24, 24, 3, -1, -1, 31, 17, 10], np.int32)
    tt = np.array([0, 1, 2, 3, 4, 5, 6, -1, -60, 7, 7, 0, 0, 1, 49, 55, 7], np.float32)
    ta = rng.uniform(0, 255, tp.shape[0]).astype(np.float32)
    _check(params, (sim, lp, ad, tp, tt, ta), cuda)
    _check(params, (sim, lp, ad, tp, tt, ta), cuda, sigma=120.0)
    # target exactly on the pixels, one hit each: every hit valid
    tp1 = sim[3:].copy()
    _check(params, (sim, lp, ad, tp1, np.full(tp1.shape[0], 3.7, np.float32), ta[:1].repeat(tp1.shape[0])),
           cuda)


def test_strategy_no_target_hits(cuda, params):
    sim, lp, ad, _, _, _ = prob_loss_inputs()
    e = np.zeros(0, np.int32)
    loss, aux, (g_lp, g_ad) = _strategy_call(params, sim, lp, ad, e, e.astype(np.float32),
                                              e.astype(np.float32), cuda)
    assert loss == 0.0 and all(v == 0.0 for v in aux.values())
    assert not g_lp.any() and not g_ad.any()


def test_strategy_front_end_sized_case(cuda, params):
    """4096 pixels x 10 hits x 2000 ticks (the front end's shape on a
    batch), 30k target hits."""
    rng = np.random.default_rng(11)
    ids = np.sort(rng.choice(2_000_000, 4000, replace=False)).astype(np.int32)
    sim = np.concatenate([np.full(96, -1, np.int32), ids])
    P, H, T = sim.shape[0], 10, 2000
    lp = rng.uniform(-40, 0, (P, H, T)).astype(np.float32)
    ad = rng.uniform(0, 255, (P, H, T)).astype(np.float32)
    hit = rng.choice(ids, 12000, replace=True)
    tp = np.sort(np.concatenate([hit, rng.integers(0, 2_000_000, 18000)])).astype(np.int32)
    tt = rng.integers(-5, T + 5, tp.shape[0]).astype(np.float32)
    ta = rng.uniform(0, 255, tp.shape[0]).astype(np.float32)
    _check(params, (sim, lp, ad, tp, tt, ta), cuda)


def test_strategy_rejects_bad_inputs(cuda, params):
    from larndsim_gb300 import _abi
    sim, lp, ad, tp, tt, ta = prob_loss_inputs()
    with pytest.raises(ValueError):
        _strategy_call(params, sim[:-1], lp, ad, tp, tt, ta, cuda, grad=False)
    e = np.zeros(0, np.int32)
    with pytest.raises(_abi.LsimError, match="no simulated pixels"):
        _strategy_call(params, e, lp[:0], ad[:0], tp, tt, ta, cuda, grad=False)


def test_occurrence_indices_match_oracle(cuda):
    rng = np.random.default_rng(2)
    for n in (1, 5, 1023, 1024, 1025, 5000, 3_000_001):
        runs = rng.integers(1, 3000 if n > 10000 else 40, n)
        ids = np.repeat(np.arange(runs.shape[0]), runs)[:n].astype(np.int32)
        ids[rng.random(n) < 0.01] = -1
        got = strategies.compute_occurrence_indices(torch.from_numpy(ids).to(cuda)).cpu().numpy()
        assert np.array_equal(got, PL.compute_occurrence_indices(ids)), n
    one_run = np.full(70_000, 4, np.int32)          # a run across many tiles
    got = strategies.compute_occurrence_indices(one_run).cpu().numpy()
    assert np.array_equal(got, np.arange(70_000))
    assert strategies.compute_occurrence_indices(np.zeros(0, np.int32)).shape == (0,)


def test_llhd_loss_matches_oracle_and_reference(cuda):
    gold = np.load(GOLDEN / "prob_loss_ref.npz")
    for args in (llhd_inputs(), llhd_inputs(seed=21, N=3000, T=2000)):
        tpd, tk, nh, cd, cm = args
        ts = [torch.from_numpy(a).to(cuda).requires_grad_(True) for a in (tpd, nh, cd, cm)]
        loss, aux = losses.llhd_loss(ts[0], tk, ts[1], ts[2], ts[3])
        assert aux == {}
        lo, _ = PL.llhd_loss(*args)
        assert abs(float(loss.detach()) - lo) <= 1e-6 * abs(lo)
        loss.backward()
        go = PL.llhd_loss_grad(*args)
        for t, b in zip(ts, (go[0], go[1], go[2], go[3])):
            a = t.grad.cpu().numpy()
            assert np.abs(a - b).max() <= 1e-5 * max(np.abs(b).max(), 1e-30)
    l0, _ = losses.llhd_loss(*llhd_inputs())
    assert abs(float(l0) - float(gold["llhd/loss32"])) <= 1e-6 * abs(float(gold["llhd/loss32"]))


def _prob_chain(cuda):
    from gpu_common import small_params
    from larndsim_gb300 import grad, sim, workloads
    p = small_params(n_neighbors=1, RESET_NOISE_CHARGE=900)
    tmpl, p = sim.load_lut(workloads.synthetic_response(seed=0, nx=15, ny=15), p)
    tracks, fields = workloads.muon_event(seed=3, n_tracks=2)
    chain = grad.LUTChain(p, tmpl, tracks, fields)
    # the fitter's target: stochastic hits of the LUT simulation at nominal values
    tgt = strategies.LUTSimulation(tmpl).predict(p, tracks, fields, 0)
    target = {"pixel_id": tgt["hit_pixels"], "ticks": tgt["ticks"], "adcs": tgt["adcs"],
              "pixel_x": tgt["pixel_x"], "pixel_y": tgt["pixel_y"], "pixel_z": tgt["pixel_z"],
              "hit_prob": tgt["hit_prob"], "event": tgt["event"]}
    pp = p.replace(lifetime=2000.0, eField=0.51)
    theta = grad.theta_of(pp).requires_grad_(True)
    wfs, unique = grad.wfs_fn(theta, chain, pp)
    # LUTProbabilisticSimulation.predict: rows padded at the front to 128
    u = strategies.pad_to_closest_multiple(unique, multiple=128, pad_value=-1, pad_front=True)
    w = strategies.pad_to_closest_multiple(wfs, dims_to_pad=(0,), multiple=128, pad_value=0.0, pad_front=True)
    adcs, x, y, tp, ev = sim.simulate_probabilistic(pp, w, u)
    _, _, plane, _ = sim.pixel_coordinates(pp, u)
    pred = {"adcs_distrib": adcs, "hit_prob": tp, "pixel_x": x, "pixel_y": y, "pixel_plane": plane, "event": ev,
            "unique_pixels": u, "theta": theta}
    return pp, theta, pred, target


def test_probabilistic_strategy_reaches_the_parameters(cuda):
    """wfs_fn -> simulate_probabilistic -> ProbabilisticLossStrategy: the
    loss equals the oracle's on the same distributions, and autograd's
    parameter gradient equals the oracle's cotangents pulled back through
    the same chain (digitize, lsim_fee_prob_vjp, lsim_lut_wfs_vjp)."""
    from larndsim_gb300 import grad
    pp, theta, pred, target = _prob_chain(cuda)
    loss, aux = strategies.ProbabilisticLossStrategy().compute(pp, pred, target)
    lp = pred["hit_prob"].detach().cpu().numpy()
    ad = pred["adcs_distrib"].detach().cpu().numpy()
    args = (pred["unique_pixels"].cpu().numpy(), lp, ad, target["pixel_id"].cpu().numpy(),
            target["ticks"].cpu().numpy(), target["adcs"].cpu().numpy())
    cst = PL.adc_charge_consts(pp)
    lo, auxo = PL.prob_llhd(*args, cst)
    assert abs(float(loss.detach()) - lo) <= 1e-6 * abs(lo)
    assert abs(float(aux["no_match_penalty"]) - auxo["no_match_penalty"]) <= 1e-6 * max(abs(auxo["no_match_penalty"]), 1)
    loss.backward(retain_graph=True)
    g = theta.grad.clone()
    assert torch.isfinite(g).all() and g[grad.GRAD_PARAMS.index("eField")] != 0
    theta.grad = None
    g_lp, g_ad = PL.prob_llhd_grad(*args, cst)
    torch.autograd.backward([pred["hit_prob"], pred["adcs_distrib"]],
                            [torch.from_numpy(g_lp.astype(np.float32)).to(cuda),
                             torch.from_numpy(g_ad.astype(np.float32)).to(cuda)])
    g2 = theta.grad
    assert torch.allclose(g, g2, rtol=1e-4, atol=1e-6 * float(g2.abs().max()))


def test_collapsed_strategy_pseudo_hits(cuda):
    """CollapsedProbabilisticLossStrategy's collapsed pseudo-hits against
    numpy (get_average_hit_values on the prediction's hit_prob, adc2charge,
    get_hit_z at the expected tick), and the mse_adc loss on them
    differentiates to the parameters.  The strategy reads hit_prob as it is
    given; the case gives it probabilities (exp of the front end's
    log-probabilities)."""
    from oracle import reference_np as R
    pp, theta, pred, target = _prob_chain(cuda)
    pred = dict(pred, hit_prob=torch.exp(pred["hit_prob"]))
    st = strategies.CollapsedProbabilisticLossStrategy(losses.mse_adc)
    Q, x, y, z, t, hp, ev = st._prepare_probabilistic_output(pp, pred)
    tp = pred["hit_prob"].detach().cpu().numpy().astype(np.float64)
    ad = pred["adcs_distrib"].detach().cpu().numpy().astype(np.float64)
    lam = tp.sum(axis=2)
    den = np.maximum(lam, 1e-10)
    et = (np.arange(tp.shape[2]) * tp).sum(axis=2) / den
    ea = (ad * tp).sum(axis=2) / den
    np.testing.assert_allclose(hp.detach().cpu().numpy(), lam, rtol=1e-5)
    np.testing.assert_allclose(t.detach().cpu().numpy(), et, rtol=1e-4, atol=1e-3)
    np.testing.assert_allclose(Q.detach().cpu().numpy(), R.adc2charge(ea.astype(np.float32), pp), rtol=1e-4,
                               atol=1e-4)
    plane = pred["pixel_plane"].cpu().numpy()
    zo = R.get_hit_z(pp, et.astype(np.float32), np.repeat(plane[:, None], tp.shape[1], axis=1))
    np.testing.assert_allclose(z.detach().cpu().numpy(), zo, rtol=1e-4, atol=1e-2)
    assert np.array_equal(ev.cpu().numpy(), np.repeat(pred["event"].cpu().numpy()[:, None], tp.shape[1], 1))
    loss, _ = st.compute(pp, pred, target)
    loss.backward()
    assert torch.isfinite(theta.grad).all()


@pytest.mark.parametrize("name,sparse,collapsed", [("collapsed", False, True), ("entries", True, False)])
def test_collapsed_strategy_matches_reference(cuda, params, name, sparse, collapsed):
    """CollapsedProbabilisticLossStrategy with mse_adc (expected values per
    (pixel, hit), or one pseudo-hit per entry above the hit threshold)
    against the reference's own strategy run on the numpy stand-in, 1e-5
    relative (float32 sums in a different order)."""
    from make_prob_loss_golden import collapsed_inputs
    gold = np.load(GOLDEN / "prob_loss_ref.npz")
    pred, tgt = collapsed_inputs(sparse=sparse)
    pred_t = {k: torch.from_numpy(v).to(cuda) for k, v in pred.items()}
    tgt_t = {k: torch.from_numpy(v).to(cuda) for k, v in tgt.items()}
    st = strategies.CollapsedProbabilisticLossStrategy(losses.mse_adc, collapsed=collapsed)
    loss, _ = st.compute(params, pred_t, tgt_t)
    ref = float(gold[f"{name}/loss32"])
    assert abs(float(loss.detach()) - ref) <= 1e-5 * abs(ref), (float(loss.detach()), ref)
