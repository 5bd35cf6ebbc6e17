"""Pin the likelihood-loss oracle (oracle/prob_loss_np.py) to the
reference's ProbabilisticLossStrategy, compute_occurrence_indices and
llhd_loss run from its own source (tests/golden/prob_loss_ref.npz, made by
tests/golden/make_prob_loss_golden.py on the numpy stand-in for jax), and
check the oracle's indexing semantics on small hand cases."""

import sys
from pathlib import Path

import numpy as np
import pytest

from larndsim_gb300 import consts
from oracle import prob_loss_np as PL

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

from make_prob_loss_golden import llhd_inputs, prob_loss_inputs  # noqa: E402


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN / "prob_loss_ref.npz")


@pytest.fixture(scope="module")
def cst():
    return PL.adc_charge_consts(consts.Params())


def test_occurrence_indices_match_reference(gold):
    _, _, _, tp, _, _ = prob_loss_inputs()
    assert np.array_equal(PL.compute_occurrence_indices(tp), gold["occurrence"])
    assert PL.compute_occurrence_indices(np.array([100, 100, 100, 200, 200, 300])).tolist() == [0, 1, 2, 0, 1, 0]
    assert PL.compute_occurrence_indices(np.array([5, 7, 5, 5])).tolist() == [0, 0, 0, 1]
    assert PL.compute_occurrence_indices(np.array([], np.int32)).shape == (0,)


def test_prob_llhd_matches_reference(gold, cst):
    args = prob_loss_inputs()
    loss, aux = PL.prob_llhd(*args, cst)
    assert abs(loss - float(gold["prob/loss32"])) <= 2e-7 * abs(loss)
    assert abs(loss - float(gold["prob/loss64"])) <= 2e-7 * abs(loss)
    for k, v in aux.items():
        assert abs(v - float(gold[f"prob/aux32/{k}"])) <= 2e-7 * max(abs(v), 1.0), k


def test_prob_llhd_gradient_matches_reference_differences(gold, cst):
    g_lp, g_ad = PL.prob_llhd_grad(*prob_loss_inputs(), cst)
    pos = gold["prob/fd_pos"]
    for name, g in (("log_prob", g_lp), ("adcs", g_ad)):
        a = g[pos[:, 0], pos[:, 1], pos[:, 2]]
        b = gold[f"prob/fd_{name}"]
        assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max(), name
    # the clamped entries (log-probability below log(1e-10)) carry none
    lp = prob_loss_inputs()[1]
    clamped = lp[pos[:, 0], pos[:, 1], pos[:, 2]] < np.log(np.float32(1e-10))
    assert clamped.any() and (g_lp[pos[:, 0], pos[:, 1], pos[:, 2]][clamped] == 0).all()


def test_llhd_loss_matches_reference(gold):
    args = llhd_inputs()
    loss, _ = PL.llhd_loss(*args)
    assert abs(loss - float(gold["llhd/loss32"])) <= 2e-7 * abs(loss)
    g = PL.llhd_loss_grad(*args)
    tk = args[1]
    rows = np.arange(16)
    k = np.minimum(tk[:16], args[0].shape[1] - 1)
    for name, a in (("ticks_prob", g[0][rows, k]), ("no_hit_prob", g[1][:16]), ("charge", g[2][rows, k]),
                    ("charge_mc", g[3][:16])):
        b = gold[f"llhd/fd_{name}"]
        assert np.abs(a - b).max() <= 1e-5 * max(np.abs(b).max(), 1e-12), name


def test_jax_index_semantics():
    assert PL.jax_index([-1, -5, 0, 3, 7, 100], 5).tolist() == [4, 0, 0, 3, 4, 4]


def test_prob_llhd_hand_case(cst):
    """Two simulated pixels, distributions of 2 hits x 6 ticks; target hits:
    three on pixel 9 (the third clamps to hit row 1), one on an absent
    pixel (penalty), one pad (-1, matched by the pad row: no penalty), one
    with a negative tick (reads tick 5)."""
    sim = np.array([-1, 4, 9], np.int32)
    lp = np.full((3, 2, 6), -2.0, np.float32)
    lp[2, 1, 3] = -50.0                      # below log(eps): clamped
    ad = np.full((3, 2, 6), 100.0, np.float32)
    tp = np.array([4, 9, 9, 9, 11, -1], np.int32)
    tt = np.array([-1, 0, 1, 3, 2, 0], np.float32)
    ta = np.full(6, 100.0, np.float32)
    loss, aux = PL.prob_llhd(sim, lp, ad, tp, tt, ta, cst)
    le = float(np.log(np.float32(1e-10)))
    T = 3 * -2.0 + le + le * 1                # hits on 4 and 9 (x2), the clamped one, one miss
    assert abs(aux["log_likelihood_tick"] + T) < 1e-4
    assert abs(aux["no_match_penalty"] + le) < 1e-6
    g_lp, g_ad = PL.prob_llhd_grad(sim, lp, ad, tp, tt, ta, cst)
    assert g_lp[1, 0, 5] != 0 and g_lp[2, 0, 0] != 0 and g_lp[2, 1, 1] != 0 and g_lp[2, 1, 3] == 0
    assert loss > 0


def _collapsed_oracle(params, pred, tgt, collapsed, threshold=1e-8):
    """CollapsedProbabilisticLossStrategy.compute (strategies.py:262-335)
    with mse_adc, composed from the oracle's pieces."""
    from oracle import losses_np as L
    from oracle import reference_np as R
    tp, ad = pred["hit_prob"], pred["adcs_distrib"]
    P, H, T = tp.shape
    if collapsed:
        et, ea, hp = R.get_average_hit_values(tp, ad)
        Q = R.adc2charge(ea, params)
        z = R.get_hit_z(params, et, np.repeat(pred["pixel_plane"][:, None], H, axis=1))
        rep = lambda v: np.repeat(np.asarray(v)[:, None], H, axis=1)   # noqa: E731
    else:
        mask = tp > np.float32(threshold)
        hp = tp[mask]
        Q = R.adc2charge(ad[mask], params)
        ticks = np.broadcast_to(np.arange(T, dtype=np.float32), tp.shape)[mask]
        z = R.get_hit_z(params, ticks, np.broadcast_to(pred["pixel_plane"][:, None, None], tp.shape)[mask])
        rep = lambda v: np.broadcast_to(np.asarray(v)[:, None, None], tp.shape)[mask]   # noqa: E731
    x = rep(pred["pixel_x"]).astype(np.float32)
    y = rep(pred["pixel_y"]).astype(np.float32)
    ev = rep(pred["event"])
    ref_Q = R.adc2charge(tgt["adcs"], params)
    return L.mse_adc(np.ravel(Q), np.ravel(x), np.ravel(y), np.ravel(z), np.ravel(hp), np.ravel(ev), ref_Q,
                     tgt["pixel_x"], tgt["pixel_y"], tgt["pixel_z"], tgt["hit_prob"], tgt["event"])[0]


@pytest.mark.parametrize("name,sparse,collapsed", [("collapsed", False, True), ("entries", True, False)])
def test_collapsed_strategy_oracle_matches_reference(gold, name, sparse, collapsed):
    from make_prob_loss_golden import collapsed_inputs
    pred, tgt = collapsed_inputs(sparse=sparse)
    v = _collapsed_oracle(consts.Params(), pred, tgt, collapsed)
    ref = float(gold[f"{name}/loss32"])
    assert abs(v - ref) <= 1e-5 * abs(ref), (v, ref)
