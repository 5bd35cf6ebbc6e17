"""The oracle's fit losses against the reference's own source.

tests/golden/loss_ref.npz holds what larnd-sim-jax's mse_adc, chamfer_3d
and nll_loss return on two hit sets (the reference's own simulated hits and
a seeded perturbation of them; tests/golden/make_loss_golden.py, the
reference's modules run with a numpy stand-in for jax): the loss of a
32-bit run, the loss of a run with 64-bit types on the same float32-stacked
coordinates, and central differences of the latter with respect to Q, z
(and hit_prob for nll_loss) of 12 predicted hits.  The oracle
(oracle/losses_np.py) must give the 64-bit value within 1e-7 relative
(observed: mse_adc identical, 8e-9 and 2e-9), the 32-bit value within
1e-5 (float32 rounding of the reference's own evaluation, observed 2e-7),
and the gradient components within 1e-6 of the largest of them.
"""

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import losses_np as L

GOLD = Path(__file__).resolve().parent / "golden" / "loss_ref.npz"
COLS = ("Q", "x", "y", "z", "ticks", "hit_prob", "event")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def hit_columns(gold):
    """(predicted, reference) hit columns of the golden file."""
    return ({k: gold[f"pred_{k}"] for k in COLS}, {k: gold[f"ref_{k}"] for k in COLS})


def chamfer_pad(n_pred, n_ref):
    """pad_size's first bucket for (reference, prediction) sizes with an
    empty history (sim_jax.py:61-102, pad_threshold 0.05)."""
    return int(n_pred * 1.025 + 0.5), int(n_ref * 1.025 + 0.5)


def _check(gold, name, loss, grads):
    n_fd = json.loads(str(gold["config"]))["n_fd"]
    assert abs(loss - float(gold[f"{name}/loss64"])) <= 1e-7 * abs(float(gold[f"{name}/loss64"]))
    assert abs(loss - float(gold[f"{name}/loss32"])) <= 1e-5 * abs(float(gold[f"{name}/loss32"]))
    for col, g in grads.items():
        fd = gold[f"{name}/fd_{col}"]
        assert np.abs(np.asarray(g)[:n_fd] - fd).max() <= 1e-6 * np.abs(fd).max(), col


def test_mse_adc_matches_reference_source(gold):
    P, R = hit_columns(gold)
    loss, _, _ = L.mse_adc(P["Q"], P["x"], P["y"], P["z"], P["hit_prob"], P["event"], R["Q"], R["x"], R["y"],
                           R["z"], R["hit_prob"], R["event"])
    gw, gz = L.mse_adc_grad(P["Q"].astype(np.float64) * P["hit_prob"], P["x"], P["y"], P["z"], P["event"],
                            R["Q"].astype(np.float64) * R["hit_prob"], R["x"], R["y"], R["z"], R["event"])
    _check(gold, "mse_adc", loss, {"Q": gw * P["hit_prob"], "z": gz})


def test_chamfer_3d_matches_reference_source(gold):
    P, R = hit_columns(gold)
    loss, gq, gz = L.chamfer_3d(P["Q"], P["x"], P["y"], P["z"], P["event"], R["Q"], R["x"], R["y"], R["z"],
                                R["event"], pad_to=chamfer_pad(len(P["Q"]), len(R["Q"])))
    _check(gold, "chamfer_3d", loss, {"Q": gq, "z": gz})


def test_nll_loss_matches_reference_source(gold):
    P, R = hit_columns(gold)
    loss, gq, gz, ghp = L.nll_loss(P["Q"], P["x"], P["y"], P["z"], P["hit_prob"], P["event"], R["Q"], R["x"],
                                   R["y"], R["z"], R["hit_prob"], R["event"])
    _check(gold, "nll_loss", loss, {"Q": gq, "z": gz, "hit_prob": ghp})
