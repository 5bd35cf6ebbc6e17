"""The oracle's probabilistic front end against the reference's own source.

tests/golden/prob_ref.npz holds what larnd-sim-jax's
get_adc_values_average_noise_vmap, simulate_probabilistic and
get_average_hit_values return on rows of the reference's own waveforms
(tests/golden/make_prob_golden.py: the reference's modules run with a numpy
stand-in for jax whose log_ndtr is scipy's, evaluated in float64 and
rounded, where the oracle restates JAX's float32 piecewise form).  On the
same rows the oracle must give:

* the expected charge of every entry with probability above 1e-6 bit for
  bit (the paths chosen by the top-K selection are the same);
* probabilities exp(log p) within 5e-5 absolute (observed 1e-5) and log p
  within 5e-4 above -5 (observed 6e-5); below -5 the two log_ndtr
  evaluations meet float32 cancellation in log(Phi(a) - Phi(b)) (observed
  1-15 % relative at weights under e^-5), so there only the support is
  compared: the entries above -59 are the ones the reference keeps above -60;
* per (pixel, hit) the total probability within 1e-4 and the expected tick
  and ADC within 1e-5 relative where the total probability exceeds 1e-3;
* pixel centres and events bit for bit.
"""

import json
from pathlib import Path

import numpy as np
import pytest

from larndsim_gb300 import consts
from oracle import reference_np as R

GOLD = Path(__file__).resolve().parent / "golden" / "prob_ref.npz"
PROB_ATOL = 5e-5
LOGP_ATOL = 5e-4
LAMBDA_ATOL = 1e-4
EXPECTED_RTOL = 1e-5


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def prob_cases():
    with np.load(GOLD) as g:
        return sorted({k.split("/")[0] for k in g.files})


def prob_setup(gold, name):
    """The case's parameters, waveform rows, their pixel ids and the index
    of the stored distribution entries."""
    cfg = json.loads(str(gold[f"{name}/config"]))
    params = consts.Params(number_pix_neighbors=cfg["n"], RESET_NOISE_CHARGE=cfg["reset_noise"],
                           UNCORRELATED_NOISE_CHARGE=0, fee_paths_scaling=cfg["fee_paths_scaling"],
                           long_diff_template=consts.jax_linspace_f32(0.001, 10, cfg["n_templates"]))
    rows = np.zeros(tuple(gold[f"{name}/rows_shape"]), np.float32)
    rows[gold[f"{name}/rows_row"], gold[f"{name}/rows_tick"].astype(np.int64)] = gold[f"{name}/rows_value"]
    keep = (gold[f"{name}/keep_pixel"].astype(np.int64), gold[f"{name}/keep_hit"].astype(np.int64),
            gold[f"{name}/keep_tick"].astype(np.int64))
    return cfg, params, rows, gold[f"{name}/row_pixels"], keep


def check_distributions(log_prob, charge, gold, name, keep, cfg, charge_rtol=0.0, support_margin=(1.0, 10.0)):
    """The comparisons of the module docstring on (P, H, T-1) arrays.
    ``charge_rtol`` 0 asks for identical charges, else a bound relative to
    the largest charge; ``support_margin`` (a, b): no entry outside the
    reference's kept set lies above -60 + a, and every kept entry lies
    above -60 - b."""
    assert log_prob.shape == tuple(gold[f"{name}/dist_shape"])
    ref_lp = gold[f"{name}/log_prob"]
    lp = log_prob[keep]
    assert np.abs(np.exp(lp.astype(np.float64)) - np.exp(ref_lp.astype(np.float64))).max() <= PROB_ATOL
    top = ref_lp > -5
    assert top.sum() > 100
    assert np.abs(lp - ref_lp)[top].max() <= LOGP_ATOL
    kept = np.zeros(log_prob.shape, bool)
    kept[keep] = True
    assert not (log_prob[~kept] > cfg["keep_logp"] + support_margin[0]).any(), "entries the reference holds below -60"
    assert (lp > cfg["keep_logp"] - support_margin[1]).all(), "entries the reference holds above -60"
    sig = np.exp(ref_lp.astype(np.float64)) > 1e-6
    ref_q = gold[f"{name}/charge"]
    if charge_rtol == 0.0:
        np.testing.assert_array_equal(charge[keep][sig], ref_q[sig])
    else:
        scale = np.abs(ref_q).max()
        assert np.abs(charge[keep][sig] - ref_q[sig]).max() <= charge_rtol * scale


def check_expected(e_tick, e_adc, lam, gold, name, rtol=EXPECTED_RTOL):
    ref_lam = gold[f"{name}/lambda"]
    assert np.abs(lam - ref_lam).max() <= LAMBDA_ATOL
    m = ref_lam > 1e-3
    assert m.sum() > 10
    np.testing.assert_allclose(e_tick[m], gold[f"{name}/expected_ticks"][m], rtol=rtol)
    np.testing.assert_allclose(e_adc[m], gold[f"{name}/expected_adcs"][m], rtol=rtol)


@pytest.mark.parametrize("name", prob_cases())
def test_beam_search_matches_reference_source(gold, name):
    cfg, params, rows, _, keep = prob_setup(gold, name)
    log_prob, charge = R.get_adc_values_average_noise(params, rows)
    check_distributions(log_prob, charge, gold, name, keep, cfg)
    e_tick, e_adc, lam = R.get_average_hit_values(np.exp(log_prob), R.digitize(params, charge))
    check_expected(e_tick, e_adc, lam, gold, name)


@pytest.mark.parametrize("name", prob_cases())
def test_simulate_probabilistic_matches_reference_source(gold, name):
    cfg, params, rows, pixels, keep = prob_setup(gold, name)
    adcs, px, py, log_prob, event = R.simulate_probabilistic(params, rows, pixels)
    np.testing.assert_array_equal(px, gold[f"{name}/pixel_x"])
    np.testing.assert_array_equal(py, gold[f"{name}/pixel_y"])
    np.testing.assert_array_equal(event, gold[f"{name}/event"])
    sig = np.exp(gold[f"{name}/log_prob"].astype(np.float64)) > 1e-6
    np.testing.assert_allclose(adcs[keep][sig], gold[f"{name}/adcs"][sig], rtol=1e-6)
