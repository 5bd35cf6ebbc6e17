"""The oracle's LUT path against the reference's own source code.

tests/golden/lut_ref.npz holds the outputs of larnd-sim-jax's load_lut,
simulate_wfs, get_adc_values, digitize and simulate_stochastic on seeded
events (tests/golden/make_lut_golden.py: the reference's modules run in a
process without JAX, with a numpy stand-in for jax).  The oracle
(oracle/reference_np.py) must reproduce them on the same inputs:

* template bank samples and per-template sums within 1e-5 relative;
* unique_pixels identical;
* waveforms within 1e-5 of each simulated row's largest |w| (observed
  5e-7 to 8e-7: summation order), and the rows of pixel id -1, where the
  reference collects every unmatched neighbour contribution, within 1e-5
  of their own largest |w|;
* the front end on the reference's own waveforms bit for bit: crossing
  ticks, integrals and digitised values;
* the whole chain: hit count, pixel ids, events, ticks, hit probabilities,
  pixel centres and hit z bit for bit; ADCs within 1e-5 relative (observed
  2e-7, from the waveforms' summation order).
"""

import json
import zlib
from pathlib import Path

import numpy as np
import pytest

from larndsim_gb300 import consts, workloads
from oracle import reference_np as R

GOLD = Path(__file__).resolve().parent / "golden" / "lut_ref.npz"
HIT_KEYS = ("adcs", "pixel_x", "pixel_y", "pixel_z", "ticks", "hit_prob", "event", "pixels")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _cases():
    with np.load(GOLD) as g:
        return sorted({k.split("/")[0] for k in g.files})


def _setup(gold, name, strict=True):
    """The case's options, oracle parameters, response LUT, tracks and
    fields.  ``strict``: skip where this platform's numpy makes a response
    LUT that differs in its last bits from the one the golden file used
    (the bit-for-bit assertions need the same inputs)."""
    cfg = json.loads(str(gold[f"{name}/config"]))
    resp = workloads.synthetic_response(seed=cfg["response_seed"], nx=cfg["lut"], ny=cfg["lut"])
    if strict and zlib.crc32(np.ascontiguousarray(resp, np.float32).tobytes()) != cfg["response_crc32"]:
        pytest.skip("the synthetic response LUT differs from the one the golden file was made with on this platform")
    params = consts.Params(number_pix_neighbors=cfg["n"], signal_length=cfg["L"], time_window=cfg["L"],
                           RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0,
                           recombination_mode=getattr(consts.RecombinationMode, cfg["mode"]),
                           long_diff_template=consts.jax_linspace_f32(0.001, 10, cfg["n_templates"]))
    return cfg, params, resp, gold[f"{name}/tracks"], tuple(cfg["fields"])


def _dense_wfs(gold, name):
    w = np.zeros(tuple(gold[f"{name}/wfs_shape"]), np.float32)
    w[gold[f"{name}/wfs_row"], gold[f"{name}/wfs_tick"].astype(np.int64)] = gold[f"{name}/wfs_value"]
    return w


@pytest.mark.parametrize("name", _cases())
def test_templates_match_reference_load_lut(gold, name):
    cfg, params, resp, _, _ = _setup(gold, name)
    tmpl = R.load_lut_templates(resp, params)
    ref = gold[f"{name}/tmpl_value"]
    got = tmpl.ravel()[gold[f"{name}/tmpl_index"]]
    scale = np.abs(tmpl).max()
    assert np.abs(got - ref).max() <= 1e-5 * scale
    sums = tmpl.astype(np.float64).reshape(tmpl.shape[0], -1).sum(axis=1)
    np.testing.assert_allclose(sums, gold[f"{name}/tmpl_sum"], rtol=1e-5)


@pytest.mark.parametrize("name", _cases())
def test_waveforms_match_reference_simulate_wfs(gold, name):
    cfg, params, resp, tracks, fields = _setup(gold, name)
    tmpl = R.load_lut_templates(resp, params)
    wfs, unique = R.simulate_wfs(params, tmpl, tracks, fields, history={})
    np.testing.assert_array_equal(unique, gold[f"{name}/unique_pixels"])
    ref = _dense_wfs(gold, name)
    assert wfs.shape == ref.shape
    valid = unique >= 0
    scale = np.abs(ref[valid]).max(axis=1, keepdims=True)
    assert (scale > 0).all()
    err = np.abs(wfs[valid] - ref[valid]) / scale
    assert err.max() <= 1e-5, f"waveforms differ by {err.max():.3g} of the row scale"
    if (~valid).any():
        garbage = np.abs(ref[~valid]).max()
        assert np.abs(wfs[~valid] - ref[~valid]).max() <= 1e-5 * garbage


@pytest.mark.parametrize("name", _cases())
def test_front_end_matches_reference_on_its_waveforms(gold, name):
    """get_adc_values + digitize on the reference's own waveforms: the
    crossing search, the integration window and the reset are restated
    exactly, so every tick agrees."""
    cfg, params, _, _, _ = _setup(gold, name)
    integral, ticks = R.get_adc_values(params, _dense_wfs(gold, name))
    np.testing.assert_array_equal(ticks, gold[f"{name}/ticks"])
    np.testing.assert_array_equal(integral.view(np.uint32), gold[f"{name}/integral"].view(np.uint32))
    adcs = R.digitize(params, gold[f"{name}/integral"])
    np.testing.assert_array_equal(adcs.view(np.uint32), gold[f"{name}/grid_adcs"].view(np.uint32))
    assert (ticks < 1997).any(), "no pixel crossed the threshold"


@pytest.mark.parametrize("name", _cases())
def test_chain_matches_reference_simulate_stochastic(gold, name):
    cfg, params, resp, tracks, fields = _setup(gold, name)
    tmpl = R.load_lut_templates(resp, params)
    wfs, unique = R.simulate_wfs(params, tmpl, tracks, fields, history={})
    out = R.simulate_stochastic(params, wfs, unique)
    ref = {k: gold[f"{name}/hits_{k}"] for k in HIT_KEYS}
    assert out["nb_valid"] == ref["adcs"].shape[0] > 0
    for k in ("ticks", "hit_prob", "event", "pixels", "pixel_x", "pixel_y", "pixel_z"):
        np.testing.assert_array_equal(np.asarray(out[k]), ref[k], err_msg=k)
    np.testing.assert_allclose(out["adcs"], ref["adcs"], rtol=1e-5, atol=0)
