"""The oracle's parametrised-current path against the reference's own source.

tests/golden/param_ref.npz holds what larnd-sim-jax's simulate_parametrized
returns on seeded events, with the Monte-Carlo diffusion draws it used and
the waveforms it handed to its front end (tests/golden/make_param_golden.py:
the reference's modules run with a numpy stand-in for jax).  Given the same
draws, the oracle (oracle/reference_np.py) must reproduce:

* unique_pixels identical;
* waveforms within 1e-5 of each simulated row's largest |w| (observed: bit
  for bit in two cases, 2.3e-9 in the third: float32 scatter order);
* the front end on the reference's own waveforms bit for bit;
* the 8 outputs (ADCs, pixel centres, hit z, ticks, hit probabilities,
  events, pixel ids) bit for bit, ADCs within 1e-5 relative.
"""

import json
from pathlib import Path

import numpy as np
import pytest

from larndsim_gb300 import consts
from oracle import reference_np as R

GOLD = Path(__file__).resolve().parent / "golden" / "param_ref.npz"
HIT_KEYS = ("adcs", "pixel_x", "pixel_y", "pixel_z", "ticks", "hit_prob", "event", "pixels")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def param_cases():
    with np.load(GOLD) as g:
        return sorted({k.split("/")[0] for k in g.files})


def param_setup(gold, name):
    """The case's parameters (module0, n = 0, Monte-Carlo diffusion, noise
    off), tracks, fields and recorded diffusion draws."""
    cfg = json.loads(str(gold[f"{name}/config"]))
    params = consts.Params(number_pix_neighbors=0, mc_diff=True, RESET_NOISE_CHARGE=0,
                           UNCORRELATED_NOISE_CHARGE=0,
                           recombination_mode=getattr(consts.RecombinationMode, cfg["mode"]))
    return params, gold[f"{name}/tracks"], tuple(cfg["fields"]), gold[f"{name}/draws"]


def param_dense_wfs(gold, name):
    w = np.zeros(tuple(gold[f"{name}/wfs_shape"]), np.float32)
    w[gold[f"{name}/wfs_row"], gold[f"{name}/wfs_tick"].astype(np.int64)] = gold[f"{name}/wfs_value"]
    return w


@pytest.mark.parametrize("name", param_cases())
def test_parametrized_matches_reference_source(gold, name):
    params, tracks, fields, draws = param_setup(gold, name)
    out = R.simulate_parametrized(params, tracks, fields, draws, history={})
    unique = gold[f"{name}/unique_pixels"]
    np.testing.assert_array_equal(out["unique_pixels"], unique)
    ref = param_dense_wfs(gold, name)
    valid = unique >= 0
    scale = np.abs(ref[valid]).max(axis=1, keepdims=True)
    assert (scale > 0).all()
    assert (np.abs(out["wfs"][valid] - ref[valid]) / scale).max() <= 1e-5
    assert out["nb_valid"] == gold[f"{name}/hits_adcs"].shape[0] > 0
    for k in HIT_KEYS[1:]:
        np.testing.assert_array_equal(np.asarray(out[k]), gold[f"{name}/hits_{k}"], err_msg=k)
    np.testing.assert_allclose(out["adcs"], gold[f"{name}/hits_adcs"], rtol=1e-5, atol=0)


@pytest.mark.parametrize("name", param_cases())
def test_parametrized_front_end_on_reference_waveforms(gold, name):
    params, _, _, _ = param_setup(gold, name)
    integral, ticks = R.get_adc_values(params, param_dense_wfs(gold, name))
    np.testing.assert_array_equal(ticks, gold[f"{name}/ticks"])
    np.testing.assert_array_equal(integral.view(np.uint32), gold[f"{name}/integral"].view(np.uint32))
    assert (ticks < 1997).any(), "no pixel crossed the threshold"
