"""The gradient oracle against derivatives of the reference's own code.

tests/golden/grad_ref.npz holds, for seeded events, central differences of
the reference's LUT chain (simulate_wfs + get_adc_values + digitize) run
in float64 on the numpy stand-in for jax, at perturbed parameters whose
discrete decisions (pixel ids, crossing ticks, transverse bins, cathode
ticks, template indices) equal the 32-bit run's and stay fixed across every
step (tests/golden/make_grad_golden.py).  That is the derivative
jax.value_and_grad takes.  Two functionals are differentiated: the
sum-of-squared-ADC loss against a target at the nominal parameters, and
sum(c * ADC) with c = 2 (ADC - target) from the 32-bit run, the
vector-Jacobian product jax.grad forms for that loss.

The oracle's float64 adjoint (oracle/grad64.py) must give, at the same
parameters and target:

* the 32-bit run's decisions: the same simulated pixels and crossing ticks;
* the vector-Jacobian product for c within 1e-4 relative, component by
  component (observed 1e-7 to 4.3e-5), and exactly zero where the
  reference's derivative is (vdrift, which the reference never reads; Ab
  and kb under the Box model);
* the loss within 1e-3 relative and its gradient within 5e-3 relative per
  component: here the residuals themselves differ by the float32 rounding
  of the forward values (the reference's float32 cumulative sum of the
  template bank moves a waveform by up to about 1e-4 of its scale), and
  the gradient is proportional to them (observed up to 6.4e-4 at
  number_pix_neighbors 1 and 2, 2.9e-3 on d/d long_diff at 4, where 80
  neighbour windows add to each waveform).
"""

import json
from pathlib import Path

import numpy as np
import pytest

from larndsim_gb300 import consts, workloads
from oracle import grad64 as G
from oracle import reference_np as R

GOLD = Path(__file__).resolve().parent / "golden" / "grad_ref.npz"
VJP_RTOL = 1e-4


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def grad_cases():
    with np.load(GOLD) as g:
        return sorted({k.split("/")[0] for k in g.files})


def grad_setup(gold, name):
    """Parameters at the case's perturbed values, the oracle's template
    bank, tracks and fields."""
    cfg = json.loads(str(gold[f"{name}/config"]))
    theta = dict(zip(cfg["grad_params"], gold[f"{name}/theta"].tolist()))
    params = consts.Params(number_pix_neighbors=cfg["n"], signal_length=cfg["L"], time_window=cfg["L"],
                           RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0,
                           recombination_mode=getattr(consts.RecombinationMode, cfg["mode"]),
                           long_diff_template=consts.jax_linspace_f32(0.001, 10, cfg["n_templates"]), **theta)
    resp = workloads.synthetic_response(seed=cfg["response_seed"], nx=cfg["lut"], ny=cfg["lut"])
    return cfg, params, R.load_lut_templates(resp, params), gold[f"{name}/tracks"], tuple(cfg["fields"])


@pytest.fixture(scope="module")
def frozen(gold):
    out = {}
    for name in grad_cases():
        cfg, params, tmpl, tracks, fields = grad_setup(gold, name)
        fr = G.Frozen(params, tmpl, tracks, fields, gold[f"{name}/target_pixels"], gold[f"{name}/target_adc"])
        out[name] = (cfg, fr, G.theta_dict(params))
    return out


@pytest.mark.parametrize("name", grad_cases())
def test_oracle_takes_the_reference_decisions(gold, frozen, name):
    cfg, fr, _ = frozen[name]
    np.testing.assert_array_equal(fr.unique[fr.valid], gold[f"{name}/pixels32"])
    T = fr.masks.shape[2]
    ticks = np.where(fr.cond, T - 2, fr.idx)[fr.valid]
    np.testing.assert_array_equal(ticks, gold[f"{name}/ticks32"])


@pytest.mark.parametrize("name", grad_cases())
def test_vjp_matches_reference_central_differences(gold, frozen, name):
    cfg, fr, th = frozen[name]
    got = G.adjoint64(fr, th, g_adc=gold[f"{name}/cotangent"])
    ref = dict(zip(cfg["grad_params"], gold[f"{name}/fd_vjp"]))
    for k, r in ref.items():
        if r == 0.0:
            assert got[k] == 0.0, k
        else:
            assert abs(got[k] - r) <= VJP_RTOL * abs(r), (k, got[k], r)
    assert ref["vdrift"] == 0.0
    if cfg["mode"] == "BOX":
        assert ref["Ab"] == 0.0 and ref["kb"] == 0.0


@pytest.mark.parametrize("name", grad_cases())
def test_loss_gradient_matches_reference_central_differences(gold, frozen, name):
    cfg, fr, th = frozen[name]
    assert abs(G.loss64(fr, th) - float(gold[f"{name}/loss"])) <= 1e-3 * float(gold[f"{name}/loss"])
    got = G.adjoint64(fr, th)
    for k, r in zip(cfg["grad_params"], gold[f"{name}/fd_gradient"]):
        assert abs(got[k] - r) <= 5e-3 * abs(r), (k, got[k], r)
