"""The parametrised-mode gradient oracle against derivatives of the
reference's own code.

tests/golden/param_grad_ref.npz holds central differences of the
functional sum(c * W) (c seeded standard normals over the simulated rows,
W the waveforms simulate_parametrized hands to its front end) with respect
to the 8 parameters, from the reference's source run in float64 on the
numpy stand-in for jax with the diffusion draws of tests/golden/param_ref.npz
held fixed, at steps across which no pixel or t0 tick changes
(tests/golden/make_param_grad_golden.py).  The oracle (oracle/grad64.py
param_waveforms64, complex step) must freeze the same pixels and t0 ticks,
give exactly zero for vdrift (never read) and each other component within
5e-4 relative.  Observed: 3e-5 to 2e-4, largest for the parameters that
scale the charge (Ab, kb, lArDensity, lifetime), whose derivative is
proportional to the waveform values: the two float64 evaluations agree to
1e-6 of a row's scale at the median tick and to 4e-7 in each row's sum,
but differ by up to 1.5e-4 of the scale at a few ticks, where the oracle
evaluates from the float32 inputs a 32-bit run sees.
"""

import json
from pathlib import Path

import numpy as np

from oracle import grad64 as G
from test_oracle_param_golden import GOLD as PARAM_GOLD
from test_oracle_param_golden import param_setup

GOLD = Path(__file__).resolve().parent / "golden" / "param_grad_ref.npz"


def test_parametrized_gradient_matches_reference_central_differences():
    gold = np.load(GOLD)
    cfg = json.loads(str(gold["config"]))
    p0, tracks, fields, draws = param_setup(np.load(PARAM_GOLD), cfg["case"])
    p = p0.replace(**dict(zip(cfg["grad_params"], gold["theta"].tolist())))
    th = G.theta_dict(p)
    W, fr, pixels = G.param_waveforms64(p, tracks, fields, draws, th)
    np.testing.assert_array_equal(np.asarray(pixels), gold["pixels"])
    np.testing.assert_array_equal(fr["t0_tick"], gold["t0_tick"])
    cot = np.random.default_rng(cfg["cot_seed"]).standard_normal(W.shape)
    for k, ref in zip(cfg["grad_params"], gold["fd_vjp"]):
        tc = {q: complex(v) for q, v in th.items()}
        h = 1e-30 * abs(th[k])
        tc[k] = th[k] + 1j * h
        got = float((G.param_waveforms64(p, tracks, fields, draws, tc, fr)[0] * cot).sum().imag / h)
        if k == "vdrift":
            assert ref == 0.0 and got == 0.0
        else:
            assert abs(got - ref) <= 5e-4 * abs(ref), (k, got, ref)
