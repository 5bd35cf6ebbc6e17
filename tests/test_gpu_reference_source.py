"""The CUDA LUT and parametrised paths against outputs of the reference's
own source code.

tests/golden/lut_ref.npz holds what larnd-sim-jax's load_lut,
simulate_wfs, get_adc_values, digitize and simulate_stochastic return on
seeded events (made by tests/golden/make_lut_golden.py, which runs the
reference's modules with a numpy stand-in for jax; the oracle reproduces
them, tests/test_oracle_lut_golden.py).  Here the same inputs go through
this package's load_lut, simulate_wfs, get_adc_values and
simulate_stochastic on the GPU, at the tolerances of the other parity
tests: template bank within 2e-5 relative (2e-6 of its largest value),
unique_pixels identical, waveforms within 1e-5 of each simulated row's
largest |w|, hit ticks identical except near-threshold crossings (under
0.5 % of the hit slots), ADCs within 1e-5 relative.  The waveform and hit
comparisons use the oracle's template bank, as the other parity tests do.
The cases at signal_length 150 run here; the signal_length 100 case is
checked by the oracle test only.  The parametrised-mode cases
(tests/golden/param_ref.npz, tests/golden/make_param_golden.py) run
simulate_parametrized with the diffusion draws the reference made.  The
probabilistic front end (tests/golden/prob_ref.npz,
tests/golden/make_prob_golden.py) runs at the default 20 paths with the
tolerances of tests/test_gpu_fee_prob.py.  The gradient
(tests/golden/grad_ref.npz, tests/golden/make_grad_golden.py: central
differences of the reference's own chain in float64 at fixed decisions)
is compared as the vector-Jacobian product for the reference's cotangent,
within 1e-4 relative per component (the gradient tolerance of the
reference-parity contract), at number_pix_neighbors 1, 2 and 4.  The fit losses
(tests/golden/loss_ref.npz, tests/golden/make_loss_golden.py) are compared
at the tolerances of tests/test_gpu_losses.py: values within 1e-5
relative, gradients within 1e-4 of the largest central difference.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_common import ADC_RTOL, WFS_RTOL, compare_fee, compare_wfs
from test_oracle_lut_golden import GOLD, HIT_KEYS, _cases, _dense_wfs, _setup
from test_oracle_param_golden import GOLD as PARAM_GOLD
from test_oracle_param_golden import param_cases, param_dense_wfs, param_setup
from test_oracle_prob_golden import GOLD as PROB_GOLD
from test_oracle_prob_golden import check_distributions, check_expected, prob_cases, prob_setup
from test_oracle_grad_golden import GOLD as GRAD_GOLD
from test_oracle_grad_golden import grad_cases, grad_setup
from test_oracle_loss_golden import GOLD as LOSS_GOLD
from test_oracle_loss_golden import COLS as LOSS_COLS

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _gpu_cases():
    with np.load(GOLD) as g:
        import json
        return [n for n in _cases() if json.loads(str(g[f"{n}/config"]))["L"] == 150]


@pytest.mark.parametrize("name", _gpu_cases())
def test_cuda_lut_path_matches_reference_source(cuda, gold, name):
    from larndsim_gb300 import sim
    from oracle import reference_np as R
    cfg, p, resp, tracks, fields = _setup(gold, name, strict=False)

    tmpl_gpu, _ = sim.load_lut(resp, p)
    got = tmpl_gpu.cpu().numpy().ravel()[gold[f"{name}/tmpl_index"]]
    ref = gold[f"{name}/tmpl_value"]
    np.testing.assert_allclose(got, ref, rtol=2e-5, atol=2e-6 * float(tmpl_gpu.abs().max()))

    tmpl = torch.from_numpy(R.load_lut_templates(resp, p)).cuda()
    sim.reset_size_history()
    wfs, unique = sim.simulate_wfs(p, tmpl, tracks, fields)
    w, u = wfs.cpu().numpy(), unique.cpu().numpy()
    ref_w = _dense_wfs(gold, name)
    assert compare_wfs(w, u, ref_w, gold[f"{name}/unique_pixels"]) < WFS_RTOL
    assert np.all(w[u < 0] == 0)          # rows of negative pixel id are zero here by design

    # the front end on the reference's own waveforms
    integral, ticks = sim.get_adc_values(p, torch.from_numpy(ref_w).cuda())
    frac, err = compare_fee(integral.cpu().numpy(), ticks.cpu().numpy(), gold[f"{name}/integral"],
                            gold[f"{name}/ticks"], p)
    assert frac < 0.005 and err < ADC_RTOL, (frac, err)

    # the whole chain, on the simulated rows (parse_output drops the rows of
    # negative pixel id, which are zero here and hold the reference's
    # unmatched neighbour charge there)
    out, (grid_adcs, grid_ticks) = sim.simulate_stochastic(p, wfs, unique, 0, return_grids=True)
    v = u >= 0
    frac, err = compare_fee(grid_adcs.cpu().numpy()[v], grid_ticks.cpu().numpy()[v], gold[f"{name}/grid_adcs"][v],
                            gold[f"{name}/ticks"][v])
    assert frac < 0.005 and err < ADC_RTOL, (frac, err)
    if frac == 0:
        hits = {k: v.cpu().numpy() for k, v in zip(HIT_KEYS, out)}
        ref_hits = {k: gold[f"{name}/hits_{k}"] for k in HIT_KEYS}
        assert hits["adcs"].shape == ref_hits["adcs"].shape
        for k in ("pixels", "event", "ticks", "hit_prob"):
            np.testing.assert_array_equal(hits[k], ref_hits[k], err_msg=k)
        np.testing.assert_allclose(hits["adcs"], ref_hits["adcs"], rtol=ADC_RTOL)
        for k in ("pixel_x", "pixel_y", "pixel_z"):
            np.testing.assert_allclose(hits[k], ref_hits[k], rtol=3e-7, atol=3e-6, err_msg=k)


@pytest.mark.parametrize("name", param_cases())
def test_cuda_parametrized_path_matches_reference_source(cuda, name):
    """simulate_parametrized on the GPU with the diffusion draws the
    reference used (tests/golden/param_ref.npz)."""
    from larndsim_gb300 import sim
    pgold = np.load(PARAM_GOLD)
    p, tracks, fields, draws = param_setup(pgold, name)
    sim.reset_size_history()
    out, wfs, unique = sim.simulate_parametrized(p, tracks, fields, offsets=torch.from_numpy(draws).cuda(),
                                                 return_wfs=True)
    w, u = wfs.cpu().numpy(), unique.cpu().numpy()
    ref_w = param_dense_wfs(pgold, name)
    assert compare_wfs(w, u, ref_w, pgold[f"{name}/unique_pixels"]) < WFS_RTOL
    integral, ticks = sim.get_adc_values(p, torch.from_numpy(ref_w).cuda())
    frac, err = compare_fee(integral.cpu().numpy(), ticks.cpu().numpy(), pgold[f"{name}/integral"],
                            pgold[f"{name}/ticks"], p)
    assert frac < 0.005 and err < ADC_RTOL, (frac, err)
    hits = {k: v.cpu().numpy() for k, v in zip(HIT_KEYS, out)}
    ref_hits = {k: pgold[f"{name}/hits_{k}"] for k in HIT_KEYS}
    if hits["adcs"].shape == ref_hits["adcs"].shape and np.array_equal(hits["ticks"], ref_hits["ticks"]):
        for k in ("pixels", "event", "hit_prob"):
            np.testing.assert_array_equal(hits[k], ref_hits[k], err_msg=k)
        np.testing.assert_allclose(hits["adcs"], ref_hits["adcs"], rtol=ADC_RTOL)
        for k in ("pixel_x", "pixel_y", "pixel_z"):
            np.testing.assert_allclose(hits[k], ref_hits[k], rtol=3e-7, atol=3e-6, err_msg=k)
    else:
        # a near-threshold crossing moved: at most a few hit slots differ
        n_ref = ref_hits["adcs"].shape[0]
        assert abs(hits["adcs"].shape[0] - n_ref) <= max(1, n_ref // 200)


def _prob_cases_default_paths():
    import json
    with np.load(PROB_GOLD) as g:
        return [n for n in prob_cases() if json.loads(str(g[f"{n}/config"]))["fee_paths_scaling"] == 20]


@pytest.mark.parametrize("name", _prob_cases_default_paths())
def test_cuda_probabilistic_front_end_matches_reference_source(cuda, name):
    """The beam search, the fused expected values and
    simulate_probabilistic on the GPU, on rows of the reference's own
    waveforms."""
    from larndsim_gb300 import sim
    pgold = np.load(PROB_GOLD)
    cfg, p, rows, pixels, keep = prob_setup(pgold, name)
    w = torch.from_numpy(rows).cuda()
    log_prob, charge = sim.get_adc_values_average_noise_vmap(p, w)
    check_distributions(log_prob.cpu().numpy(), charge.cpu().numpy(), pgold, name, keep, cfg, charge_rtol=1e-5,
                        support_margin=(20.0, 20.0))
    e_tick, e_adc, lam = (t.cpu().numpy() for t in sim.average_hit_values(p, w))
    check_expected(e_tick, e_adc, lam, pgold, name, rtol=1e-3)
    _, px, py, _, event = sim.simulate_probabilistic(p, w, torch.from_numpy(pixels).cuda())
    real = pixels >= 0                      # the all-zero row carries pixel id -1
    np.testing.assert_allclose(px.cpu().numpy()[real], pgold[f"{name}/pixel_x"][real], rtol=3e-7, atol=3e-6)
    np.testing.assert_allclose(py.cpu().numpy()[real], pgold[f"{name}/pixel_y"][real], rtol=3e-7, atol=3e-6)
    np.testing.assert_array_equal(event.cpu().numpy()[real], pgold[f"{name}/event"][real])


@pytest.mark.parametrize("name", grad_cases())
def test_cuda_gradient_matches_reference_central_differences(cuda, name):
    from larndsim_gb300 import grad
    ggold = np.load(GRAD_GOLD)
    cfg, p, tmpl, tracks, fields = grad_setup(ggold, name)
    chain = grad.LUTChain(p, torch.from_numpy(tmpl).cuda(), tracks, fields)
    adc, ticks, pids = (t.cpu().numpy() for t in chain.adc(p))
    ref_ticks = ggold[f"{name}/ticks32"]
    accepted = ref_ticks < 1998                 # crossings the front end accepted
    if not (np.array_equal(pids, ggold[f"{name}/pixels32"]) and np.array_equal(ticks[accepted], ref_ticks[accepted])):
        pytest.skip("the GPU's float32 forward took another crossing decision than the reference's 32-bit run")
    cot = torch.from_numpy(ggold[f"{name}/cotangent"].astype(np.float32)).cuda()
    got = dict(zip(grad.GRAD_PARAMS, [float(v) for v in chain.vjp(p, cot)]))
    worst = 0.0
    for k, r in zip(cfg["grad_params"], ggold[f"{name}/fd_vjp"]):
        if r == 0.0:
            assert got[k] == 0.0, k
        else:
            worst = max(worst, abs(got[k] - r) / abs(r))
            assert abs(got[k] - r) <= 1e-4 * abs(r), (k, got[k], r)
    print(f"\n{name}: largest relative deviation from the reference's float64 central differences {worst:.2e}")


@pytest.mark.parametrize("name", ["mse_adc", "chamfer_3d", "nll_loss"])
def test_cuda_losses_match_reference_source(cuda, name):
    from larndsim_gb300 import consts, losses, sim
    lgold = np.load(LOSS_GOLD)
    pred = {k: torch.from_numpy(lgold[f"pred_{k}"]).cuda() for k in LOSS_COLS}
    ref = {k: torch.from_numpy(lgold[f"ref_{k}"]).cuda() for k in LOSS_COLS}
    wrt = ("Q", "z", "hit_prob") if name == "nll_loss" else ("Q", "z")
    for k in wrt:
        pred[k] = pred[k].clone().requires_grad_(True)
    sim.reset_size_history()
    loss, _ = getattr(losses, name)(consts.Params(), *[pred[k] for k in LOSS_COLS], *[ref[k] for k in LOSS_COLS])
    loss.backward()
    value = float(loss.detach())
    assert abs(value - float(lgold[f"{name}/loss64"])) <= 1e-5 * abs(float(lgold[f"{name}/loss64"]))
    for k in wrt:
        fd = lgold[f"{name}/fd_{k}"]
        g = pred[k].grad.cpu().numpy()[:fd.shape[0]]
        assert np.abs(g - fd).max() <= 1e-4 * np.abs(fd).max(), k
