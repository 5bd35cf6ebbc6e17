"""Device-resident fit loop (optimize/fit_params.py:704-731, :781-895):
the segment stage with device-side parameters, the gradient and the
optimiser update, captured in one CUDA graph.  The graph replays the eager
trajectory exactly; the fit step follows the reference's chain (the
sigmoid, exp_log and divide normalisations, NaN skip, clip_by_global_norm,
optax.adam, clip_values_from_range) restated below in float64; a fit with
the reference's default settings recovers hidden parameters."""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    from larndsim_gb300 import consts, grad, sim, workloads
    p = consts.Params(number_pix_neighbors=4, RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0)
    tmpl, p = sim.load_lut(workloads.synthetic_response(seed=0), p)
    tracks, fields = workloads.batched_events(seed=5, n_events=8, min_segments=2000, max_segments=2001)
    hidden = p.replace(lifetime=float(p.lifetime) * 1.021, long_diff=float(p.long_diff) * 0.883,
                       tran_diff=float(p.tran_diff) * 1.029)
    target = grad.LUTChain(p, tmpl, tracks, fields).target(hidden)
    return p, tmpl, tracks, fields, hidden, target


def test_adam_step_matches_optax_formula(cuda):
    from larndsim_gb300 import _abi
    lib = _abi.load()
    rng = np.random.default_rng(0)
    theta = rng.uniform(0.5, 2.0, 8).astype(np.float32)
    scale = rng.uniform(0.1, 3.0, 8).astype(np.float32)
    lr = np.where(np.arange(8) == 4, 0.0, 0.01).astype(np.float32)
    t_th, t_sc, t_lr = (torch.from_numpy(a).cuda() for a in (theta, scale, lr))
    state = torch.zeros(17, dtype=torch.float32, device="cuda")
    m = np.zeros(8, np.float64)
    v = np.zeros(8, np.float64)
    x = theta.astype(np.float64)
    for step in range(1, 4):
        g = rng.standard_normal(8).astype(np.float32)
        t_g = torch.from_numpy(g).cuda()
        _abi.check(lib, lib.lsim_adam_step(t_th.data_ptr(), t_g.data_ptr(), t_sc.data_ptr(), t_lr.data_ptr(),
                                           state.data_ptr(), 0.9, 0.999, 1e-8, None))
        gn = g.astype(np.float64) * scale
        m = 0.9 * m + 0.1 * gn
        v = 0.999 * v + 0.001 * gn * gn
        mh, vh = m / (1 - 0.9 ** step), v / (1 - 0.999 ** step)
        x = (x / scale - lr * mh / (np.sqrt(vh) + 1e-8)) * scale
        np.testing.assert_allclose(t_th.cpu().numpy(), x, rtol=2e-6, atol=1e-7)
    assert state[16].item() == 3
    # a non-finite gradient skips the update
    before = t_th.clone()
    bad = torch.full((8,), float("nan"), device="cuda")
    _abi.check(lib, lib.lsim_adam_step(t_th.data_ptr(), bad.data_ptr(), t_sc.data_ptr(), t_lr.data_ptr(),
                                       state.data_ptr(), 0.9, 0.999, 1e-8, None))
    assert torch.equal(t_th, before) and state[16].item() == 3


# ---- the reference's fit step restated in float64 (fit_params.py:168-199, :833-895)

def _sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def _to_phys(scheme, k, u, o):
    if scheme == "sigmoid":
        return o["lo"] + (o["hi"] - o["lo"]) * _sigmoid(k * u)
    if scheme == "exp_log":
        return o["nom"] * np.exp(k * u)
    return u * o["norm"]


def _dphys(scheme, k, u, o):
    if scheme == "sigmoid":
        s = _sigmoid(k * u)
        return (o["hi"] - o["lo"]) * s * (1 - s) * k
    if scheme == "exp_log":
        return o["nom"] * np.exp(k * u) * k
    return o["norm"]


def _to_norm(scheme, k, v, o):
    if scheme == "sigmoid":
        eps = np.finfo(np.float32).eps
        fr = np.clip((v - o["lo"]) / (o["hi"] - o["lo"]), eps, 1 - eps)
        return np.log(fr / (1 - fr)) / k
    if scheme == "exp_log":
        return np.log(np.maximum(v, np.finfo(np.float32).tiny) / o["nom"]) / k
    return np.where(v != 0, 1.0, 0.0)


def _reference_fit(scheme, k, theta0, grads, mask, lr, o, max_norm=None, clip_range=False, b1=0.9, b2=0.999,
                   eps=1e-8):
    """Physical parameters after each step of optax.chain([clip_by_global_norm],
    adam) on the normalised parameters, as GradientDescentFitter applies it."""
    u = np.where(mask, _to_norm(scheme, k, theta0, o), 0.0)
    theta = np.where(mask, _to_phys(scheme, k, u, o), theta0)
    m = np.zeros(8)
    v = np.zeros(8)
    t = 0
    out = []
    for g_phys in grads:
        g = np.where(mask, g_phys * _dphys(scheme, k, u, o), 0.0)
        if np.isnan(g[mask]).any():
            out.append(theta.copy())
            continue
        if scheme == "divide":
            g = g * o["norm"]
        if max_norm is not None:
            gn = np.sqrt((g[mask] ** 2).sum())
            if not gn < max_norm:
                g = g / gn * max_norm
        t += 1
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        upd = -lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
        u = np.where(mask, u + upd, u)
        if scheme == "divide" and clip_range:
            u = np.where(mask, np.maximum(o["down"] / o["norm"], np.minimum(o["up"] / o["norm"], u)), u)
        theta = np.where(mask, _to_phys(scheme, k, u, o), theta0)
        out.append(theta.copy())
    return out


@pytest.mark.parametrize("scheme,k,max_norm,clip_range", [("sigmoid", 1.0, None, False), ("sigmoid", 2.5, 0.5, False),
                                                          ("exp_log", 1.0, None, False), ("exp_log", 0.7, 3.0, False),
                                                          ("divide", 1.0, None, False), ("divide", 1.0, None, True)])
def test_fit_step_matches_the_reference_chain(cuda, scheme, k, max_norm, clip_range):
    from larndsim_gb300 import _abi, fit
    from larndsim_gb300.grad import GRAD_PARAMS
    lib = _abi.load()
    rng = np.random.default_rng(3)
    names = ("Ab", "kb", "eField", "lifetime", "tran_diff", "lArDensity")
    mask = np.array([n in names for n in GRAD_PARAMS])
    r = fit.RANGES
    theta0 = np.array([r[n]["nom"] * (1 + 0.02 * rng.standard_normal()) for n in GRAD_PARAMS], np.float32)
    lr = {n: float(rng.uniform(0.005, 0.05)) for n in names}
    o = fit.fit_options(names, lr, dict(zip(GRAD_PARAMS, theta0.tolist())), scheme, k, max_norm, clip_range)
    arr = {f: np.array(list(getattr(o, f)), np.float64) for f in ("lo", "hi", "nom", "norm", "down", "up", "lr")}
    # gradients of a size that drives the divide scheme past its soft range
    scale = np.array([1.0 / max(abs(float(x)), 1e-12) for x in theta0]) * (40.0 if clip_range else 1.0)
    grads = [(rng.standard_normal(8) * scale).astype(np.float32) for _ in range(5)]
    grads.insert(3, np.full(8, np.nan, np.float32))          # a NaN gradient skips its step
    theta = torch.from_numpy(theta0.copy()).cuda()
    state = torch.zeros(_abi.FIT_STATE, dtype=torch.float32, device="cuda")
    _abi.check(lib, lib.lsim_fit_init(theta.data_ptr(), o, state.data_ptr(), None))
    ref = _reference_fit(scheme, k, theta0.astype(np.float64), [g.astype(np.float64) for g in grads], mask,
                            arr["lr"], arr, max_norm, clip_range)
    for g, want in zip(grads, ref):
        tg = torch.from_numpy(g).cuda()
        _abi.check(lib, lib.lsim_fit_step(theta.data_ptr(), tg.data_ptr(), o, state.data_ptr(), None))
        got = theta.cpu().numpy()
        np.testing.assert_allclose(got[mask], want[mask], rtol=5e-6)
        np.testing.assert_array_equal(got[~mask], theta0[~mask])     # not fitted: untouched
    assert state[3 * 8].item() == len(grads) - 1                     # the NaN step left the count as it was


def test_graph_replays_the_eager_trajectory(cuda, setup):
    from larndsim_gb300 import fit
    p, tmpl, tracks, fields, hidden, target = setup
    names = ("lifetime", "long_diff", "tran_diff")
    a = fit.DeviceFit(p, tmpl, tracks, fields, target, fit_params=names, lr=3e-3, max_steps=8)
    b = fit.DeviceFit(p, tmpl, tracks, fields, target, fit_params=names, lr=3e-3, max_steps=8)
    la, ta = a.run(6, graph=False)
    lb, tb = b.run(6, graph=True)
    np.testing.assert_array_equal(la, lb)
    np.testing.assert_array_equal(ta, tb)
    assert la[0] > 0 and not np.array_equal(ta[0], ta[-1])


@pytest.mark.parametrize("scheme,lr,steps", [("sigmoid", 1e-2, 400), ("divide", 3e-3, 300)])
def test_fit_recovers_hidden_parameters(cuda, setup, scheme, lr, steps):
    """The reference's default settings (sigmoid normalisation, no clipping,
    the learning rate of its example scripts) and the divide scheme.  The
    sigmoid map spreads each parameter over its whole hard range, so the
    same offsets are larger moves in its normalised units."""
    from larndsim_gb300 import fit
    from larndsim_gb300.grad import GRAD_PARAMS
    p, tmpl, tracks, fields, hidden, target = setup
    names = ("lifetime", "long_diff", "tran_diff")
    f = fit.DeviceFit(p, tmpl, tracks, fields, target, fit_params=names, lr=lr, normalization_scheme=scheme,
                      max_steps=steps + 8)
    loss, th = f.run(steps, graph=True)
    assert loss[-1] < 0.05 * loss[0]
    for k in names:
        i = GRAD_PARAMS.index(k)
        start = abs(float(getattr(p, k)) / float(getattr(hidden, k)) - 1)
        final = abs(th[-1, i] / float(getattr(hidden, k)) - 1)
        assert final < 0.25 * start and final < 0.01, (k, start, final)
    for k in GRAD_PARAMS:                       # parameters not fitted stay put
        if k not in names:
            assert th[-1, GRAD_PARAMS.index(k)] == np.float32(getattr(p, k))


def test_fit_with_the_default_hit_level_loss(cuda):
    """The reference fitter's default loss (mse_adc on the simulated hits,
    GenericLossStrategy): each eager step's gradient is the one
    grad.params_loss gives at the step's parameters, and a short fit of the
    electron lifetime lowers the loss and moves toward the hidden value."""
    from gpu_common import small_params
    from larndsim_gb300 import fit, grad, losses, sim, strategies, workloads
    p = small_params(n_neighbors=1)
    tmpl, p = sim.load_lut(workloads.synthetic_response(seed=0, nx=15, ny=15), p)
    tracks, fields = workloads.muon_event(seed=3, n_tracks=4)
    hidden = p.replace(lifetime=float(p.lifetime) * 0.8)
    h = strategies.LUTSimulation(tmpl).predict(hidden, tracks, fields, 0)
    ref = (losses.adc2charge(h["adcs"], p), h["pixel_x"], h["pixel_y"], h["pixel_z"], h["ticks"], h["hit_prob"],
           h["event"])
    f = fit.DeviceFit(p, tmpl, tracks, fields, fit_params=("lifetime",), lr=3e-2, loss_fn=losses.mse_adc,
                      ref_hits=ref, normalization_scheme="divide", max_steps=64)
    with pytest.raises(ValueError):
        f.capture()
    chain = grad.LUTChain(p, tmpl, tracks, fields)
    theta0 = grad.theta_of(p, device=cuda).requires_grad_(True)
    l0, _, _ = grad.params_loss(p, chain, ref, losses.mse_adc, theta=theta0)
    l0.backward()
    f.step()
    torch.cuda.synchronize()
    assert abs(float(f.out[0]) - float(l0.detach())) <= 1e-6 * abs(float(l0.detach()))
    assert torch.allclose(f.out[1:], theta0.grad.to(torch.float32), rtol=1e-5, atol=0)
    loss, th = f.run(30)
    assert loss.shape[0] == 31 and np.isfinite(loss).all()
    assert loss.min() < 0.25 * loss[0] and loss[-1] < loss[0]
    k = grad.GRAD_PARAMS.index("lifetime")
    assert abs(th[-1, k] - float(hidden.lifetime)) < abs(th[0, k] - float(hidden.lifetime))
