"""Adjoint of the probabilistic front end (lsim_fee_prob_vjp) against
float64 central differences of the beam search with the GPU's own top-K
choices and executed steps held (oracle/reference_np.py beam_search64):
directional derivatives along random waveform perturbations.

The waveforms get a small positive pedestal so the cumulative charge rises
strictly and the running maximum has no ties (the reference splits the
cotangent of tied maxima, this library gives it to the first tick).
Tolerance: 5e-3 relative on each directional derivative (observed up to
1.2e-3: float32 log-probabilities cancel in log(Phi(a) - Phi(b)))."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_common import small_params

pytestmark = pytest.mark.gpu
RTOL = 5e-3


@pytest.fixture(scope="module")
def case():
    from larndsim_gb300 import workloads
    from oracle import reference_np as R
    p = small_params(n_neighbors=1, RESET_NOISE_CHARGE=900)
    tmpl = R.load_lut_templates(workloads.synthetic_response(seed=0, nx=25, ny=25), p)
    tracks, fields = workloads.muon_event(seed=7, n_tracks=3)
    w, u = R.simulate_wfs(p, tmpl, tracks, fields, history={})
    w = w[u >= 0][:12].astype(np.float64) + 2.0
    return p, w.astype(np.float32)


def _run(p, w, gl=None, gq=None, red=None):
    from larndsim_gb300 import _abi, sim
    lib = _abi.load()
    lp = _abi.make_params(p)
    P, T = w.shape
    K = int(p.fee_paths_scaling)
    H = int(p.MAX_ADC_VALUES)
    ws = torch.zeros(lib.lsim_fee_prob_vjp_workspace_bytes(lp, P, K), dtype=torch.uint8, device="cuda")
    wt = torch.from_numpy(w).cuda()
    g = torch.empty_like(wt)
    dev = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()  # noqa: E731
    gr = [None, None, None] if red is None else [dev(r) for r in red]
    gl_t, gq_t = dev(gl), dev(gq)
    _abi.check(lib, lib.lsim_fee_prob_vjp(lp, wt.data_ptr(), P, T, K, 1e-9, sim._ptr(gl_t), sim._ptr(gq_t),
                                          sim._ptr(gr[0]), sim._ptr(gr[1]), sim._ptr(gr[2]), g.data_ptr(),
                                          ws.data_ptr(), ws.numel(), sim._stream()))
    torch.cuda.synchronize()
    raw = ws.cpu().numpy()
    flags_bytes = (H * 4 + 255) & ~255
    states = P * H * K
    off = flags_bytes + ((8 * states + 255) & ~255)
    top = raw[off:off + 4 * states].view(np.int32).reshape(P, H, K)
    flags = raw[:4 * H].view(np.int32)
    n_exec = H
    for h in range(1, H):
        if not flags[h - 1]:
            n_exec = h
            break
    return g.cpu().numpy().astype(np.float64), top, n_exec


def _functional(p, w, top, n_exec, gl, gq, red):
    from oracle import reference_np as R
    lp, ch = R.beam_search64(p, w, top, n_exec)
    val = 0.0
    if gl is not None:
        val += float((gl * lp).sum())
    if gq is not None:
        val += float((gq * ch).sum())
    if red is not None:
        pr = np.exp(lp)
        lam = pr.sum(axis=2)
        den = np.maximum(lam, 1e-10)
        T1 = lp.shape[2]
        et = (np.arange(T1)[None, None, :] * pr).sum(axis=2) / den
        adc = R.digitize(p, ch.astype(np.float32)).astype(np.float64)
        # digitize is linear inside its clamps: differentiate it in float64 too
        pre = (ch * p.GAIN + p.V_PEDESTAL) - p.V_CM
        adc = np.where((pre > 0) & (adc < p.ADC_COUNTS), pre * p.ADC_COUNTS / (p.V_REF - p.V_CM), adc)
        ea = (adc * pr).sum(axis=2) / den
        val += float((red[0] * et).sum() + (red[1] * ea).sum() + (red[2] * lam).sum())
    return val


@pytest.fixture(scope="module")
def case_flat():
    """Rows as simulated, with their flat stretches (no charge arriving):
    long runs of ticks with identical inputs, which the adjoint evaluates
    once per run."""
    from larndsim_gb300 import workloads
    from oracle import reference_np as R
    p = small_params(n_neighbors=1, RESET_NOISE_CHARGE=900)
    tmpl = R.load_lut_templates(workloads.synthetic_response(seed=0, nx=25, ny=25), p)
    tracks, fields = workloads.muon_event(seed=8, n_tracks=3)
    w, u = R.simulate_wfs(p, tmpl, tracks, fields, history={})
    w = w[u >= 0][:12]
    assert (w == 0).mean() > 0.5
    return p, w.astype(np.float32)


@pytest.mark.parametrize("kind", ["reductions", "distributions", "reductions-flat", "distributions-flat"])
def test_fee_prob_vjp_matches_frozen_fd(cuda, case, case_flat, kind):
    """On flat rows the perturbations leave the flat stretches flat (zero
    where the row is zero), so tied running maxima stay tied and the
    direction does not depend on how their cotangent is shared."""
    flat = kind.endswith("-flat")
    kind = kind.replace("-flat", "")
    p, w = case_flat if flat else case
    rng = np.random.default_rng((11 if kind == "reductions" else 12) + (100 if flat else 0))
    P, T = w.shape
    H = int(p.MAX_ADC_VALUES)
    gl = gq = red = None
    if kind == "reductions":
        red = [rng.standard_normal((P, H)) * 1e-2, rng.standard_normal((P, H)), rng.standard_normal((P, H))]
    else:
        from oracle import reference_np as R
        lp0, _ = R.get_adc_values_average_noise(p, w)
        gl = rng.standard_normal((P, H, T - 1)) * (lp0 > -30)     # likely ticks only
        gq = rng.standard_normal((P, H, T - 1)) * 1e-4
    g, top, n_exec = _run(p, w, gl, gq, red)
    assert n_exec >= 2 and np.all(np.isfinite(g))
    w64 = w.astype(np.float64)
    for d in range(3):
        delta = rng.standard_normal(w.shape) * (w != 0 if flat else 1.0)
        eps = 1e-2
        fp = _functional(p, w64 + eps * delta, top, n_exec, gl, gq, red)
        fm = _functional(p, w64 - eps * delta, top, n_exec, gl, gq, red)
        fd = (fp - fm) / (2 * eps)
        an = float((g * delta).sum())
        assert abs(an - fd) <= RTOL * abs(fd) + 1e-9, (d, an, fd)


def test_probabilistic_chain_gradient(cuda):
    """wfs_fn -> average_hit_values -> a collapsed-hit loss (the
    CollapsedProbabilisticLossStrategy path of optimize/strategies.py):
    torch autograd reaches the physics parameters through lsim_fee_prob_vjp
    and lsim_lut_wfs_vjp; the eField and lifetime gradients are finite and
    non-zero."""
    from larndsim_gb300 import grad, sim, workloads
    p = small_params(n_neighbors=1, RESET_NOISE_CHARGE=900)
    tmpl, p = sim.load_lut(workloads.synthetic_response(seed=0, nx=15, ny=15), p)
    tracks, fields = workloads.muon_event(seed=3, n_tracks=2)
    chain = grad.LUTChain(p, tmpl, tracks, fields)
    with torch.no_grad():
        w0, u0 = grad.wfs_fn(grad.theta_of(p), chain, p)
        t0, a0, l0 = sim.average_hit_values(p, w0[u0 >= 0])
    pp = p.replace(lifetime=2000.0, eField=0.51)
    theta = grad.theta_of(pp).requires_grad_(True)
    wfs, unique = grad.wfs_fn(theta, chain, pp)
    v = wfs[unique >= 0]
    et, ea, lam = sim.average_hit_values(pp, v)
    loss = ((ea - a0) ** 2 * l0).sum() + 1e-4 * ((et - t0) ** 2 * l0).sum() + ((lam - l0) ** 2).sum()
    loss.backward()
    g = theta.grad.cpu().numpy()
    assert np.all(np.isfinite(g))
    assert g[grad.GRAD_PARAMS.index("eField")] != 0.0 and g[grad.GRAD_PARAMS.index("lifetime")] != 0.0
