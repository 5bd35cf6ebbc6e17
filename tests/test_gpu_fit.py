"""Device-resident fit loop (optimize/fit_params.py:704-731, :872-895):
the segment stage with device-side parameters, the gradient and an Adam
update, captured in one CUDA graph.  The graph replays the eager
trajectory exactly, the Adam kernel follows optax.adam in the "divide"
normalisation, and a fit recovers hidden parameters."""

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


def test_fit_recovers_hidden_parameters(cuda, setup):
    from larndsim_gb300 import fit
    from larndsim_gb300.grad import GRAD_PARAMS
    p, tmpl, tracks, fields, hidden, target = setup
    names = ("lifetime", "long_diff", "tran_diff")
    f = fit.DeviceFit(p, tmpl, tracks, fields, target, fit_params=names, lr=3e-3, max_steps=400)
    loss, th = f.run(300, graph=True)
    assert loss[-1] < 0.05 * loss[0]
    for k in names:
        i = GRAD_PARAMS.index(k)
        start = abs(float(getattr(p, k)) / float(getattr(hidden, k)) - 1)
        final = abs(th[-1, i] / float(getattr(hidden, k)) - 1)
        assert final < 0.25 * start and final < 0.01, (k, start, final)
    for k in GRAD_PARAMS:                       # parameters not fitted stay put
        if k not in names:
            assert th[-1, GRAD_PARAMS.index(k)] == np.float32(getattr(p, k))
