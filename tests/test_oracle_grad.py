"""The FP64 gradient oracle agrees with itself three ways: reverse-mode
adjoint, complex-step derivative and central finite differences of the
frozen-decision loss; and vdrift's gradient is identically zero, as in the
reference (params.vdrift is never read)."""

import numpy as np
import pytest

from larndsim_gb300 import consts, workloads
from oracle import grad64 as G
from oracle import reference_np as R


@pytest.fixture(scope="module")
def frozen():
    p = consts.Params(number_pix_neighbors=1, RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0,
                      long_diff_template=consts.jax_linspace_f32(0.001, 10, 10))
    resp = workloads.synthetic_response(seed=0, nx=15, ny=15)
    tmpl = R.load_lut_templates(resp, p)
    tracks, fields = workloads.muon_event(seed=3, n_tracks=3)
    w, u = R.simulate_wfs(p, tmpl, tracks, fields, history={})
    out = R.simulate_stochastic(p, w, u)
    v = u >= 0
    pp = p.replace(Ab=0.83, kb=0.05, eField=0.52, lifetime=2000.0, long_diff=5e-6, tran_diff=9e-6, lArDensity=1.39)
    return G.Frozen(pp, tmpl, tracks, fields, u[v], out["grid_adcs"][v]), G.theta_dict(pp)


def test_adjoint_equals_complex_step(frozen):
    fr, th = frozen
    adj, cs = G.adjoint64(fr, th), G.complex_step_gradient(fr, th)
    for k in G.GRAD_PARAMS:
        assert abs(adj[k] - cs[k]) <= 1e-9 * abs(cs[k]) + 1e-12, k
    assert adj["vdrift"] == 0.0


def test_complex_step_equals_central_differences(frozen):
    fr, th = frozen
    cs, fd = G.complex_step_gradient(fr, th), G.fd_gradient(fr, th, 1e-6)
    for k in G.GRAD_PARAMS:
        assert abs(cs[k] - fd[k]) <= 1e-5 * abs(cs[k]) + 1e-9, k


def test_vjp_is_linear_in_the_cotangent(frozen):
    fr, th = frozen
    rng = np.random.default_rng(0)
    g1 = rng.standard_normal((int(fr.valid.sum()), 10))
    g2 = rng.standard_normal(g1.shape)
    a = G.adjoint64(fr, th, g1)
    b = G.adjoint64(fr, th, g2)
    c = G.adjoint64(fr, th, 2 * g1 - g2)
    for k in G.GRAD_PARAMS:
        assert abs(c[k] - (2 * a[k] - b[k])) <= 1e-9 * (abs(a[k]) + abs(b[k])) + 1e-12
