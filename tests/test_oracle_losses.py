"""The mse_adc oracle (losses_jax.py:13-79) against its definition: the
analytic weight and z gradients match float64 central differences, and
hits of different events do not interact."""

import numpy as np

from oracle import losses_np as L


def _hits(rng, n, n_events=3):
    ev = np.sort(rng.integers(0, n_events, n)).astype(np.int32)
    return (rng.uniform(-30, 30, n).astype(np.float32), rng.uniform(-60, 60, n).astype(np.float32),
            rng.uniform(-30, 30, n).astype(np.float32), ev)


def test_mse_adc_gradients_match_central_differences():
    rng = np.random.default_rng(0)
    x, y, z, ev = _hits(rng, 40)
    # put the hits close together so that the kernel terms matter
    x, y, z = (x * 0.05).astype(np.float32), (y * 0.05).astype(np.float32), (z * 0.05).astype(np.float32)
    rx, ry, rz = (x + 0.3).astype(np.float32), (y - 0.2).astype(np.float32), (z + 0.1).astype(np.float32)
    w = rng.uniform(1, 5, 40)
    v = rng.uniform(1, 5, 40)
    gw, gz = L.mse_adc_grad(w, x, y, z, ev, v, rx, ry, rz, ev, sigma=1.0, lambda_Q=0.7)

    def loss(ww, zz):
        return L.mse_adc(ww, x, y, zz, np.ones_like(ww), ev, v, rx, ry, rz, np.ones_like(v), ev, 1.0, 0.7)[0]

    for i in (0, 7, 23):
        h = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        assert abs((loss(wp, z) - loss(wm, z)) / (2 * h) - gw[i]) <= 1e-6 * max(1.0, abs(gw[i]))
    # z enters through float32 stacking; perturb in float64 by evaluating the
    # kernel directly on a float64 copy
    a = L.stacked(x, y, z, ev)
    b = L.stacked(rx, ry, rz, ev)

    def loss_z(zz):
        aa = a.copy()
        aa[:, 2] = zz
        m = L.mmd(aa, b, w, v, 1.0)
        return m

    for i in (3, 11):
        h = 1e-6
        zp, zm = a[:, 2].copy(), a[:, 2].copy()
        zp[i] += h
        zm[i] -= h
        assert abs((loss_z(zp) - loss_z(zm)) / (2 * h) - gz[i]) <= 1e-5 * max(1e-3, abs(gz[i]))


def test_events_do_not_interact():
    rng = np.random.default_rng(1)
    x, y, z, _ = _hits(rng, 30)
    ev0 = np.zeros(30, np.int32)
    ev1 = np.ones(30, np.int32)
    a0 = L.stacked(x, y, z, ev0)
    a1 = L.stacked(x, y, z, ev1)
    assert np.all(L.rbf_kernel(a0, a1, 1.0) == 0.0)
