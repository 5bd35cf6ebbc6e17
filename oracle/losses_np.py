"""float64 restatement of larnd-sim-jax's hit-level fit loss mse_adc.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

src/larndsim/losses_jax.py:13-19 (rbf_kernel), :21-39 (mmd), :60-79
(mse_adc).  The stacked coordinates x + event * 1e5 are formed in float32
as the reference forms them (that rounding decides which hits are close);
everything after is evaluated in float64.  ``mse_adc_grad`` gives the
derivatives of the loss with respect to the predicted weights
w = Q * hit_prob and the predicted z, the quantities through which
jax.value_and_grad reaches the physics parameters.
"""

from __future__ import annotations

import numpy as np

F32 = np.float32


def stacked(x, y, z, event):
    sx = (np.asarray(x, F32) + (np.asarray(event).astype(F32) * F32(1e5)).astype(F32)).astype(F32)
    return np.stack([sx, np.asarray(y, F32), np.asarray(z, F32)], axis=-1).astype(np.float64)


def rbf_kernel(a, b, sigma):
    """losses_jax.py:13-19: exp(-|a_i - b_j|^2 / (2 sigma^2))."""
    d = ((a[:, None, :] - b[None, :, :]) ** 2).sum(-1)
    return np.exp(-d / (2 * sigma ** 2))


def mmd(a, b, pa, pb, sigma):
    """losses_jax.py:21-39: weighted MMD^2 between point sets a and b."""
    kxx = (rbf_kernel(a, a, sigma) * pa[:, None] * pa[None, :]).sum()
    kyy = (rbf_kernel(b, b, sigma) * pb[:, None] * pb[None, :]).sum()
    kxy = (rbf_kernel(a, b, sigma) * pa[:, None] * pb[None, :]).sum()
    sa, sb = pa.sum(), pb.sum()
    return kxx / sa ** 2 + kyy / sb ** 2 - 2 * kxy / (sa * sb)


def mse_adc(Q, x, y, z, hit_prob, event, ref_Q, ref_x, ref_y, ref_z, ref_hit_prob, ref_event, sigma=1.0,
            lambda_Q=1.0):
    """losses_jax.py:60-79: (loss, mmd term, charge term)."""
    w = np.asarray(Q, np.float64) * np.asarray(hit_prob, np.float64)
    v = np.asarray(ref_Q, np.float64) * np.asarray(ref_hit_prob, np.float64)
    a, b = stacked(x, y, z, event), stacked(ref_x, ref_y, ref_z, ref_event)
    m = mmd(a, b, w, v, sigma)
    charge = ((w.sum() - v.sum()) / (v.sum() + 1e-6)) ** 2
    return m + lambda_Q * charge, m, charge


def mse_adc_grad(w, x, y, z, event, v, ref_x, ref_y, ref_z, ref_event, sigma=1.0, lambda_Q=1.0):
    """dL/dw and dL/dz of the predicted hits (analytic)."""
    w = np.asarray(w, np.float64)
    v = np.asarray(v, np.float64)
    a, b = stacked(x, y, z, event), stacked(ref_x, ref_y, ref_z, ref_event)
    kxx, kxy, kyy = rbf_kernel(a, a, sigma), rbf_kernel(a, b, sigma), rbf_kernel(b, b, sigma)
    sw, sv = w.sum(), v.sum()
    A, B = w @ kxx @ w, w @ kxy @ v
    ai, bi = kxx @ w, kxy @ v
    gw = 2 * ai / sw ** 2 - 2 * A / sw ** 3 - 2 * bi / (sw * sv) + 2 * B / (sw ** 2 * sv)
    gw += lambda_Q * 2 * (sw - sv) / (sv + 1e-6) ** 2
    za, zb = a[:, 2], b[:, 2]
    az = (kxx * (za[:, None] - za[None, :])) @ w
    bz = (kxy * (za[:, None] - zb[None, :])) @ v
    gz = -2 * w / sigma ** 2 * (az / sw ** 2 - bz / (sw * sv))
    return gw, gz
