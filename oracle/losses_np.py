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


def stacked_1e9(x, y, z, event, extra=None):
    """(x + event * 1e9, y, z[, extra]) in float32, as chamfer_3d and
    nll_loss stack them (losses_jax.py:221-222, :337-338)."""
    sx = (np.asarray(x, F32) + (np.asarray(event).astype(F32) * F32(1e9)).astype(F32)).astype(F32)
    cols = [sx, np.asarray(y, F32), np.asarray(z, F32)]
    if extra is not None:
        cols.append(np.asarray(extra, F32))
    return np.stack(cols, axis=-1)


def chamfer_distance_3d_og(a, b, wa, wb):
    """losses_jax.py:181-211: nearest neighbours both ways (first index on
    ties), sum of min distance x own weight x neighbour weight over pairs
    closer than 1e4.  a, b are float32 stacked coordinates; the squared
    distances are float32 as the reference computes them; returns
    (loss, argmin a->b, argmin b->a, min distances a->b, b->a)."""
    diff = (a[:, None, :] - b[None, :, :]).astype(F32)
    sq = (diff * diff).astype(F32)
    d = ((sq[..., 0] + sq[..., 1]).astype(F32) + sq[..., 2]).astype(F32).astype(np.float64)
    ia = np.argmin(d, axis=1)
    ib = np.argmin(d, axis=0)
    ma = d[np.arange(len(a)), ia]
    mb = d[ib, np.arange(len(b))]
    wa = np.asarray(wa, np.float64)
    wb = np.asarray(wb, np.float64)
    loss = (ma * wa * wb[ia])[ma < 1e4].sum() + (mb * wb * wa[ib])[mb < 1e4].sum()
    return loss, ia, ib, ma, mb


def chamfer_3d(Q, x, y, z, event, ref_Q, ref_x, ref_y, ref_z, ref_event, adc_norm=10.0, pad_to=None):
    """losses_jax.py:213-229 with the padded sizes given: (loss, grad_Q,
    grad_z) of the predicted hits (the argmins carry no gradient)."""
    n, m = len(Q), len(ref_Q)
    nc, nr = (n, m) if pad_to is None else pad_to
    a = np.zeros((nc, 3), F32)
    b = np.zeros((nr, 3), F32)
    a[:n] = stacked_1e9(x, y, z, event)
    b[:m] = stacked_1e9(ref_x, ref_y, ref_z, ref_event)
    wa = np.zeros(nc)
    wb = np.zeros(nr)
    wa[:n] = np.asarray(Q, np.float64) / adc_norm
    wb[:m] = np.asarray(ref_Q, np.float64) / adc_norm
    loss, ia, ib, ma, mb = chamfer_distance_3d_og(a, b, wa, wb)
    ka, kb = ma < 1e4, mb < 1e4
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    gwa = np.where(ka, ma * wb[ia], 0.0)
    np.add.at(gwa, ib, np.where(kb, mb * wb, 0.0))
    gz = np.where(ka, wa * wb[ia] * 2 * (a64[:, 2] - b64[ia, 2]), 0.0)
    np.add.at(gz, ib, np.where(kb, wb * wa[ib] * 2 * (a64[ib, 2] - b64[:, 2]), 0.0))
    return loss, gwa[:n] / adc_norm, gz[:n]


def nll_loss(Q, x, y, z, hit_prob, event, ref_Q, ref_x, ref_y, ref_z, ref_hit_prob, ref_event, adc_norm=10.0,
             sigma=1.0):
    """losses_jax.py:329-359 (padding rows sit at -1e9 with zero
    probabilities and add nothing): (loss, grad_Q, grad_z, grad_hit_prob)."""
    a = stacked_1e9(x, y, z, event, np.asarray(Q, F32) / F32(adc_norm)).astype(np.float64)
    b = stacked_1e9(ref_x, ref_y, ref_z, ref_event, np.asarray(ref_Q, F32) / F32(adc_norm)).astype(np.float64)
    hp = np.asarray(hit_prob, np.float64)
    mref = (np.asarray(ref_hit_prob) > 0.5).astype(np.float64)
    d = ((a[:, None, :] - b[None, :, :]) ** 2).sum(-1)
    K = np.exp(-d / (2 * sigma ** 2))
    lam = hp @ K
    loss = hp.sum() - (np.log(lam + 1e-10) * mref).sum()
    c = mref / (lam + 1e-10)
    g_hp = 1 - K @ c
    g_q = hp / sigma ** 2 * ((K * (a[:, 3][:, None] - b[None, :, 3])) @ c)
    g_z = hp / sigma ** 2 * ((K * (a[:, 2][:, None] - b[None, :, 2])) @ c)
    return loss, g_q / adc_norm, g_z, g_hp
