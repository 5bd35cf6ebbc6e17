"""Restatement of larnd-sim-jax's likelihood losses on the probabilistic
front end's distributions.  TEST INFRASTRUCTURE ONLY (see
``oracle/__init__.py``).

- ``compute_occurrence_indices``: optimize/strategies.py:14-40.
- ``prob_llhd``: ProbabilisticLossStrategy.compute, optimize/strategies.py:
  338-567 (target hits matched to the simulated pixels by searchsorted, the
  hit's occurrence index within its run of equal pixel ids picks the
  distribution row, the tick's log-probability clamped at log(eps), a
  Gaussian charge term, loss = sqrt(T * C) of the two log-likelihood sums).
- ``llhd_loss``: src/larndsim/losses_jax.py:414-441.

The per-hit terms are evaluated in float32 in the reference's operation
order (the clamp and the tick cut are decisions); the sums are taken in
float64.  Gathers follow jax.numpy indexing: a negative index counts from
the end, an out-of-range index is clamped to the array.  ``*_grad``
functions give the float64 derivatives of the loss with respect to the
dense inputs, the cotangents jax.grad pushes into the distributions (ties
of the clamp split 1/2 each, as jax.lax.max's derivative does).
"""

from __future__ import annotations

import numpy as np

F32 = np.float32


def compute_occurrence_indices(ids):
    """strategies.py:14-40: index of each element within its run of equal
    consecutive ids ([100, 100, 100, 200, 200, 300] -> [0, 1, 2, 0, 1, 0])."""
    ids = np.asarray(ids)
    n = ids.shape[0]
    if n == 0:
        return np.zeros(0, np.int32)
    change = np.concatenate([[True], ids[1:] != ids[:-1]])
    pos = np.arange(1, n + 1, dtype=np.int64)
    start = np.maximum.accumulate(np.where(change, pos, 0))
    return (pos - start).astype(np.int32)


def jax_index(idx, size):
    """The position jax.numpy indexing reads for integer index ``idx`` on an
    axis of ``size``: negatives count from the end, then clamp."""
    idx = np.asarray(idx, np.int64)
    return np.clip(np.where(idx < 0, idx + size, idx), 0, size - 1)


def adc_charge_consts(params):
    """float32 constants of adc2charge (losses_jax.py:380-383)."""
    return (F32(params.ADC_COUNTS), F32(params.V_REF - params.V_CM), F32(params.V_CM), F32(params.V_PEDESTAL),
            F32(params.GAIN))


def adc2charge32(dw, consts):
    a, r, cm, ped, g = consts
    return (((((np.asarray(dw, F32) / a) * r) + cm) - ped) / g * F32(1e-3)).astype(F32)


def adc2charge_slope(consts):
    """d adc2charge / d dw in the order reverse mode forms it."""
    a, r, cm, ped, g = consts
    return float(F32(F32(F32(F32(1e-3) / g) * r) / a))


def _prob_terms(sim_pixels, log_prob, adcs, tgt_pixels, tgt_ticks, tgt_adcs, consts, sigma_charge, eps):
    sim = np.asarray(sim_pixels, np.int64)
    lp = np.asarray(log_prob, F32)
    ad = np.asarray(adcs, F32)
    P, H, T = lp.shape
    tp = np.asarray(tgt_pixels, np.int64)
    tt = np.asarray(tgt_ticks).astype(np.int64)
    idx = np.searchsorted(sim, tp, side="left")
    safe = np.clip(idx, 0, P - 1)
    valid = (sim[safe] == tp) & (tp >= 0)
    nb = jax_index(compute_occurrence_indices(tp), H)
    tk = jax_index(tt, T)
    p = lp[safe, nb, tk]
    log_eps = F32(np.log(F32(eps)))
    llt = np.where(valid, np.maximum(p, log_eps), F32(0)).astype(F32)
    tq = adc2charge32(tgt_adcs, consts)
    hq = np.where(valid, adc2charge32(ad[safe, nb, tk], consts), F32(0)).astype(F32)
    s = F32(sigma_charge / 1000)
    hl = F32(F32(0.5) * F32(np.log(F32(2 * np.pi * (sigma_charge / 1000) ** 2))))
    r = ((tq - hq) / s).astype(F32)
    llc = (F32(-0.5) * (r * r) - hl).astype(F32)
    n_miss = int((sim[safe] != tp).sum())
    penalty = float(F32(log_eps * F32(n_miss)))
    return dict(safe=safe, nb=nb, tk=tk, p=p, valid=valid, llt=llt, llc=llc, r=r, s=s, log_eps=log_eps,
                penalty=penalty, shape=(P, H, T))


def prob_llhd(sim_pixels, log_prob, adcs, tgt_pixels, tgt_ticks, tgt_adcs, consts, sigma_charge=500.0, eps=1e-10):
    """ProbabilisticLossStrategy.compute (strategies.py:365-567) on the
    prediction's sorted ``unique_pixels`` [P], ``hit_prob`` (log-
    probabilities) and ``adcs_distrib`` [P, H, T] and the target's hit
    pixel ids, ticks and ADC counts.  Returns (loss, aux) with the
    reference's aux keys."""
    t = _prob_terms(sim_pixels, log_prob, adcs, tgt_pixels, tgt_ticks, tgt_adcs, consts, sigma_charge, eps)
    T = float(t["llt"].astype(np.float64).sum()) + t["penalty"]
    C = float(t["llc"].astype(np.float64).sum())
    loss = float(np.sqrt(T * C))
    return loss, {"log_likelihood_charge": -C, "log_likelihood_tick": -T, "no_match_penalty": -t["penalty"]}


def prob_llhd_grad(sim_pixels, log_prob, adcs, tgt_pixels, tgt_ticks, tgt_adcs, consts, sigma_charge=500.0,
                   eps=1e-10):
    """(d loss / d log_prob, d loss / d adcs), float64 arrays of the inputs'
    shape."""
    t = _prob_terms(sim_pixels, log_prob, adcs, tgt_pixels, tgt_ticks, tgt_adcs, consts, sigma_charge, eps)
    T = float(t["llt"].astype(np.float64).sum()) + t["penalty"]
    C = float(t["llc"].astype(np.float64).sum())
    half = 0.5 / np.sqrt(T * C)
    dT, dC = half * C, half * T
    p = t["p"].astype(np.float64)
    le = float(t["log_eps"])
    tie = np.where(p > le, 1.0, np.where(p == le, 0.5, 0.0))
    g_lp = np.zeros(t["shape"])
    g_ad = np.zeros(t["shape"])
    v = t["valid"]
    np.add.at(g_lp, (t["safe"][v], t["nb"][v], t["tk"][v]), dT * tie[v])
    slope = adc2charge_slope(consts)
    dhq = t["r"].astype(np.float64) / float(t["s"])
    np.add.at(g_ad, (t["safe"][v], t["nb"][v], t["tk"][v]), dC * dhq[v] * slope)
    return g_lp, g_ad


def llhd_loss(ticks_prob_distrib, ticks_mc, no_hit_prob, charge_distrib, charge_mc, sigma=500):
    """losses_jax.py:414-441: -sum over rows of log(p[tick] + eps), or
    log(no_hit_prob + eps) where tick >= T - 3, plus a Gaussian charge term
    of width sigma at the distribution's charge (0 where tick >= T - 3)."""
    tpd = np.asarray(ticks_prob_distrib, F32)
    cd = np.asarray(charge_distrib, F32)
    N, T = tpd.shape
    tm = np.asarray(ticks_mc).astype(np.int64)
    k = jax_index(tm, T)
    rows = np.arange(N)
    p, q = tpd[rows, k], cd[rows, k]
    eps = F32(1e-10)
    on = tm < T - 3
    llt = np.where(on, np.log(p + eps), np.log(np.asarray(no_hit_prob, F32) + eps)).astype(F32)
    s = F32(sigma)
    r = ((np.asarray(charge_mc, F32) - q) / s).astype(F32)
    hl = F32(F32(0.5) * F32(np.log(F32(2 * np.pi * sigma ** 2))))
    llc = np.where(on, F32(-0.5) * (r * r) - hl, F32(0)).astype(F32)
    return -float((llt + llc).astype(np.float64).sum()), {}


def llhd_loss_grad(ticks_prob_distrib, ticks_mc, no_hit_prob, charge_distrib, charge_mc, sigma=500):
    """float64 derivatives of llhd_loss: (d/d ticks_prob_distrib [N, T],
    d/d no_hit_prob [N], d/d charge_distrib [N, T], d/d charge_mc [N])."""
    tpd = np.asarray(ticks_prob_distrib, F32)
    cd = np.asarray(charge_distrib, F32)
    N, T = tpd.shape
    tm = np.asarray(ticks_mc).astype(np.int64)
    k = jax_index(tm, T)
    rows = np.arange(N)
    on = tm < T - 3
    eps = 1e-10
    g_t = np.zeros((N, T))
    g_c = np.zeros((N, T))
    p = tpd[rows, k].astype(np.float64)
    np.add.at(g_t, (rows[on], k[on]), -1.0 / (p[on] + eps))
    g_nh = np.where(on, 0.0, -1.0 / (np.asarray(no_hit_prob, np.float64) + eps))
    r = (np.asarray(charge_mc, np.float64) - cd[rows, k].astype(np.float64)) / sigma
    np.add.at(g_c, (rows[on], k[on]), -(r[on] / sigma))
    g_cm = np.where(on, r / sigma, 0.0)
    return g_t, g_nh, g_c, g_cm
