"""FP64 pathwise-gradient oracle for the LUT-mode ADC loss.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

``jax.value_and_grad`` of the reference (optimize/fit_params.py:704, :731)
differentiates simulate_wfs + simulate_stochastic with every integer or
comparison-derived quantity held fixed: sub-pixel bins, the cathode tick
``floor(t0/ts)`` (sim_jax.py:158), the template index (sim_jax.py:163), the
pixel renumbering, the FEE crossing index, integration and reset indices,
the accept/reject decision and the ``where(C < 0, 0, C)`` reset masks
(fee_jax.py:197-265), and the clamp branches of digitize (fee_jax.py:68).
``Frozen`` records those decisions from a float32 oracle forward pass;
``loss64`` re-evaluates the loss in float64 with them fixed, so its central
finite differences are the pathwise gradient, free of the jumps a full
re-simulation shows when an index flips.

Parameters: Ab, kb, eField, lifetime, vdrift, long_diff, tran_diff,
lArDensity (Birks, Box and ellipsoid Box recombination; the Box models'
max(0, f) branch is frozen too).  ``vdrift`` does not enter (the reference
never reads params.vdrift), so its derivative is 0.  ``param_waveforms64``
does the same for the parametrised mode's waveforms (sim_jax.py:122-139,
:289-335).
"""

from __future__ import annotations

import numpy as np
from scipy import special

from . import reference_np as R

GRAD_PARAMS = ("Ab", "kb", "eField", "lifetime", "vdrift", "long_diff", "tran_diff", "lArDensity")


def vdrift64(params, eField):
    a0, a1, a2, a3, a4, a5 = params.ELECTRON_MOBILITY_PARAMS
    e = eField
    num = a0 + a1 * e + a2 * e ** 1.5 + a3 * e ** 2.5
    den = 1 + (a1 / a0) * e + a4 * e ** 2 + a5 * e ** 3
    return num / den * (params.temperature / 89) ** -1.5 / 1000 * e


class Frozen:
    """Discrete decisions of one float32 forward pass plus the inputs."""

    def __init__(self, params, templates, tracks, fields, target_pids, target_adc):
        self.mode = int(getattr(params.recombination_mode, "value", params.recombination_mode))
        self.params = params
        self.T = np.asarray(templates, np.float32)   # widened to float64 per slice
        self.fields = tuple(fields)
        d = R.simulate_drift_new(params, tracks, fields)
        t = d["tracks"]
        self.d = d
        sh = R.shift_tracks(params, tracks, fields)
        self.z = sh[:, fields.index("z")].astype(np.float64)
        self.dE = sh[:, fields.index("dE")].astype(np.float64)
        self.dEdx = sh[:, fields.index("dEdx")].astype(np.float64)
        # ellipsoid Box model: the angle factor beta / sqrt(sin^2 + cos^2 / R^2)
        # (no parameter dependence); Box models: the max(0, f) branch taken
        zs, ze = sh[:, fields.index("z_start")], sh[:, fields.index("z_end")]
        cosphi = (np.abs(ze - zs) / (sh[:, fields.index("dx")] + np.float32(1e-10))).astype(np.float64)
        self.b_phi = params.beta / np.sqrt((1 - cosphi ** 2) + cosphi ** 2 / params.R_param ** 2)
        q32 = R.quench(params, sh, fields)[:, fields.index("n_electrons")]
        self.recomb_on = q32 > 0
        mask, plane = R.tpc_membership(params, sh[:, fields.index("x")], sh[:, fields.index("y")], sh[:, fields.index("z")])
        self.mask = mask.astype(np.float64)
        self.plane = plane
        b = np.asarray(params.tpc_borders, np.float32)
        self.z_anode = b[plane, 2, 0].astype(np.float64)
        self.z_cathode = b[plane, 2, 1].astype(np.float64)
        nb = params.nb_sampling_bins_per_pixel
        width = params.pixel_pitch / nb
        self.x0 = R.remainder_f32(sh[:, fields.index("x")] - b[plane, 0, 0], width).astype(np.float64)
        self.y0 = R.remainder_f32(sh[:, fields.index("y")] - b[plane, 1, 0], width).astype(np.float64)
        self.edges = R.jax_linspace_f32(-2 * width, 3 * width, 6).astype(np.float64)
        # frozen time / template decisions (float32 forward)
        ts = np.float32(params.t_sampling)
        Nt = self.T.shape[-1]
        ft = (d["t0"] / ts).astype(np.float32)
        self.cath = np.clip(np.floor(ft).astype(np.int64), 0, Nt - 1)
        tmpl = np.asarray(params.long_diff_template, np.float32)
        self.tidx = np.clip(np.searchsorted(tmpl, d["ld"], side="left"), 1, len(tmpl) - 2)
        self.tmpl = tmpl.astype(np.float64)
        # pixel rows and the f32 forward
        self.unique = R.unique_pixel_rows(d["main_pixels"], history={})
        wfs32 = R.simulate_signals(params, self.unique, d, np.asarray(templates, np.float32))[:, 1:]
        self.valid = self.unique >= 0
        self._fee_decisions(wfs32)
        # target aligned on the valid rows; target pixels absent here add a constant
        H = int(params.MAX_ADC_VALUES)
        adc0 = float(R.digitize(params, np.float32(0)))
        tp = np.asarray(target_pids)
        ta = np.asarray(target_adc, np.float64)
        vp = self.unique[self.valid]
        pos = np.searchsorted(tp, vp)
        ok = (pos < len(tp)) & (tp[np.minimum(pos, len(tp) - 1)] == vp)
        self.tgt = np.full((vp.shape[0], H), adc0)
        self.tgt[ok] = ta[pos[ok]]
        missing = ~np.isin(tp, vp) & (tp >= 0)
        self.const = float(((adc0 - ta[missing]) ** 2).sum())

    def _fee_decisions(self, wfs32):
        p = self.params
        thr = np.float32(p.DISCRIMINATION_THRESHOLD)
        H = int(p.MAX_ADC_VALUES)
        P, T = wfs32.shape
        qc = np.cumsum((wfs32 * np.float32(p.t_sampling)).astype(np.float32), axis=-1, dtype=np.float32)
        interval = R.fee_interval(p)
        rows = np.arange(P)
        self.idx = np.zeros((P, H), np.int64)
        self.e = np.zeros((P, H), np.int64)
        self.e2 = np.zeros((P, H), np.int64)
        self.cond = np.zeros((P, H), bool)
        self.masks = np.zeros((H, P, T), bool)
        self.adc_f32 = np.zeros((P, H), np.float32)
        for h in range(H):
            cross = (qc[:, 1:] >= thr) & (qc[:, :-1] <= thr)
            has = cross.any(1)
            idx = np.where(has, cross.argmax(1), T - 2)
            e = np.minimum(idx + 1 + interval, T - 1)
            adc = qc[rows, e]
            cond = (adc < thr) | (idx == T - 2)
            e2 = np.minimum(idx + 2 + interval, T - 1)
            r = qc[rows, e2]
            c2 = (qc - r[:, None]).astype(np.float32)
            self.masks[h] = ~(c2 < 0)
            qc = np.where(c2 < 0, np.float32(0), c2).astype(np.float32)
            self.idx[:, h], self.e[:, h], self.e2[:, h], self.cond[:, h] = idx, e, e2, cond
            self.adc_f32[:, h] = np.where(cond, 0, adc)
        # digitize branches: inside (0, ADC_COUNTS) or clamped
        pre = (self.adc_f32.astype(np.float64) * p.GAIN + p.V_PEDESTAL) - p.V_CM
        y = np.maximum(pre, 0) * p.ADC_COUNTS / (p.V_REF - p.V_CM)
        self.dig_lin = (pre > 0) & (y < p.ADC_COUNTS)
        self.dig_const = np.where(pre <= 0, 0.0, float(p.ADC_COUNTS))


def segment_quantities(fr: Frozen, th: dict):
    """n_e, sigma_T, long diffusion (ticks), t0 in float64 (quench + drift)."""
    p = fr.params
    v = vdrift64(p, th["eField"])
    erho = th["eField"] * th["lArDensity"]
    if fr.mode == 2:                                       # Birks, quenching_jax.py:23-25
        R_ = th["Ab"] / (1 + th["kb"] * fr.dEdx / erho)
    elif fr.mode == 1:                                     # Box, :18-21
        csi = p.beta * fr.dEdx / erho
        R_ = np.where(fr.recomb_on, np.log(p.alpha + csi) / csi, 0.0)
    else:                                                  # ellipsoid Box, :30-35, :55-66
        csi = fr.b_phi * fr.dEdx / erho
        R_ = np.where(fr.recomb_on, np.log(p.alpha + csi) / (csi + 1e-10), 0.0)
    dist = np.abs(fr.z - fr.z_anode) + 1e-6
    t = dist / v
    ne = R_ * fr.dE * p.MeVToElectrons * np.exp(-t / th["lifetime"]) * fr.mask
    sigL = np.sqrt(2 * t * th["long_diff"])
    sigT = np.sqrt(2 * t * th["tran_diff"])
    t0 = np.abs(fr.z - fr.z_cathode) / v
    ld = sigL / v / p.t_sampling
    return ne, sigT, ld, t0


def _weights(edges, x0, sig):
    e = np.ones((x0.shape[0], 6), dtype=np.result_type(sig, x0, np.float64))
    e[:, 0] = -1
    e[:, 1:5] = special.erf((edges[None, 1:5] - x0[:, None]) / (np.sqrt(2.0) * sig[:, None]))
    return 0.5 * (e[:, 1:] - e[:, :-1])


def waveforms64(fr: Frozen, th: dict):
    """LUT accumulation (sim_jax.py:141-286) in float64, decisions frozen."""
    p = fr.params
    d = fr.d
    ne, sigT, ld, t0 = segment_quantities(fr, th)
    Tb = fr.T
    Ntemp, Nx, Ny, Nt = Tb.shape
    L = int(p.signal_length)
    Nticks = R.n_ticks(p)
    P = fr.unique.shape[0]
    cplx = np.iscomplexobj(ne)
    out = np.zeros(P * Nticks, dtype=np.complex128 if cplx else np.float64)
    ex = _weights(fr.edges, fr.x0, sigT)
    ey = _weights(fr.edges, fr.y0, sigT)
    S = ne.shape[0]
    frac = t0 / p.t_sampling - fr.cath
    i = fr.tidx
    x0, x1, x2 = fr.tmpl[i - 1], fr.tmpl[i], fr.tmpl[i + 1]
    a = (ld - x1) * (ld - x2) / ((x0 - x1) * (x0 - x2))
    b = (ld - x0) * (ld - x2) / ((x1 - x0) * (x1 - x2))
    c = (ld - x0) * (ld - x1) / ((x2 - x0) * (x2 - x1))
    ks = np.arange(L)
    st0 = Nt - L - fr.cath
    tt0 = st0[:, None] + ks[None, :]
    col0 = np.where((tt0 <= 0) | (tt0 >= Nticks - 1), 0, tt0 + 1)
    tt1 = tt0 - 1
    col1 = np.where((tt1 <= 0) | (tt1 >= Nticks - 1), 0, tt1 + 1)
    cc0 = np.where((st0 <= 0) | (st0 >= Nticks - 1), 0, st0)
    cc1 = np.where((st0 - 1 <= 0) | (st0 - 1 >= Nticks - 1), 0, st0 - 1)

    def add(rows, cols, vals):
        idx = (rows[:, None] * Nticks + cols) if cols.ndim == 2 else rows * Nticks + cols
        idx = idx.ravel()
        ok = (idx >= 0) & (rows.repeat(idx.size // rows.size) >= 0)
        v = vals.ravel()[ok]
        if cplx:
            out[:] += np.bincount(idx[ok], weights=v.real, minlength=out.size) + \
                1j * np.bincount(idx[ok], weights=v.imag, minlength=out.size)
        else:
            out[:] += np.bincount(idx[ok], weights=v, minlength=out.size)

    def renum(pids, neigh):
        r = np.searchsorted(fr.unique, pids)
        rc = np.minimum(r, P - 1)
        m = (r < P) & (fr.unique[rc] == pids)
        return np.where(m, r, 0 if neigh else -1)

    ci = d["currents_idx"].reshape(S, 25, 2)
    pix = d["pixels"].reshape(S, 25)
    w = (ex[:, :, None] * ey[:, None, :]).reshape(S, 25) * ne[:, None]
    for k in range(25):
        r = renum(pix[:, k], False)
        vi = Tb[i, ci[:, k, 0], ci[:, k, 1], Nt - L:].astype(np.float64)
        vm = Tb[i - 1, ci[:, k, 0], ci[:, k, 1], Nt - L:].astype(np.float64)
        vp = Tb[i + 1, ci[:, k, 0], ci[:, k, 1], Nt - L:].astype(np.float64)
        m2 = (vi * b[:, None] + vm * a[:, None] + vp * c[:, None]) * w[:, k:k + 1]
        add(r, col0, m2 * (1 - frac)[:, None])
        add(r, col1, m2 * frac[:, None])
        cum = np.cumsum(Tb[i, ci[:, k, 0], ci[:, k, 1], :], axis=-1, dtype=np.float64)
        rows = np.arange(S)
        interp = cum[rows, fr.cath] * (1 - frac) + cum[rows, np.minimum(fr.cath + 1, Nt - 1)] * frac
        dm = (cum[rows, Nt - L] - interp) * w[:, k]
        add(r, cc0, dm * (1 - frac))
        add(r, cc1, dm * frac)
    nn = (2 * p.number_pix_neighbors + 1) ** 2
    cin = d["currents_idx_neigh"].reshape(S, nn, 2)
    pid = d["pIDs_neigh"].reshape(S, nn)
    cum0 = np.cumsum(Tb[0], axis=-1, dtype=np.float64)
    for k in range(nn):
        r = renum(pid[:, k], True)
        vals = Tb[0, cin[:, k, 0], cin[:, k, 1], Nt - L:].astype(np.float64) * ne[:, None]
        add(r, col0, vals * (1 - frac)[:, None])
        add(r, col1, vals * frac[:, None])
        cr = cum0[cin[:, k, 0], cin[:, k, 1]]
        rows = np.arange(S)
        interp = cr[rows, fr.cath] * (1 - frac) + cr[rows, np.minimum(fr.cath + 1, Nt - 1)] * frac
        dn = (cr[rows, Nt - L] - interp) * ne
        add(r, cc0, dn * (1 - frac))
        add(r, cc1, dn * frac)
    return out.reshape(P, Nticks)[:, 1:]


def fee64(fr: Frozen, w):
    """Frozen-decision FEE + digitize on given float64 waveforms."""
    p = fr.params
    C = np.cumsum(w * p.t_sampling, axis=-1)
    H = int(p.MAX_ADC_VALUES)
    rows = np.arange(C.shape[0])
    adc = np.zeros((C.shape[0], H))
    for h in range(H):
        v = C[rows, fr.e[:, h]]
        adc[:, h] = np.where(fr.cond[:, h], 0.0, v)
        Rv = C[rows, fr.e2[:, h]]
        C = np.where(fr.masks[h], C - Rv[:, None], 0.0)
    pre = (adc * p.GAIN + p.V_PEDESTAL) - p.V_CM
    lin = pre * p.ADC_COUNTS / (p.V_REF - p.V_CM)
    return np.where(fr.dig_lin, lin, fr.dig_const)


def adc64(fr: Frozen, th: dict):
    """Frozen-decision ADC grid at parameters th."""
    return fee64(fr, waveforms64(fr, th))


def fee_adjoint64(fr: Frozen, g_adc, dtype=np.float64):
    """dL/dW for a cotangent on the ADC grid (frozen FEE, reverse mode), in
    ``dtype`` (float64 by default; float32 is the reference's own type)."""
    p = fr.params
    ft = np.dtype(dtype)
    P, H = g_adc.shape
    T = fr.masks.shape[2]
    rows = np.arange(P)
    gint = np.where(fr.dig_lin, np.asarray(g_adc, ft) * ft.type(p.GAIN * p.ADC_COUNTS / (p.V_REF - p.V_CM)),
                    ft.type(0)).astype(ft)
    g = np.zeros((P, T), ft)
    for h in range(H - 1, -1, -1):
        m = fr.masks[h]
        S = (g * m).sum(axis=1)
        g = np.where(m, g, 0.0)
        np.add.at(g, (rows, fr.e2[:, h]), -S)
        np.add.at(g, (rows, fr.e[:, h]), np.where(fr.cond[:, h], ft.type(0), gint[:, h]))
    return (np.cumsum(g[:, ::-1], axis=1, dtype=ft)[:, ::-1] * ft.type(p.t_sampling)).astype(ft)


def loss_cotangent(fr: Frozen, th: dict):
    """Waveform cotangent g_W (all rows) of the SSE loss at th."""
    adc = adc64(fr, th)
    g = np.zeros_like(adc)
    g[fr.valid] = 2 * (adc[fr.valid] - fr.tgt)
    return fee_adjoint64(fr, g)


def complex_step_gradient(fr: Frozen, th0: dict, h=1e-30):
    """Exact pathwise gradient: <g_W, dW/dtheta> with dW/dtheta by complex step."""
    gw = loss_cotangent(fr, th0)
    out = {}
    for k in GRAD_PARAMS:
        t = {q: complex(v) for q, v in th0.items()}
        step = h * max(abs(th0[k]), 1e-300)
        t[k] = th0[k] + 1j * step
        dw = waveforms64(fr, t).imag / step
        out[k] = float((gw * dw).sum())
    return out


def loss64(fr: Frozen, th: dict) -> float:
    adc = adc64(fr, th)[fr.valid]
    return float(((adc - fr.tgt) ** 2).sum()) + fr.const


def theta_dict(params):
    return {k: float(getattr(params, k)) for k in GRAD_PARAMS}


def fd_gradient(fr: Frozen, th0: dict, rel_step=1e-4):
    """Central finite differences of loss64, step rel_step * |theta|."""
    g = {}
    for k in GRAD_PARAMS:
        h = rel_step * abs(th0[k]) if th0[k] != 0 else rel_step
        tp, tm = dict(th0), dict(th0)
        tp[k] += h
        tm[k] -= h
        g[k] = (loss64(fr, tp) - loss64(fr, tm)) / (2 * h)
    return g


def _jacobian(fr: Frozen, th0: dict, h=1e-30):
    """d(n_e, sigma_T, ld, t0)/dtheta per segment by complex step."""
    J = {}
    for k in GRAD_PARAMS:
        t = {q: complex(v) for q, v in th0.items()}
        step = h * max(abs(th0[k]), 1e-300)
        t[k] = th0[k] + 1j * step
        J[k] = [q.imag / step for q in segment_quantities(fr, t)]
    return J


def adjoint64(fr: Frozen, th: dict, g_adc=None, dtype=np.float64):
    """Reverse-mode gradient (same chain rule as the CUDA adjoint, in
    float64): FEE adjoint -> waveform cotangent -> per-contribution partials
    (charge, transverse weights, template weights, sub-tick fraction) ->
    per-segment partials -> parameters.  Without ``g_adc`` the cotangent is
    that of loss64; with ``g_adc`` (valid rows x H) it is the vector-Jacobian
    product g_adc . dADC/dtheta.  With ``dtype=np.float32`` (and ``g_adc``
    given) the reverse pass runs in float32, the reference's own arithmetic
    type; the per-segment Jacobian and the final parameter sums stay
    float64."""
    p = fr.params
    d = fr.d
    ft = np.dtype(dtype)
    ne, sigT, ld, t0 = (q.astype(ft) for q in segment_quantities(fr, th))
    if g_adc is None:
        gw = loss_cotangent(fr, th)
    else:
        g = np.zeros((fr.unique.shape[0], int(p.MAX_ADC_VALUES)), ft)
        g[fr.valid] = g_adc
        gw = fee_adjoint64(fr, g, ft)
    P = gw.shape[0]
    Nticks = R.n_ticks(p)
    gwc = np.zeros((P, Nticks), ft)
    gwc[:, 1:] = gw
    Tb = fr.T
    Ntemp, Nx, Ny, Nt = Tb.shape
    L = int(p.signal_length)
    S = ne.shape[0]
    rows = np.arange(S)
    s64 = sigT.astype(np.float64)
    ex = _weights(fr.edges, fr.x0, s64).astype(ft)
    ey = _weights(fr.edges, fr.y0, s64).astype(ft)
    hs = 1e-30 * np.maximum(s64, 1e-300)
    dex = (_weights(fr.edges, fr.x0, s64 + 1j * hs).imag / hs[:, None]).astype(ft)
    dey = (_weights(fr.edges, fr.y0, s64 + 1j * hs).imag / hs[:, None]).astype(ft)
    frac = (t0 / ft.type(p.t_sampling) - fr.cath.astype(ft)).astype(ft)
    i = fr.tidx
    x0, x1, x2 = (fr.tmpl[j].astype(ft) for j in (i - 1, i, i + 1))
    a = (ld - x1) * (ld - x2) / ((x0 - x1) * (x0 - x2))
    b = (ld - x0) * (ld - x2) / ((x1 - x0) * (x1 - x2))
    c = (ld - x0) * (ld - x1) / ((x2 - x0) * (x2 - x1))
    da = ((ld - x1) + (ld - x2)) / ((x0 - x1) * (x0 - x2))
    db = ((ld - x0) + (ld - x2)) / ((x1 - x0) * (x1 - x2))
    dc = ((ld - x0) + (ld - x1)) / ((x2 - x0) * (x2 - x1))
    ks = np.arange(L)
    st0 = Nt - L - fr.cath
    tt0 = st0[:, None] + ks[None, :]
    col0 = np.where((tt0 <= 0) | (tt0 >= Nticks - 1), 0, tt0 + 1)
    tt1 = tt0 - 1
    col1 = np.where((tt1 <= 0) | (tt1 >= Nticks - 1), 0, tt1 + 1)
    cc0 = np.where((st0 <= 0) | (st0 >= Nticks - 1), 0, st0)
    cc1 = np.where((st0 - 1 <= 0) | (st0 - 1 >= Nticks - 1), 0, st0 - 1)
    A_ne = np.zeros(S, ft)
    A_sig = np.zeros(S, ft)
    A_a = np.zeros(S, ft)
    A_b = np.zeros(S, ft)
    A_c = np.zeros(S, ft)
    A_fr = np.zeros(S, ft)

    def renum(pids, neigh):
        r = np.searchsorted(fr.unique, pids)
        rc = np.minimum(r, P - 1)
        m = (r < P) & (fr.unique[rc] == pids)
        return np.where(m, r, 0 if neigh else -1)

    def gather(r, cols):
        ok = r >= 0
        rr = np.where(ok, r, 0)
        g = gwc[rr[:, None], cols] if cols.ndim == 2 else gwc[rr, cols]
        return np.where(ok[:, None] if cols.ndim == 2 else ok, g, ft.type(0))

    ci = d["currents_idx"].reshape(S, 25, 2)
    pix = d["pixels"].reshape(S, 25)
    wts = (ex[:, :, None] * ey[:, None, :]).reshape(S, 25)
    dwts = (dex[:, :, None] * ey[:, None, :] + ex[:, :, None] * dey[:, None, :]).reshape(S, 25)
    for k in range(25):
        r = renum(pix[:, k], False)
        vi = Tb[i, ci[:, k, 0], ci[:, k, 1], Nt - L:].astype(ft)
        vm = Tb[i - 1, ci[:, k, 0], ci[:, k, 1], Nt - L:].astype(ft)
        vp = Tb[i + 1, ci[:, k, 0], ci[:, k, 1], Nt - L:].astype(ft)
        B = vi * b[:, None] + vm * a[:, None] + vp * c[:, None]
        q = wts[:, k] * ne
        G0, G1 = gather(r, col0), gather(r, col1)
        gv = G0 * (1 - frac)[:, None] + G1 * frac[:, None]
        cum = np.cumsum(Tb[i, ci[:, k, 0], ci[:, k, 1], :], axis=-1, dtype=ft)
        c0v, c1v = cum[rows, fr.cath], cum[rows, np.minimum(fr.cath + 1, Nt - 1)]
        D = cum[rows, Nt - L] - (c0v * (1 - frac) + c1v * frac)
        Gc0, Gc1 = gather(r, cc0), gather(r, cc1)
        gd = Gc0 * (1 - frac) + Gc1 * frac
        dq = (B * gv).sum(1) + gd * D
        A_ne += wts[:, k] * dq
        A_sig += ne * dwts[:, k] * dq
        A_a += q * (vm * gv).sum(1)
        A_b += q * (vi * gv).sum(1)
        A_c += q * (vp * gv).sum(1)
        A_fr += (B * q[:, None] * (G1 - G0)).sum(1) + D * q * (Gc1 - Gc0) + gd * q * (c0v - c1v)
    nn = (2 * p.number_pix_neighbors + 1) ** 2
    cin = d["currents_idx_neigh"].reshape(S, nn, 2)
    pid = d["pIDs_neigh"].reshape(S, nn)
    cum0 = np.cumsum(Tb[0], axis=-1, dtype=ft)
    for k in range(nn):
        r = renum(pid[:, k], True)
        T0 = Tb[0, cin[:, k, 0], cin[:, k, 1], Nt - L:].astype(ft)
        G0, G1 = gather(r, col0), gather(r, col1)
        gv = G0 * (1 - frac)[:, None] + G1 * frac[:, None]
        cr = cum0[cin[:, k, 0], cin[:, k, 1]]
        c0v, c1v = cr[rows, fr.cath], cr[rows, np.minimum(fr.cath + 1, Nt - 1)]
        D = cr[rows, Nt - L] - (c0v * (1 - frac) + c1v * frac)
        Gc0, Gc1 = gather(r, cc0), gather(r, cc1)
        gd = Gc0 * (1 - frac) + Gc1 * frac
        A_ne += (T0 * gv).sum(1) + gd * D
        A_fr += (T0 * ne[:, None] * (G1 - G0)).sum(1) + D * ne * (Gc1 - Gc0) + gd * ne * (c0v - c1v)
    A_ld = A_a * da.astype(ft) + A_b * db.astype(ft) + A_c * dc.astype(ft)
    A_t0 = A_fr / ft.type(p.t_sampling)
    J = _jacobian(fr, th)
    return {k: float((A_ne * J[k][0] + A_sig * J[k][1] + A_ld * J[k][2] + A_t0 * J[k][3]).sum()) for k in GRAD_PARAMS}


# ---------------------------------------------------------------- parametrised mode

def param_waveforms64(params, tracks, fields, normals, th: dict, frozen=None):
    """Parametrised-mode waveforms (sim_jax.py:122-139, :289-335;
    detsim_jax.py:376-400, :440-474, :581-639, :207-228) in float64 / complex
    (complex-step ready), with the discrete decisions of the float32
    forward frozen: TPC plane and mask, electron pixel, t0 tick, the
    min(a, 1) branch.  Returns (W (P_valid, T), frozen, valid pixel ids)."""
    p = params
    f = tuple(fields)
    cplx = any(isinstance(v, complex) for v in th.values())
    dt = np.complex128 if cplx else np.float64
    sh = R.shift_tracks(p, tracks, f)
    x = sh[:, f.index("x")].astype(np.float64)
    y = sh[:, f.index("y")].astype(np.float64)
    z = sh[:, f.index("z")].astype(np.float64)
    dE = sh[:, f.index("dE")].astype(np.float64)
    dEdx = sh[:, f.index("dEdx")].astype(np.float64)
    nrm = np.asarray(normals, np.float64)
    if frozen is None:
        mask, plane = R.tpc_membership(p, sh[:, f.index("x")], sh[:, f.index("y")], sh[:, f.index("z")])
        # float32 forward for the decisions
        t32 = R.drift(p, R.quench(p, sh, f), f)
        e32 = R.generate_electrons(p, t32, f, normals)
        pids = R.get_pixels(p, e32, f).ravel()
        xp, yp, pl, _ = R.id2pixel(p, pids)
        coords = R.get_pixel_coordinates(p, xp, yp, pl)
        t0_tick, _ = R.current_mc(p, e32, coords, f)
        ev = sh[:, f.index("eventID")].astype(int)
        valid = np.unique(pids[(pids >= 0)])
        frozen = dict(mask=mask.astype(np.float64), plane=plane, pids=pids, coords=coords.astype(np.float64),
                      t0_tick=t0_tick, valid=valid, ev=ev)
    fr = frozen
    E, rho = th["eField"], th["lArDensity"]
    Rb = th["Ab"] / (1 + th["kb"] * dEdx / (E * rho))                          # quenching_jax.py:23-25
    ne0 = Rb * dE * p.MeVToElectrons
    b = np.asarray(p.tpc_borders, np.float32)[fr["plane"]]
    za = b[:, 2, 0].astype(np.float64)
    dist = np.abs(z - za) + 1e-6
    v = vdrift64(p, E)
    tdr = dist / v
    ne = ne0 * np.exp(-tdr / th["lifetime"]) * fr["mask"]
    sT = np.sqrt(2 * tdr * th["tran_diff"])
    sL = np.sqrt(2 * tdr * th["long_diff"])
    xe = x + nrm[:, 0] * sT
    ye = y + nrm[:, 1] * sT
    ux = xe - fr["coords"][:, 0]
    uy = ye - fr["coords"][:, 1]
    xd = np.sign(np.real(ux)) * ux
    yd = np.sign(np.real(uy)) * uy
    uz = z - za
    t0 = np.sign(uz) * uz / v
    t0f = t0 - fr["t0_tick"] * p.t_sampling
    sig = sL / v
    nt = int(5 / p.t_sampling) + 1
    tk = R.jax_linspace_f32(0, 5, nt).astype(np.float64)
    dts = 5.0 / (nt - 1)
    Bp = (1.060, -0.909, -0.909, 5.856, 0.207, 0.207)
    Cp = (0.679, -1.083, -1.083, 8.772, -5.521, -5.521)
    Dp = (2.644, -9.174, -9.174, 13.483, 45.887, 45.887)
    Tp = (2.948, -2.705, -2.705, 4.825, 20.814, 20.814)

    def quad(c):
        return c[0] + c[1] * xd + c[2] * yd + c[3] * xd * yd + c[4] * xd * xd + c[5] * yd * yd

    a = quad(Bp)
    a = np.where(np.real(a) < 1, a, 1.0)
    bq, cq = quad(Cp), quad(Dp)
    st0 = t0f + quad(Tp)

    def ied(xx, loc, scale, diff):
        lam = 1 / scale
        coeff = lam / 2
        expo = coeff * (2 * loc + lam * diff ** 2 - 2 * xx)
        pdf = coeff * np.exp(expo) * special.erfc((loc + lam * diff ** 2 - xx) / (np.sqrt(2) * diff))
        return 0.5 * special.erf((xx - loc) / (np.sqrt(2) * diff)) - pdf / lam

    X = -tk[None, :]
    loc = (-st0)[:, None]
    dd = sig[:, None]

    def shape(scale):
        up = ied(X + dts / 2, loc, scale[:, None], dd)
        lo = ied(X - dts / 2, loc, scale[:, None], dd)
        return (up - lo) / (lo[:, :1] - up[:, -1:]) / dts

    cur = (a[:, None] * shape(bq) + (1 - a[:, None]) * shape(cq)) * ne[:, None]
    Nt = R.n_ticks(p)
    start = fr["t0_tick"] - nt
    tt = start[:, None] + np.arange(nt)[None, :]
    col = np.where((tt < 0) | (tt >= Nt - 1), 0, tt + 1)
    rows = np.searchsorted(fr["valid"], fr["pids"])
    ok = (fr["pids"] >= 0) & (rows < len(fr["valid"]))
    W = np.zeros((len(fr["valid"]), Nt), dtype=dt)
    for s in np.nonzero(ok)[0]:
        np.add.at(W[rows[s]], col[s], cur[s])
    return W[:, 1:], frozen, fr["valid"]
