"""float32 numpy restatement of the larnd-sim-jax simulate path (oracle).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Every function follows one reference function and keeps its float32
operation order; Python-float parameter expressions are evaluated in float64
and rounded once, as the reference's static parameters are.  Integer and
index arithmetic is reproduced exactly (floor division and modulo with
Python/JAX semantics, int32 pixel-id packing).

Summation: the reference sums waveform contributions with an unsorted
``segment_sum``; here contributions are summed in float64 (``np.bincount``)
and rounded to float32 once, which is at least as accurate as any float32
order.  Garbage rows (pixel id < 0) are reproduced as the reference computes
them.
"""

from __future__ import annotations

import numpy as np
from scipy import special

F32 = np.float32
I32 = np.int32


# ---------------------------------------------------------------- scalars

def get_vdrift(params) -> float:
    """consts_jax.py:192-217, float64 (static parameters)."""
    a0, a1, a2, a3, a4, a5 = params.ELECTRON_MOBILITY_PARAMS
    e = params.eField
    num = a0 + a1 * e + a2 * pow(e, 1.5) + a3 * pow(e, 2.5)
    denom = 1 + (a1 / a0) * e + a4 * pow(e, 2) + a5 * pow(e, 3)
    temp_corr = pow(params.temperature / 89, -1.5)
    return num / denom * temp_corr / 1000 * e


def vdrift32(params):
    return F32(get_vdrift(params))


def n_ticks(params) -> int:
    return int(params.time_interval[1] / params.t_sampling) + 1   # sim_jax.py:147


def jax_linspace_f32(start, stop, num):
    """jax.numpy.linspace arithmetic in float32 (start*(1-s)+stop*s, exact endpoint)."""
    s, e = F32(start), F32(stop)
    div = num - 1
    step = (np.arange(div, dtype=F32) / F32(div)).astype(F32)
    return np.concatenate([(s * (F32(1) - step) + e * step).astype(F32), [e]]).astype(F32)


def floor_divide_f32(a, b):
    """jnp.floor_divide on float32 (fmod-based divmod, rounded quotient)."""
    a = np.asarray(a, F32)
    b = F32(b)
    mod = np.fmod(a, b)
    div = ((a - mod) / b).astype(F32)
    ind = (mod != 0) & ((b < 0) != (mod < 0))
    div = np.where(ind, div - F32(1), div).astype(F32)
    # lax.round rounds half away from zero
    return (np.sign(div) * np.floor(np.abs(div) + F32(0.5))).astype(F32)


def remainder_f32(a, b):
    """jnp.remainder on float32 (sign of the divisor)."""
    a = np.asarray(a, F32)
    b = F32(b)
    mod = np.fmod(a, b)
    plus = (mod != 0) & ((mod < 0) != (b < 0))
    return np.where(plus, mod + b, mod).astype(F32)


def erf32(x):
    return special.erf(np.asarray(x, F32)).astype(F32)


# ---------------------------------------------------------------- tracks

def shift_tracks(params, tracks, fields):
    """sim_jax.py:108-119."""
    t = np.array(tracks, dtype=F32, copy=True)
    for ax, sh in (("x", params.shift_x), ("y", params.shift_y), ("z", params.shift_z)):
        for suffix in ("_start", "_end", ""):
            c = fields.index(ax + suffix)
            t[:, c] = t[:, c] - F32(sh)
    return t


def quench(params, tracks, fields):
    """quenching_jax.py:37-74 (Box, Birks, ellipsoid Box)."""
    mode = getattr(params.recombination_mode, "value", params.recombination_mode)
    dEdx = tracks[:, fields.index("dEdx")]
    erho = params.eField * params.lArDensity
    if mode == 1:
        csi = (F32(params.beta) * dEdx) / F32(erho)
        recomb = np.maximum(F32(0), np.log(F32(params.alpha) + csi) / csi)
    elif mode == 2:
        recomb = F32(params.Ab) / (F32(1) + (F32(params.kb) * dEdx) / F32(erho))
    elif mode == 3:
        z_end = tracks[:, fields.index("z_end")]
        z_start = tracks[:, fields.index("z_start")]
        cosphi = np.abs(z_end - z_start) / (tracks[:, fields.index("dx")] + F32(1e-10))
        cos2 = cosphi ** 2
        b_phi = F32(params.beta) / np.sqrt((F32(1) - cos2) + F32(1.0 / params.R_param ** 2) * cos2)
        csi = (b_phi * dEdx) / F32(erho)
        recomb = np.maximum(F32(0), np.log(F32(params.alpha) + csi) / (csi + F32(1e-10)))
    else:
        raise ValueError(f"Invalid recombination mode {params.recombination_mode}")
    out = np.array(tracks, copy=True)
    out[:, fields.index("n_electrons")] = (recomb * tracks[:, fields.index("dE")]) * F32(params.MeVToElectrons)
    return out.astype(F32)


def tpc_membership(params, x, y, z):
    """TPC membership mask and pixel plane (drifting_jax.py:21-35)."""
    b = np.asarray(params.tpc_borders, F32)
    m = F32(params.size_margin)
    zmin = np.minimum(b[:, 2, 1] - m, b[:, 2, 0] - m)
    zmax = np.maximum(b[:, 2, 1] + m, b[:, 2, 0] + m)
    cond = x[:, None] >= (b[:, 0, 0] - m)[None]
    cond &= x[:, None] <= (b[:, 0, 1] + m)[None]
    cond &= y[:, None] >= (b[:, 1, 0] - m)[None]
    cond &= y[:, None] <= (b[:, 1, 1] + m)[None]
    cond &= z[:, None] >= zmin[None]
    cond &= z[:, None] <= zmax[None]
    return cond.sum(axis=-1) >= 1, cond.astype(int).argmax(axis=-1)


def drift(params, tracks, fields):
    """drifting_jax.py:18-58."""
    t = np.array(tracks, dtype=F32, copy=True)
    x, y, z = (t[:, fields.index(a)] for a in "xyz")
    mask, plane = tpc_membership(params, x, y, z)
    b = np.asarray(params.tpc_borders, F32)
    z_anode = b[plane, 2, 0]
    v = vdrift32(params)
    drift_distance = np.abs(z - z_anode) + F32(1e-6)
    zs, ze = t[:, fields.index("z_start")], t[:, fields.index("z_end")]
    drift_start = np.abs(np.minimum(zs, ze) - z_anode)
    drift_end = np.abs(np.maximum(zs, ze) - z_anode)
    t[:, fields.index("pixel_plane")] = plane
    drift_time = drift_distance / v
    lifetime_red = np.exp(-drift_time / F32(params.lifetime)).astype(F32)
    mf = mask.astype(F32)
    ne = t[:, fields.index("n_electrons")]
    t[:, fields.index("n_electrons")] = (ne * lifetime_red) * mf
    t[:, fields.index("long_diff")] = np.sqrt((drift_time * F32(2)) * F32(params.long_diff))
    t[:, fields.index("tran_diff")] = np.sqrt((drift_time * F32(2)) * F32(params.tran_diff))
    t0 = t[:, fields.index("t0")]
    t[:, fields.index("t")] = (t[:, fields.index("t")] + drift_time * mf) + t0
    t[:, fields.index("t_start")] = (t[:, fields.index("t_start")] + (np.minimum(drift_start, drift_end) / v) * mf) + t0
    t[:, fields.index("t_end")] = (t[:, fields.index("t_end")] + (np.maximum(drift_start, drift_end) / v) * mf) + t0
    return t.astype(F32)


def pixel2id(params, px, py, plane, event):
    """detsim_jax.py:230-244 with int32 packing (JAX runs without x64)."""
    nx, ny = int(params.n_pixels_x), int(params.n_pixels_y)
    ntpc = int(np.asarray(params.tpc_borders).shape[0])
    px, py = np.asarray(px, np.int64), np.asarray(py, np.int64)
    outside = (px >= nx) | (py >= ny) | (px < 0) | (py < 0)
    pid = ((np.asarray(event, np.int64) * ntpc + np.asarray(plane, np.int64)) * ny + py) * nx + px
    pid = pid.astype(np.int64).astype(I32)    # int32 wrap-around like the reference
    return np.where(outside, I32(-1), pid).astype(I32)


def id2pixel(params, pid):
    """detsim_jax.py:264-278 (Python floor division / modulo)."""
    pid = np.asarray(pid, np.int64)
    nx, ny = int(params.n_pixels_x), int(params.n_pixels_y)
    ntpc = int(np.asarray(params.tpc_borders).shape[0])
    return (pid % nx, (pid // nx) % ny, (pid // (nx * ny)) % ntpc, pid // (nx * ny * ntpc))


def get_pixel_coordinates(params, xpitch, ypitch, plane):
    """detsim_jax.py:296-306."""
    b = np.asarray(params.tpc_borders, F32)[np.asarray(plane, int)]
    pitch = params.pixel_pitch
    pix_x = (np.asarray(xpitch).astype(F32) * F32(pitch) + b[..., 0, 0]) + F32(pitch / 2)
    pix_y = (np.asarray(ypitch).astype(F32) * F32(pitch) + b[..., 1, 0]) + F32(pitch / 2)
    return np.stack([pix_x, pix_y], axis=-1).astype(F32)


def get_hit_z(params, ticks, plane):
    """detsim_jax.py:308-319 (fixed_v=False)."""
    b = np.asarray(params.tpc_borders, F32)[np.asarray(plane, int)]
    z_anode, z_high = b[..., 2, 0], b[..., 2, 1]
    return (z_anode + ((np.asarray(ticks, F32) * F32(params.t_sampling)) * vdrift32(params))
            * np.sign(z_high - z_anode)).astype(F32)


# ---------------------------------------------------------------- LUT mode

def gaussian_1d_integral_new(bin_edges, x0, std):
    """detsim_jax.py:332-341: bins of a unit Gaussian, open outer edges."""
    edges = (bin_edges[None, :] - x0[:, None]).astype(F32)
    e = np.ones_like(edges)
    e[:, 0] = -1
    e[:, 1:-1] = erf32(edges[:, 1:-1] / (F32(np.sqrt(F32(2))) * std[:, None]))
    return (F32(0.5) * (e[:, 1:] - e[:, :-1])).astype(F32)


def simulate_drift_new(params, tracks, fields):
    """sim_jax.py:374-453: per-segment charge, bins, pixel ids, LUT indices."""
    t = shift_tracks(params, tracks, fields)
    t = quench(params, t, fields)
    t = drift(params, t, fields)
    x, y, z = (t[:, fields.index(a)] for a in "xyz")
    plane = t[:, fields.index("pixel_plane")].astype(int)
    event = t[:, fields.index("eventID")].astype(int)
    b = np.asarray(params.tpc_borders, F32)[plane]
    nb = params.nb_sampling_bins_per_pixel
    width = params.pixel_pitch / nb
    # get_bin_shifts, detsim_jax.py:493-512
    bx = floor_divide_f32(x - b[:, 0, 0], width).astype(np.int64)
    by = floor_divide_f32(y - b[:, 1, 0], width).astype(np.int64)
    ntd = params.nb_tran_diff_bins
    sym = (ntd - 1) // 2
    edges = jax_linspace_f32(-sym * width, (sym + 1) * width, ntd + 1)
    x0 = remainder_f32(x - b[:, 0, 0], width)
    y0 = remainder_f32(y - b[:, 1, 0], width)
    sigma = t[:, fields.index("tran_diff")]
    ex = gaussian_1d_integral_new(edges, x0, sigma)
    ey = gaussian_1d_integral_new(edges, y0, sigma)
    w = (ex[:, :, None] * ey[:, None, :]).astype(F32)                       # density_2d
    ne = t[:, fields.index("n_electrons")]
    nelectrons = (w * ne[:, None, None]).reshape(-1).astype(F32)
    v = vdrift32(params)
    z_cathode = np.asarray(params.tpc_borders, F32)[plane, 2, 1]
    t0 = (np.abs(z - z_cathode) / v).astype(F32)
    long_diff = ((t[:, fields.index("long_diff")] / v) / F32(params.t_sampling)).astype(F32)
    S = t.shape[0]
    sh = np.arange(-sym, sym + 1)
    bxs = bx[:, None] + sh[None, :]                                          # (S,5)
    bys = by[:, None] + sh[None, :]
    pxs, pys = bxs // nb, bys // nb
    pixels = pixel2id(params, pxs[:, :, None], pys[:, None, :], plane[:, None, None], event[:, None, None])
    main_pixels = pixels[:, sym, sym]
    cix = np.abs((bxs % nb - nb // 2).astype(F32) + F32(0.5)).astype(int)   # (S,5)
    ciy = np.abs((bys % nb - nb // 2).astype(F32) + F32(0.5)).astype(int)
    currents_idx = np.stack([np.broadcast_to(cix[:, :, None], (S, ntd, ntd)),
                             np.broadcast_to(ciy[:, None, :], (S, ntd, ntd))], axis=-1).reshape(-1, 2)
    n = params.number_pix_neighbors
    g = np.arange(-n, n + 1)
    cnx = np.abs(((bx % nb - nb // 2).astype(F32) + F32(0.5))[:, None] - (g * nb).astype(F32)[None, :]).astype(int)
    cny = np.abs(((by % nb - nb // 2).astype(F32) + F32(0.5))[:, None] - (g * nb).astype(F32)[None, :]).astype(int)
    currents_idx_neigh = np.stack([np.broadcast_to(cnx[:, :, None], (S, 2 * n + 1, 2 * n + 1)),
                                   np.broadcast_to(cny[:, None, :], (S, 2 * n + 1, 2 * n + 1))], axis=-1).reshape(-1, 2)
    ppx, ppy = pxs[:, sym], pys[:, sym]
    pIDs = pixel2id(params, (ppx[:, None] + g[None, :])[:, :, None], (ppy[:, None] + g[None, :])[:, None, :],
                    plane[:, None, None], event[:, None, None]).copy()
    pIDs[:, n, n] = -999
    return dict(main_pixels=main_pixels, pixels=pixels, nelectrons=nelectrons,
                t0_after_diff=np.repeat(t0, ntd * ntd), long_diff=np.repeat(long_diff, ntd * ntd),
                currents_idx=currents_idx, pIDs_neigh=pIDs, currents_idx_neigh=currents_idx_neigh,
                nelectrons_neigh=ne.astype(F32), t0_neigh=t0, t0=t0, ld=long_diff, ne=ne.astype(F32),
                ex=ex, ey=ey, bx=bx, by=by, plane=plane, event=event, sigmaT=sigma,
                tracks=t)


_SIZE_HISTORY: dict = {}


def pad_size(cur_size, tag, pad_threshold=0.05, history=None):
    """sim_jax.py:61-102 (size-bucket history; an explicit dict may be passed)."""
    hist = _SIZE_HISTORY if history is None else history
    scalar = isinstance(cur_size, (int, np.integer))
    cur = (int(cur_size),) if scalar else tuple(int(c) for c in cur_size)
    sizes = hist.setdefault(tag, [])
    if cur in sizes:
        return cur[0] if scalar else cur
    for s in sizes:
        if all(c <= q <= c * (1 + pad_threshold) for c, q in zip(cur, s)):
            return s[0] if scalar else s
    new = tuple(int(c * (1 + pad_threshold / 2) + 0.5) for c in cur)
    sizes.append(new)
    sizes.sort()
    return new[0] if scalar else new


def unique_pixel_rows(main_pixels, padded_size=None, history=None):
    """sim_jax.py:717-721: unique main pixels, an appended -1, padding, sort."""
    u = np.unique(main_pixels.ravel())
    u = np.append(u, -1)
    if padded_size is None:
        padded_size = pad_size(u.shape[0], "unique_pixels", 0.2, history)
    u = np.sort(np.pad(u, (0, padded_size - u.shape[0]), constant_values=-1)).astype(I32)
    return u


def simulate_signals(params, unique_pixels, d, response_template, seg_chunk=1024):
    """sim_jax.py:141-286 (LUT accumulation) -> waveforms (P, Nticks)."""
    P = unique_pixels.shape[0]
    Nticks = n_ticks(params)
    Ntemp, Nx, Ny, Nt = response_template.shape
    L = int(params.signal_length)
    ts = F32(params.t_sampling)
    tmpl = np.asarray(params.long_diff_template, F32)
    T = np.asarray(response_template, F32)
    out = np.zeros(P * Nticks, dtype=np.float64)
    ntd2 = params.nb_tran_diff_bins ** 2
    nneigh = (2 * params.number_pix_neighbors + 1) ** 2
    S = d["main_pixels"].shape[0]
    ks = np.arange(L)

    def renum_main(pix):
        r = np.searchsorted(unique_pixels, pix, side="left")
        rc = np.minimum(r, P - 1)
        return np.where(unique_pixels[rc] == pix, r, -1)

    def renum_neigh(pid):
        r = np.searchsorted(unique_pixels, pid, side="left")
        rc = np.minimum(r, P - 1)
        ok = (r < P) & (unique_pixels[rc] == pid)
        return np.where(ok, r, 0)

    # cumulative sums (sim_jax.py:228), evaluated only along the used rows
    def cum_rows(ti, cx, cy):
        keys = (ti * Nx + cx) * Ny + cy
        ukeys, inv = np.unique(keys, return_inverse=True)
        rows = T.reshape(Ntemp * Nx * Ny, Nt)[ukeys]
        return np.cumsum(rows, axis=-1, dtype=F32), inv.ravel()

    def window_ticks(start):
        tt = start[:, None] + ks[None, :]
        return np.where((tt <= 0) | (tt >= Nticks - 1), 0, tt + 1)

    def corr_tick(start):
        return np.where((start <= 0) | (start >= Nticks - 1), 0, start)

    def add(idx, val):
        idx = idx.ravel()
        val = val.ravel().astype(np.float64)
        ok = (idx >= 0) & (idx < P * Nticks)
        out[:] += np.bincount(idx[ok], weights=val[ok], minlength=P * Nticks)

    for s0 in range(0, S, seg_chunk):
        s1 = min(S, s0 + seg_chunk)
        # --- main bins
        sl = slice(s0 * ntd2, s1 * ntd2)
        pix = d["pixels"][s0:s1].ravel()
        renum = renum_main(pix)
        t0 = d["t0_after_diff"][sl]
        ft = (t0 / ts).astype(F32)
        cat = np.clip(np.floor(ft).astype(np.int64), 0, Nt - 1)
        frac = (ft - cat.astype(F32)).astype(F32)
        ld = d["long_diff"][sl]
        idx = np.clip(np.searchsorted(tmpl, ld, side="left"), 1, tmpl.shape[0] - 2)
        x0, x1, x2 = tmpl[idx - 1], tmpl[idx], tmpl[idx + 1]
        a = ((ld - x1) * (ld - x2)) / ((x0 - x1) * (x0 - x2))
        b = ((ld - x0) * (ld - x2)) / ((x1 - x0) * (x1 - x2))
        c = ((ld - x0) * (ld - x1)) / ((x2 - x0) * (x2 - x1))
        st0 = Nt - L - cat
        st1 = st0 - 1
        ci = d["currents_idx"][sl]
        vi = T[idx, ci[:, 0], ci[:, 1], Nt - L:]
        vm = T[idx - 1, ci[:, 0], ci[:, 1], Nt - L:]
        vp = T[idx + 1, ci[:, 0], ci[:, 1], Nt - L:]
        q = d["nelectrons"][sl]
        main2d = (((vi * b[:, None]).astype(F32) + (vm * a[:, None]).astype(F32)).astype(F32)
                  + (vp * c[:, None]).astype(F32)).astype(F32) * q[:, None]
        base = renum[:, None] * Nticks
        add(base + window_ticks(st0), main2d * (F32(1) - frac)[:, None])
        add(base + window_ticks(st1), main2d * frac[:, None])
        cr, rows = cum_rows(idx, ci[:, 0], ci[:, 1])
        v0 = cr[rows, cat]
        v1 = cr[rows, np.clip(cat + 1, 0, Nt - 1)]
        interp = v0 * (F32(1) - frac) + v1 * frac
        dm = (cr[rows, Nt - L] - interp) * q
        add(corr_tick(st0) + renum * Nticks, dm * (F32(1) - frac))
        add(corr_tick(st1) + renum * Nticks, dm * frac)
        # --- neighbours (template 0, undiffused charge)
        pid = d["pIDs_neigh"][s0:s1].ravel()
        rn = renum_neigh(pid)
        ci = d["currents_idx_neigh"][s0 * nneigh:s1 * nneigh]
        seg = np.repeat(np.arange(s0, s1), nneigh)
        qn = d["nelectrons_neigh"][seg]
        t0n = d["t0_neigh"][seg]
        ft = (t0n / ts).astype(F32)
        cat = np.clip(np.floor(ft).astype(np.int64), 0, Nt - 1)
        frac = (ft - cat.astype(F32)).astype(F32)
        st0 = Nt - L - cat
        st1 = st0 - 1
        vals = T[0, ci[:, 0], ci[:, 1], Nt - L:] * qn[:, None]
        base = rn[:, None] * Nticks
        add(base + window_ticks(st0), vals * (F32(1) - frac)[:, None])
        add(base + window_ticks(st1), vals * frac[:, None])
        crs, rows = cum_rows(np.zeros_like(ci[:, 0]), ci[:, 0], ci[:, 1])
        v0 = crs[rows, cat]
        v1 = crs[rows, np.clip(cat + 1, 0, Nt - 1)]
        interp = v0 * (F32(1) - frac) + v1 * frac
        dn = (crs[rows, Nt - L] - interp) * qn
        add(corr_tick(st0) + rn * Nticks, dn * (F32(1) - frac))
        add(corr_tick(st1) + rn * Nticks, dn * frac)
    return out.astype(F32).reshape(P, Nticks)


def simulate_wfs(params, response_template, tracks, fields, padded_size=None, history=None):
    """sim_jax.py:689-736 -> (wfs[:, 1:], unique_pixels)."""
    d = simulate_drift_new(params, tracks, fields)
    unique = unique_pixel_rows(d["main_pixels"], padded_size, history)
    wfs = simulate_signals(params, unique, d, response_template)
    return wfs[:, 1:], unique


# ---------------------------------------------------------------- FEE

def fee_interval(params) -> int:
    return round((3 * params.CLOCK_CYCLE + params.ADC_HOLD_DELAY * params.CLOCK_CYCLE) / params.t_sampling)


def get_adc_values(params, wfs, normals=None, cumsum=None):
    """fee_jax.py:168-279 (self-trigger, integrate, reset).

    ``normals`` (P, 1 + 3*MAX_ADC_VALUES) are the standard-normal draws of
    the reference's noise terms in the order they are consumed: initial
    reset noise, then per hit (uncorrelated, pass, fail).  ``None`` means
    zero noise (the reference's --noise off).  ``cumsum`` optionally
    replaces the float32 sequential cumulative sum.
    """
    P, T = wfs.shape
    thr = F32(params.DISCRIMINATION_THRESHOLD)
    H = int(params.MAX_ADC_VALUES)
    if normals is None:
        normals = np.zeros((P, 1 + 3 * H), F32)
    reset = F32(params.RESET_NOISE_CHARGE)
    unc = F32(params.UNCORRELATED_NOISE_CHARGE)
    q = (np.asarray(wfs, F32) * F32(params.t_sampling)).astype(F32)
    qc = np.cumsum(q, axis=-1, dtype=F32) if cumsum is None else np.asarray(cumsum, F32)
    base = (normals[:, 0] * reset).astype(F32)
    qs = (base[:, None] + qc).astype(F32)
    interval = fee_interval(params)
    rows = np.arange(P)
    adcs, ticks = [], []
    for h in range(H):
        cross = (qs[:, 1:] >= thr) & (qs[:, :-1] <= thr)
        has = cross.any(axis=1)
        idx_t = np.where(has, cross.argmax(axis=1), T - 2)
        ic = idx_t.astype(F32)
        end = idx_t + 1 + interval
        end = np.where(end >= T, T - 1, end)
        qv = qs[rows, end]
        qvn = qc[rows, end]
        extra = (normals[:, 1 + 3 * h] * unc).astype(F32)
        adc = np.where(qvn != 0, qv + extra, qvn).astype(F32)
        cond = (adc < thr) | (idx_t == T - 2)
        adc = np.where(cond, F32(0), adc).astype(F32)
        ic = np.where(cond, F32(T - 2), ic).astype(F32)
        q_pass = (normals[:, 2 + 3 * h] * reset).astype(F32)
        q_fail = (normals[:, 3 + 3 * h] * unc).astype(F32)
        base = np.where(cond, q_fail, q_pass).astype(F32)
        end2 = idx_t + 1 + interval + 1
        end2 = np.where(end2 >= T, T - 1, end2)
        r = qc[rows, end2]
        qc = (qc - r[:, None]).astype(F32)
        qc = np.where(qc < 0, F32(0), qc).astype(F32)
        qs = (base[:, None] + qc).astype(F32)
        adcs.append(adc)
        ticks.append(ic)
    return np.stack(adcs, 1), np.stack(ticks, 1)


def digitize(params, integral):
    """fee_jax.py:55-71 (continuous ADC, no rounding)."""
    x = ((np.asarray(integral, F32) * F32(params.GAIN)) + F32(params.V_PEDESTAL)) - F32(params.V_CM)
    return np.minimum((np.maximum(x, F32(0)) * F32(params.ADC_COUNTS)) / F32(params.V_REF - params.V_CM),
                      F32(params.ADC_COUNTS)).astype(F32)


def adc2charge(dw, params):
    """losses_jax.py:380-383 (ke-)."""
    return (((((np.asarray(dw, F32) / F32(params.ADC_COUNTS)) * F32(params.V_REF - params.V_CM))
              + F32(params.V_CM)) - F32(params.V_PEDESTAL)) / F32(params.GAIN) * F32(1e-3)).astype(F32)


def parse_output(params, adcs, pixel_x, pixel_y, pixel_z, ticks, hit_prob, event, unique_pixels):
    """sim_jax.py:619-647: row-major compaction of accepted hits."""
    mask = (hit_prob > F32(params.hit_prob_threshold)) & (event[:, None] >= 0) & (unique_pixels[:, None] >= 0)
    fm = mask.ravel()
    H = mask.shape[1]
    return dict(adcs=adcs.ravel()[fm], pixel_x=np.repeat(pixel_x, H)[fm], pixel_y=np.repeat(pixel_y, H)[fm],
                pixel_z=pixel_z.ravel()[fm], ticks=ticks.ravel()[fm], hit_prob=hit_prob.ravel()[fm],
                event=np.repeat(event, H)[fm], pixels=np.repeat(unique_pixels, H)[fm], nb_valid=int(fm.sum()))


def simulate_stochastic(params, wfs, unique_pixels, normals=None):
    """sim_jax.py:738-769 (noise draws supplied as ``normals``)."""
    integral, ticks = get_adc_values(params, wfs, normals)
    hit_prob = np.where(ticks < wfs.shape[1] - 3, F32(1), F32(0)).astype(F32)
    adcs = digitize(params, integral)
    px, py, plane, event = id2pixel(params, unique_pixels)
    coords = get_pixel_coordinates(params, px, py, plane)
    pz = get_hit_z(params, ticks.ravel(), np.repeat(plane, ticks.shape[1])).reshape(ticks.shape)
    out = parse_output(params, adcs, coords[:, 0], coords[:, 1], pz, ticks, hit_prob, event, unique_pixels)
    out.update(grid_adcs=adcs, grid_ticks=ticks, grid_integral=integral)
    return out


# ---------------------------------------------------------------- output side

HIT_RECORD_FIELDS = ("adc_clean", "adc", "Q", "pixels", "ticks", "eventID", "pix_x", "pix_y", "pix_z")


def adc2charge_xla(dw, params):
    """adc2charge (losses_jax.py:380-383) in the form XLA compiled it to for
    the reference's committed outputs (output/jax_ref/output_*_1.npz): folded
    constants and one fused multiply-add, fma(dw / ADC_COUNTS, V_REF - V_CM,
    V_CM - V_PEDESTAL) * (1e-3 / GAIN); reproduces their charges bit for bit
    (tests/test_oracle_golden.py).  The fma is evaluated exactly in float64
    (a float32 product fits in 48 bits) and rounded once to float32."""
    a = np.asarray(dw, F32) * (F32(1) / F32(params.ADC_COUNTS))
    c = F32(params.V_REF - params.V_CM)
    d = F32(params.V_CM) - F32(params.V_PEDESTAL)
    f = (a.astype(np.float64) * np.float64(c) + np.float64(d)).astype(F32)
    return (f * (F32(1e-3) / F32(params.GAIN))).astype(F32)


def hit_records(params, adcs, pixel_x, pixel_y, pixel_z, ticks, hit_prob, event, hit_pixels, adc_lowest=None):
    """optimize/simulate.py:129-133: the kept hit rows of one batch.

    adc_lowest = digitize(DISCRIMINATION_THRESHOLD); a hit is kept when
    adc - adc_lowest != 0 and its event is not -1.  Returns a dict of the
    kept columns (input order) with the cleaned ADC and the charge in ke-
    (adc2charge_xla, the form the committed outputs pin).
    """
    adcs = np.asarray(adcs, F32).reshape(-1)
    event = np.asarray(event).reshape(-1)
    lowest = F32(digitize(params, F32(params.DISCRIMINATION_THRESHOLD))) if adc_lowest is None else F32(adc_lowest)
    clean = (adcs - lowest).astype(F32)
    mask = (clean != 0) & (event != -1)
    return {
        "adc_clean": clean[mask], "adc": adcs[mask], "Q": adc2charge_xla(adcs[mask], params),
        "pix_x": np.asarray(pixel_x, F32).reshape(-1)[mask], "pix_y": np.asarray(pixel_y, F32).reshape(-1)[mask],
        "pix_z": np.asarray(pixel_z, F32).reshape(-1)[mask], "ticks": np.asarray(ticks, F32).reshape(-1)[mask],
        "hit_prob": np.asarray(hit_prob, F32).reshape(-1)[mask], "event": event[mask],
        "pixels": np.asarray(hit_pixels).reshape(-1)[mask],
    }


def hit_records_by_event(records, local_to_global=None):
    """optimize/simulate.py:139-156: one group per local event id >= 0 of the
    kept rows (np.unique order), keyed by the global event id, with the
    reference's dataset names; eventID is int64 filled with the global id."""
    groups = {}
    ev = records["event"]
    for local in np.unique(ev).astype(int):
        if local < 0:
            continue
        g = (local_to_global or {}).get(local, local)
        m = ev == local
        grp = {name: records[key][m] for name, key in (("adc_clean", "adc_clean"), ("adc", "adc"), ("Q", "Q"),
                                                       ("pixels", "pixels"), ("ticks", "ticks"),
                                                       ("pix_x", "pix_x"), ("pix_y", "pix_y"), ("pix_z", "pix_z"))}
        grp["eventID"] = np.full(int(m.sum()), g, dtype=np.int64)
        groups[int(g)] = grp
    return groups


# ---------------------------------------------------------------- parametrised mode

def generate_electrons(params, tracks, fields, normals):
    """detsim_jax.py:376-400 with the normal draws supplied (S, 3)."""
    e = np.array(tracks, dtype=F32, copy=True)
    st = e[:, fields.index("tran_diff")]
    sl = e[:, fields.index("long_diff")]
    rnd = (np.asarray(normals, F32) * np.stack([st, st, sl], axis=1)).astype(F32)
    e[:, fields.index("x")] = e[:, fields.index("x")] + rnd[:, 0]
    e[:, fields.index("y")] = e[:, fields.index("y")] + rnd[:, 1]
    if not params.diffusion_in_current_sim:
        e[:, fields.index("z")] = e[:, fields.index("z")] + rnd[:, 2]
    return e


def get_pixels(params, electrons, fields):
    """detsim_jax.py:477-491 (number_pix_neighbors = 0)."""
    plane = electrons[:, fields.index("pixel_plane")].astype(int)
    b = np.asarray(params.tpc_borders, F32)[plane]
    px = floor_divide_f32(electrons[:, fields.index("x")] - b[:, 0, 0], params.pixel_pitch).astype(np.int64)
    py = floor_divide_f32(electrons[:, fields.index("y")] - b[:, 1, 0], params.pixel_pitch).astype(np.int64)
    n = params.number_pix_neighbors
    g = np.arange(-n, n + 1)
    X, Y = np.meshgrid(g, g, indexing="ij")
    sx, sy = X.ravel(), Y.ravel()
    ev = electrons[:, fields.index("eventID")].astype(int)
    return pixel2id(params, px[:, None] + sx[None], py[:, None] + sy[None], plane[:, None], ev[:, None])


def emg_pdf(x, mu, sigma, lambd):
    """detsim_jax.py:440-458."""
    coeff = lambd / F32(2)
    s2 = sigma ** 2
    exponent = coeff * (((F32(2) * mu) + (lambd * s2)) - (F32(2) * x))
    erfc_term = special.erfc((((mu + lambd * s2) - x) / (F32(np.sqrt(F32(2))) * sigma)).astype(F32)).astype(F32)
    return ((coeff * np.exp(exponent).astype(F32)) * erfc_term).astype(F32)


def integrated_expon_diff(x, loc, scale, diff, dt):
    """detsim_jax.py:461-474."""
    lambd = (F32(1) / scale).astype(F32)
    a = x - F32(dt / 2)
    b = x + F32(dt / 2)
    s2d = F32(np.sqrt(F32(2))) * diff
    up = F32(0.5) * erf32((b - loc) / s2d) - emg_pdf(b, loc, diff, lambd) / lambd
    lo = F32(0.5) * erf32((a - loc) / s2d) - emg_pdf(a, loc, diff, lambd) / lambd
    tv = (up - lo).astype(F32)
    tv = tv / (lo[..., 0] - up[..., -1])[..., None]
    return (tv / F32(dt)).astype(F32)


_B = (1.060, -0.909, -0.909, 5.856, 0.207, 0.207)
_C = (0.679, -1.083, -1.083, 8.772, -5.521, -5.521)
_D = (2.644, -9.174, -9.174, 13.483, 45.887, 45.887)
_T0 = (2.948, -2.705, -2.705, 4.825, 20.814, 20.814)


def _quad(p, x, y):
    return (((((F32(p[0]) + F32(p[1]) * x) + F32(p[2]) * y) + (F32(p[3]) * x) * y) + (F32(p[4]) * x) * x)
            + (F32(p[5]) * y) * y).astype(F32)


def current_model_diff(t, t0, x, y, dt, sigma):
    """detsim_jax.py:581-615."""
    a = np.minimum(_quad(_B, x, y), F32(1))
    b = _quad(_C, x, y)
    c = _quad(_D, x, y)
    st0 = (t0 + F32(_T0[0]) + F32(_T0[1]) * x + F32(_T0[2]) * y + (F32(_T0[3]) * x) * y
           + (F32(_T0[4]) * x) * x + (F32(_T0[5]) * y) * y).astype(F32)
    return (a * integrated_expon_diff(-t, -st0, b, sigma, dt)
            + (F32(1) - a) * integrated_expon_diff(-t, -st0, c, sigma, dt)).astype(F32)


def current_mc(params, electrons, pixels_coord, fields):
    """detsim_jax.py:618-639 (diffusion_in_current_sim=True branch)."""
    nt = int(5 / params.t_sampling) + 1
    ticks = jax_linspace_f32(0, 5, nt)[None, :]
    x_dist = np.abs(electrons[:, fields.index("x")] - pixels_coord[..., 0]).astype(F32)
    y_dist = np.abs(electrons[:, fields.index("y")] - pixels_coord[..., 1]).astype(F32)
    plane = electrons[:, fields.index("pixel_plane")].astype(int)
    z_anode = np.asarray(params.tpc_borders, F32)[plane, 2, 0]
    v = vdrift32(params)
    t0 = (np.abs(electrons[:, fields.index("z")] - z_anode) / v).astype(F32)
    t0_tick = ((t0 / F32(params.t_sampling)) + F32(0.5)).astype(np.int64)
    t0 = (t0 - t0_tick.astype(F32) * F32(params.t_sampling)).astype(F32)
    dt = 5.0 / (nt - 1)
    sig = (electrons[:, fields.index("long_diff")].reshape(-1, 1) / v).astype(F32)
    if not params.diffusion_in_current_sim:
        raise NotImplementedError("diffusion_in_current_sim=False is not restated")
    cur = current_model_diff(ticks, t0[:, None], x_dist[:, None], y_dist[:, None], dt, sig)
    return t0_tick, (cur * electrons[:, fields.index("n_electrons")].reshape(-1, 1)).astype(F32)


def simulate_parametrized(params, tracks, fields, normals, padded_size=None, history=None):
    """sim_jax.py:339-372 + :122-139 + :289-335 (mc_diff, n=0), noise off."""
    if params.number_pix_neighbors != 0:
        raise ValueError("parametrised mode requires number_pix_neighbors == 0")
    t = shift_tracks(params, tracks, fields)
    t = quench(params, t, fields)
    t = drift(params, t, fields)
    e = generate_electrons(params, t, fields, normals)
    pIDs = get_pixels(params, e, fields).ravel()
    u = np.unique(pIDs)
    if padded_size is None:
        padded_size = pad_size(u.shape[0], "unique_pixels", 0.05, history)
    unique = np.sort(np.pad(u, (0, padded_size - u.shape[0]), constant_values=-1)).astype(I32)
    xp, yp, pl, _ = id2pixel(params, pIDs)
    coords = get_pixel_coordinates(params, xp, yp, pl)
    t0_tick, signals = current_mc(params, e, coords, fields)
    renum = np.searchsorted(unique, pIDs, side="left")
    Nticks = n_ticks(params)
    start = t0_tick - signals.shape[1]
    tt = start[:, None] + np.arange(signals.shape[1])[None, :]
    tt = np.where((tt < 0) | (tt >= Nticks - 1), 0, tt + 1)
    idx = (renum[:, None] * Nticks + tt).ravel()
    wfs = np.bincount(idx, weights=signals.ravel().astype(np.float64),
                      minlength=unique.shape[0] * Nticks).astype(F32).reshape(-1, Nticks)
    integral, ticks = get_adc_values(params, wfs[:, 1:])
    adcs = digitize(params, integral)
    px, py, plane, event = id2pixel(params, unique)
    pc = get_pixel_coordinates(params, px, py, plane)
    pz = get_hit_z(params, ticks.ravel(), np.repeat(plane, ticks.shape[1])).reshape(ticks.shape)
    hit_prob = np.where(ticks < wfs.shape[1] - 3, F32(1), F32(0)).astype(F32)
    out = parse_output(params, adcs, pc[:, 0], pc[:, 1], pz, ticks, hit_prob, event, unique)
    out.update(wfs=wfs[:, 1:], unique_pixels=unique, grid_adcs=adcs, grid_ticks=ticks)
    return out


# ---------------------------------------------------------------- LUT bank

def load_lut_templates(response, params):
    """consts_jax.py:387-449: Gaussian-smoothed template bank, [0] = raw.

    norm.pdf(arange(-E, E+1), scale=sigma_k) normalised, convolved along
    time with mode='same'.  Evaluated in float64 and rounded to float32.
    """
    ext = int(params.long_diff_extent)
    sig = np.asarray(params.long_diff_template, np.float64)
    k = np.arange(-ext, ext + 1, dtype=np.float64)
    gaus = np.exp(-0.5 * (k[None, :] / sig[:, None]) ** 2) / (np.sqrt(2 * np.pi) * sig[:, None])
    gaus = gaus / gaus.sum(axis=1, keepdims=True)
    r = np.asarray(response, np.float64)
    flat = r.reshape(-1, r.shape[-1])
    out = np.empty((sig.shape[0],) + r.shape, np.float32)
    for i in range(sig.shape[0]):
        conv = np.apply_along_axis(lambda row: np.convolve(row, gaus[i], mode="same"), -1, flat)
        out[i] = conv.reshape(r.shape).astype(np.float32)
    out[0] = np.asarray(response, np.float32)
    return out


# ---------------------------------------------------------------- input side

def chop_tracks(tracks, fields, precision=0.001):
    """optimize/dataio.py:63-106: cut every track into steps of length
    ``precision`` (the last step takes the remainder), vectorised.

    Arithmetic follows NumPy 2 promotion of the reference's expressions:
    the length (left-to-right float32 sum of squares, float32 sqrt), the
    direction, the step count and the per-step dE are float32; the step
    positions ``start + k*precision*direction`` and the last step's dE and
    dx are float64 and rounded once when stored; midpoints are float32.
    """
    t = np.asarray(tracks, F32)
    col = {k: fields.index(k) for k in ("x_start", "y_start", "z_start", "x_end", "y_end", "z_end",
                                           "x", "y", "z", "dE", "dx")}
    start = t[:, [col["x_start"], col["y_start"], col["z_start"]]]
    end = t[:, [col["x_end"], col["y_end"], col["z_end"]]]
    seg = (end - start).astype(F32)
    sq = (seg * seg).astype(F32)
    length = ((sq[:, 0] + sq[:, 1]).astype(F32) + sq[:, 2]).astype(F32)
    length = np.sqrt(length).astype(F32)                                   # dataio.py:98
    lpe = (length + F32(1e-10)).astype(F32)
    direction = (seg / lpe[:, None]).astype(F32)                           # :100
    nsteps = np.maximum(np.ceil((length / F32(precision)).astype(F32)), F32(1))
    if not np.all(np.isfinite(nsteps)):
        raise ValueError("chop_tracks: non-finite track length")
    nsteps = nsteps.astype(np.int64)                                       # :101
    src = np.repeat(np.arange(t.shape[0]), nsteps)
    first = np.concatenate([[0], np.cumsum(nsteps)[:-1]]).astype(np.int64)
    k = np.arange(src.shape[0], dtype=np.int64) - first[src]
    last = k == nsteps[src] - 1
    out = t[src].copy()
    out[:, col["dE"]] = ((t[src, col["dE"]] * F32(precision)).astype(F32) / lpe[src]).astype(F32)   # :67
    p = float(precision)
    for a, (cs, ce) in enumerate((("x_start", "x_end"), ("y_start", "y_end"), ("z_start", "z_end"))):
        s0 = t[src, col[cs]].astype(np.float64)
        d = direction[src, a].astype(np.float64)
        out[:, col[cs]] = (s0 + (k * p) * d).astype(F32)                   # :70-72
        out[:, col[ce]] = np.where(last, t[src, col[ce]], (s0 + (p * (k + 1)) * d).astype(F32))   # :74-76, :80-82
    out[:, col["dx"]] = F32(p)                                             # :77
    n1 = (nsteps[src] - 1).astype(np.float64)
    de_last = (t[src, col["dE"]].astype(np.float64) * (1 - p * n1 / lpe[src].astype(np.float64))).astype(F32)
    dx_last = (length[src].astype(np.float64) - p * n1).astype(F32)
    out[:, col["dE"]] = np.where(last, de_last, out[:, col["dE"]])         # :83
    out[:, col["dx"]] = np.where(last, dx_last, out[:, col["dx"]])         # :84
    for cm, cs, ce in (("x", "x_start", "x_end"), ("y", "y_start", "y_end"), ("z", "z_start", "z_end")):
        out[:, col[cm]] = (F32(0.5) * (out[:, col[cs]] + out[:, col[ce]]).astype(F32)).astype(F32)   # :87-89
    return out


# ---------------------------------------------------------------- probabilistic front end

# jax.scipy.special.log_ndtr (the third-party arithmetic this path calls;
# JAX is not vendored with the reference and is unpinned): for float32 the
# published piecewise form switches to -ndtr(-x) above x = 5 and to the
# order-3 asymptotic series below x = -10.
LOG_NDTR_LOWER32, LOG_NDTR_UPPER32 = -10.0, 5.0


def ndtr32(x):
    """Standard normal CDF as jax.scipy.special.ndtr evaluates it (erf near
    zero, erfc in the tails), float32."""
    x = np.asarray(x, F32)
    hs2 = F32(0.5 * np.sqrt(2.0))
    w = (x * hs2).astype(F32)
    z = np.abs(w)
    y = np.where(z < hs2, F32(1) + special.erf(w).astype(F32),
                 np.where(w > 0, F32(2) - special.erfc(z).astype(F32), special.erfc(z).astype(F32)))
    return (F32(0.5) * y.astype(F32)).astype(F32)


def log_ndtr32(x):
    """log of the standard normal CDF, float32, piecewise as above."""
    x = np.asarray(x, F32)
    lo, hi = F32(LOG_NDTR_LOWER32), F32(LOG_NDTR_UPPER32)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        upper = -ndtr32(-x)
        mid = np.log(ndtr32(np.maximum(x, lo))).astype(F32)
        xl = np.minimum(x, lo)
        x2 = (xl * xl).astype(F32)
        log_scale = ((-(x2 / F32(2))) - np.log(-xl).astype(F32) - F32(0.5 * np.log(2 * np.pi))).astype(F32)
        # 1 + even - odd with the terms (2n-1)!! / x^(2n), n = 1, 2, 3
        x4 = (x2 * x2).astype(F32)
        x6 = (x4 * x2).astype(F32)
        odd = (F32(1) / x2 + F32(15) / x6).astype(F32)
        even = (F32(3) / x4).astype(F32)
        series = ((F32(1) + even) - odd).astype(F32)
        lower = (log_scale + np.log(series).astype(F32)).astype(F32)
    return np.where(x > hi, upper, np.where(x > lo, mid, lower)).astype(F32)


def softplus32(y):
    """jax.nn.softplus = logaddexp(y, 0) = max(y, 0) + log1p(exp(-|y|))."""
    y = np.asarray(y, F32)
    with np.errstate(over="ignore"):
        return (np.maximum(y, F32(0)) + np.log1p(np.exp(-np.abs(y))).astype(F32)).astype(F32)


def sigmoid32(x):
    x = np.asarray(x, F32)
    with np.errstate(over="ignore"):
        return (F32(1) / (F32(1) + np.exp(-x).astype(F32))).astype(F32)


def soft_max32(x, lo, sharpness):
    """fee_jax.py:13-20: lo + softplus((x - lo) * s) / s."""
    s = F32(sharpness)
    return (F32(lo) + softplus32(((np.asarray(x, F32) - F32(lo)) * s).astype(F32)) / s).astype(F32)


def soft_where32(cond, true_val, false_val, sharpness):
    """fee_jax.py:23-30: w * true + (1 - w) * false, w = sigmoid(cond * s)."""
    w = sigmoid32((np.asarray(cond, F32) * F32(sharpness)).astype(F32))
    return ((w * np.asarray(true_val, F32)).astype(F32) + ((F32(1) - w) * F32(false_val)).astype(F32)).astype(F32)


def log_diff_ndtr32(a, b, la=None, lb=None):
    """fee_jax.py:33-53: log(Phi(a) - Phi(b)) with the smooth clamps."""
    a = np.asarray(a, F32)
    b = np.asarray(b, F32)
    la = log_ndtr32(a) if la is None else la
    lb = log_ndtr32(b) if lb is None else lb
    safe = np.where(a > b, (lb - la).astype(F32), F32(-1))
    neg = (-np.expm1(safe)).astype(F32)
    neg_safe = soft_max32(neg, 1e-30, 1e10)
    with np.errstate(divide="ignore"):
        lt = np.log(neg_safe).astype(F32)
    lts = soft_max32(lt, -100.0, 10.0)
    lp = (la + lts).astype(F32)
    return soft_where32((a - b).astype(F32), lp, -1000.0, 1000.0)


def logsumexp32(x, axis):
    x = np.asarray(x, F32)
    m = np.max(x, axis=axis, keepdims=True)
    m = np.where(np.isfinite(m), m, F32(0)).astype(F32)
    s = np.sum(np.exp((x - m).astype(F32)).astype(F32), axis=axis, keepdims=True, dtype=F32)
    with np.errstate(divide="ignore"):
        return (np.log(s).astype(F32) + m).astype(F32).squeeze(axis)


def top_k_indices(x, k):
    """lax.top_k indices: largest first, equal values in index order."""
    return np.argsort(-np.asarray(x, np.float64), axis=-1, kind="stable")[..., :k]


def find_one_hit_step(q_sum, charges, log_probs, sigma, threshold, interval, n_values):
    """fee_jax.py:334-384 for P pixels at once: q_sum (P, T), charges and
    log_probs (P, K).  Returns (charges', log_probs'), the step outputs
    (log_total_hit_dist_tick (P, T-1), esperance_value (P, T-1)) and the
    top-K tick choices (P, K)."""
    P, T = q_sum.shape
    z = F32(1.0 / sigma)
    thr = F32(threshold)
    sh = np.clip(np.arange(T - 1) + interval + 1, 0, T - 1)
    Q = (q_sum[:, None, :] - charges[:, :, None]).astype(F32)                       # (P, K, T)
    qmax = np.maximum.accumulate(Q, axis=2)
    zm = ((qmax - thr) * z).astype(F32)
    lm = log_ndtr32(zm)
    log_guess = log_diff_ndtr32(zm[..., 1:], zm[..., :-1], lm[..., 1:], lm[..., :-1])
    zq = ((Q - thr) * z).astype(F32)
    lq = log_ndtr32(zq)
    lpe = log_diff_ndtr32(zq[..., sh], zq[..., :-1], lq[..., sh], lq[..., :-1])
    lpe = np.minimum(lpe, log_guess)
    lpe = soft_max32(lpe, -1000.0, 1.0)
    esp = ((q_sum[:, sh] + thr).astype(F32) - (F32(0.5) * (q_sum[:, 1:] + q_sum[:, :-1]).astype(F32))).astype(F32)
    lpe = soft_where32((esp - thr).astype(F32)[:, None, :], lpe, -1000.0, 10.0)
    lp = log_probs[:, :, None]
    hit = logsumexp32((lpe + lp).astype(F32), axis=1)
    dist = logsumexp32((log_guess + lp).astype(F32), axis=1)
    next_q = Q[:, :, np.clip(sh + 1, 0, T - 1)]
    maxfut = np.maximum.accumulate(Q[:, :, ::-1], axis=2)[:, :, ::-1]
    fe = np.clip(sh + interval + 1, 0, T - 1)
    lf = log_ndtr32((((maxfut[:, :, fe] - next_q).astype(F32) - thr) * z).astype(F32))
    sel = logsumexp32(((log_guess + lf).astype(F32) + lp).astype(F32), axis=1)
    top = top_k_indices(sel, n_values)                                              # (P, K)
    new_lp = np.take_along_axis(dist, top, axis=1)
    best = np.clip(sh[top] + 1, 0, T - 1)
    new_c = np.take_along_axis(q_sum, best, axis=1)
    return (new_c.astype(F32), new_lp.astype(F32)), (hit, esp), top


def get_adc_values_average_noise(params, wfs, stop_threshold=1e-9, return_choices=False):
    """fee_jax.py:386-461: beam search over MAX_ADC_VALUES hits with
    fee_paths_scaling paths, stopped for the whole batch once no pixel keeps
    a total path probability above stop_threshold.  Returns
    (log_prob (P, H, T-1), charge (P, H, T-1)); with return_choices also
    the top-K tick choices of every executed step (P, H, K) and the number
    of executed steps, the inputs of beam_search64."""
    wfs = np.asarray(wfs, F32)
    P, T = wfs.shape
    K = int(params.fee_paths_scaling)
    H = int(params.MAX_ADC_VALUES)
    interval = fee_interval(params)
    q_sum = np.cumsum((wfs * F32(params.t_sampling)).astype(F32), axis=1, dtype=F32)
    c = np.zeros((P, K), F32)
    lp = np.full((P, K), F32(-1000))
    lp[:, 0] = 0
    log_stop = np.log(F32(stop_threshold)).astype(F32)
    out_lp = np.full((P, H, T - 1), F32(-1000))
    out_q = np.zeros((P, H, T - 1), F32)
    active = True
    top = np.zeros((P, H, K), np.int64)
    n_exec = 0
    for h in range(H):
        if not active:
            break
        (c, lp), (hit, esp), top[:, h] = find_one_hit_step(q_sum, c, lp, params.RESET_NOISE_CHARGE,
                                                            params.DISCRIMINATION_THRESHOLD, interval, K)
        n_exec = h + 1
        out_lp[:, h] = hit
        out_q[:, h] = esp
        active = bool(np.any(logsumexp32(lp, axis=1) > log_stop))
    if return_choices:
        return out_lp, out_q, top, n_exec
    return out_lp, out_q


def get_average_hit_values(ticks_prob, adcs_distrib):
    """fee_jax.py:463-480: per (pixel, hit) the total probability, the
    expected tick and the expected ADC."""
    tp = np.asarray(ticks_prob, F32)
    lam = tp.sum(axis=2, dtype=F32)
    ticks = np.arange(tp.shape[2], dtype=F32)
    den = np.maximum(lam, F32(1e-10))
    e_tick = ((ticks[None, None, :] * tp).sum(axis=2, dtype=F32) / den).astype(F32)
    e_adc = ((np.asarray(adcs_distrib, F32) * tp).sum(axis=2, dtype=F32) / den).astype(F32)
    return e_tick, e_adc, lam


def simulate_probabilistic(params, wfs, unique_pixels):
    """sim_jax.py:771-813: (adcs_distrib, pixel_x, pixel_y, ticks_prob, event)
    with ticks_prob the log-probabilities of the beam search."""
    log_prob, charge = get_adc_values_average_noise(params, wfs)
    adcs = digitize(params, charge)
    px, py, plane, event = id2pixel(params, np.asarray(unique_pixels))
    pc = get_pixel_coordinates(params, px, py, plane)
    return adcs, pc[:, 0], pc[:, 1], log_prob, event


# ---------------------------------------------------------------- probabilistic front end, float64, frozen

def _ndtr64(x):
    hs2 = 0.5 * np.sqrt(2.0)
    w = x * hs2
    z = np.abs(w)
    return 0.5 * np.where(z < hs2, 1 + special.erf(w), np.where(w > 0, 2 - special.erfc(z), special.erfc(z)))


def _log_ndtr64(x):
    """The float32 piecewise form (segments at -10 and 5) in float64."""
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        upper = -_ndtr64(-x)
        mid = np.log(_ndtr64(np.maximum(x, -10.0)))
        xl = np.minimum(x, -10.0)
        x2 = xl * xl
        series = (1 + 3 / x2 ** 2) - (1 / x2 + 15 / x2 ** 3)
        lower = -(x2 / 2) - np.log(-xl) - 0.5 * np.log(2 * np.pi) + np.log(series)
    return np.where(x > 5, upper, np.where(x > -10, mid, lower))


def _softplus64(y):
    with np.errstate(over="ignore"):
        return np.maximum(y, 0) + np.log1p(np.exp(-np.abs(y)))


def _sigmoid64(x):
    with np.errstate(over="ignore"):
        return 1 / (1 + np.exp(-x))


def _ldn64(a, b):
    la, lb = _log_ndtr64(a), _log_ndtr64(b)
    safe = np.where(a > b, lb - la, -1.0)
    neg = -np.expm1(safe)
    ns = 1e-30 + _softplus64((neg - 1e-30) * 1e10) / 1e10
    with np.errstate(divide="ignore"):
        lt = np.log(ns)
    lts = -100 + _softplus64((lt + 100) * 10) / 10
    w = _sigmoid64((a - b) * 1000)
    return w * (la + lts) + (1 - w) * -1000.0


def _lse64(x, axis):
    m = np.max(x, axis=axis, keepdims=True)
    return (np.log(np.sum(np.exp(x - m), axis=axis, keepdims=True)) + m).squeeze(axis)


def beam_search64(params, wfs, top, n_exec):
    """get_adc_values_average_noise_vmap (fee_jax.py:334-461) in float64 with
    the top-K tick choices ``top`` (P, H, K) and the number of executed steps
    held: (log_prob, charge), each (P, H, T-1).  Its derivatives are what
    jax.grad takes through the beam search (test infrastructure for the
    adjoint)."""
    w = np.asarray(wfs, np.float64)
    P, T = w.shape
    K = int(params.fee_paths_scaling)
    H = int(params.MAX_ADC_VALUES)
    iv = fee_interval(params)
    z = 1.0 / float(params.RESET_NOISE_CHARGE)
    thr = float(params.DISCRIMINATION_THRESHOLD)
    q = np.cumsum(w * float(params.t_sampling), axis=1)
    cm = np.maximum.accumulate(q, axis=1)
    t = np.arange(T - 1)
    sh = np.minimum(t + iv + 1, T - 1)
    esp = (q[:, sh] + thr) - 0.5 * (q[:, 1:] + q[:, :-1])
    sw = _sigmoid64((esp - thr) * 10)
    c = np.zeros((P, K))
    lp = np.full((P, K), -1000.0)
    lp[:, 0] = 0.0
    out_lp = np.full((P, H, T - 1), -1000.0)
    out_q = np.zeros((P, H, T - 1))
    rows = np.arange(P)[:, None]
    for h in range(n_exec):
        zm = ((cm[:, None, :] - c[:, :, None]) - thr) * z
        lg = _ldn64(zm[..., 1:], zm[..., :-1])
        zq = ((q[:, None, :] - c[:, :, None]) - thr) * z
        le = _ldn64(zq[..., sh], zq[..., :-1])
        le = np.minimum(le, lg)
        le = -1000.0 + _softplus64(le + 1000.0)
        le = sw[:, None, :] * le + (1 - sw[:, None, :]) * -1000.0
        out_lp[:, h] = _lse64(le + lp[:, :, None], axis=1)
        out_q[:, h] = esp
        dist = _lse64(lg + lp[:, :, None], axis=1)
        tk = np.asarray(top[:, h], np.int64)
        lp = dist[rows, tk]
        c = q[rows, np.minimum(sh[tk] + 1, T - 1)]
    return out_lp, out_q
