"""Seeded synthetic inputs in the reference's track-array format.

The reference reads edep-sim segments from HDF5 (optimize/dataio.py:108-141)
into an ``(N, F)`` float32 array plus a tuple of column names.  These
generators produce arrays with the same columns (``SEGMENT_FIELDS``, the
order of the reference's ``segments`` dtype after its x<->z swap) for the
workloads this package is measured on:

* ``muon_event``: straight tracks through a box, cut into fixed-length
  segments, dE from a Moyal distribution (mean 0.84 MeV per 0.4 cm).
* ``shower_event``: short segments (exponential length, mean 0.1 cm)
  clustered around seeded sub-tracks.
* ``batched_events``: many events with log-uniform segment counts, a mix of
  both kinds, with local event ids 0..E-1 as the reference requires
  (detsim_jax.py:117-152).
* ``synthetic_response``: a seeded smooth unipolar pixel-response LUT of
  shape (45, 45, 1950) on 0.1 us ticks.
"""

from __future__ import annotations

import numpy as np
from scipy import stats

SEGMENT_FIELDS = (
    "eventID", "trackID", "x_start", "y_start", "z_start", "x_end", "y_end",
    "z_end", "x", "y", "z", "t", "t_start", "t_end", "t0", "t0_start",
    "t0_end", "dx", "dE", "dEdx", "n_electrons", "n_photons", "long_diff",
    "tran_diff", "pixel_plane", "pdgId",
)

# Drift volumes of the module0 geometry (cm): x, y extents and the z range
# of each TPC (anode side first).
_TPC_X = (-31.038, 31.038)
_TPC_Y = (-62.076, 62.076)
_TPC_Z = ((0.15875, 30.58975), (-30.58975, -0.15875))

MOYAL_SCALE = 0.05          # MeV, width of the Moyal dE distribution
MIP_DE_PER_04CM = 0.84      # MeV, mean dE of a 0.4 cm segment


def _moyal_de(rng, n, length, ref_len=0.4):
    """dE per segment: Moyal(mean 0.84 MeV per 0.4 cm) scaled by length."""
    loc = MIP_DE_PER_04CM - MOYAL_SCALE * (np.euler_gamma + np.log(2.0))
    de = stats.moyal.rvs(loc=loc, scale=MOYAL_SCALE, size=n, random_state=rng)
    de = np.clip(de, 0.05, 20.0)
    return de * (length / ref_len)


def _rows(starts, ends, de, event_id, track_ids, pdg):
    n = starts.shape[0]
    out = np.zeros((n, len(SEGMENT_FIELDS)), dtype=np.float32)
    col = {f: i for i, f in enumerate(SEGMENT_FIELDS)}
    dx = np.linalg.norm(ends - starts, axis=1)
    out[:, col["eventID"]] = event_id
    out[:, col["trackID"]] = track_ids
    for k, ax in enumerate("xyz"):
        out[:, col[f"{ax}_start"]] = starts[:, k]
        out[:, col[f"{ax}_end"]] = ends[:, k]
        out[:, col[ax]] = 0.5 * (starts[:, k] + ends[:, k])
    out[:, col["dx"]] = dx
    out[:, col["dE"]] = de
    out[:, col["dEdx"]] = np.where(dx > 0, de / np.maximum(dx, 1e-12), 0.0)
    out[:, col["pdgId"]] = pdg
    return out


def _box_chord(rng, lo, hi):
    """Chord of a box through a uniform interior point, isotropic direction."""
    p = rng.uniform(lo, hi)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    with np.errstate(divide="ignore", invalid="ignore"):
        t1 = np.where(d != 0, (lo - p) / d, -np.inf)
        t2 = np.where(d != 0, (hi - p) / d, np.inf)
    tmin = np.max(np.minimum(t1, t2))
    tmax = np.min(np.maximum(t1, t2))
    return p + tmin * d, p + tmax * d


def _segment_line(a, b, seg_len):
    length = float(np.linalg.norm(b - a))
    n = max(int(np.ceil(length / seg_len)), 1)
    d = (b - a) / max(length, 1e-12)
    s = np.minimum(np.arange(n) * seg_len, length)
    e = np.minimum((np.arange(n) + 1) * seg_len, length)
    return a + s[:, None] * d, a + e[:, None] * d


def muon_event(seed=0, n_tracks=12, box_lo=(0.5, 0.5, 0.3), box_hi=(30.5, 30.5, 30.3),
               seg_len=0.4, event_id=0):
    """Straight muon tracks through a 30x30x30 cm box in TPC 0 (one 70x70 tile)."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(box_lo, float), np.asarray(box_hi, float)
    parts = []
    for itrk in range(n_tracks):
        a, b = _box_chord(rng, lo, hi)
        s, e = _segment_line(a, b, seg_len)
        de = _moyal_de(rng, s.shape[0], np.linalg.norm(e - s, axis=1), seg_len)
        parts.append(_rows(s, e, de, event_id, itrk, 13))
    return np.concatenate(parts, axis=0), SEGMENT_FIELDS


def _random_box(rng, size):
    """A box of the given size fully inside one randomly chosen TPC."""
    itpc = rng.integers(0, 2)
    z0, z1 = sorted(_TPC_Z[itpc])
    size = np.minimum(np.asarray(size, float), [_TPC_X[1] - _TPC_X[0] - 1, _TPC_Y[1] - _TPC_Y[0] - 1, z1 - z0 - 0.4])
    lo = np.array([rng.uniform(_TPC_X[0] + 0.5, _TPC_X[1] - 0.5 - size[0]),
                   rng.uniform(_TPC_Y[0] + 0.5, _TPC_Y[1] - 0.5 - size[1]),
                   rng.uniform(z0 + 0.2, z1 - 0.2 - size[2])])
    return lo, lo + size


def shower_segments(rng, n_segments, lo, hi, n_subtracks=8, mean_len=0.1, spread=1.5):
    """Short segments (exponential length) clustered around seeded sub-tracks."""
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    centre = 0.5 * (lo + hi)
    axes = rng.normal(size=(n_subtracks, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    origins = centre + rng.normal(scale=0.15 * (hi - lo), size=(n_subtracks, 3))
    which = rng.integers(0, n_subtracks, size=n_segments)
    u = rng.exponential(scale=0.25 * np.min(hi - lo), size=n_segments)
    sig = spread * (0.2 + u / np.min(hi - lo))
    pos = origins[which] + axes[which] * u[:, None] + rng.normal(size=(n_segments, 3)) * sig[:, None]
    pos = np.clip(pos, lo, hi)
    length = np.clip(rng.exponential(scale=mean_len, size=n_segments), 0.005, 1.0)
    d = rng.normal(size=(n_segments, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    starts = pos - 0.5 * length[:, None] * d
    ends = pos + 0.5 * length[:, None] * d
    de = _moyal_de(rng, n_segments, length)
    return starts, ends, de, which


def shower_event(seed=0, n_segments=5000, event_id=0, n_subtracks=8, box=(30.0, 30.0, 28.0)):
    """Shower-like event: short clustered segments inside one TPC."""
    rng = np.random.default_rng(seed)
    lo, hi = _random_box(rng, box)
    s, e, de, which = shower_segments(rng, n_segments, lo, hi, n_subtracks)
    return _rows(s, e, de, event_id, which, 11), SEGMENT_FIELDS


def mixed_event(rng, n_segments, event_id, seg_len=0.4):
    """Tracks plus a shower, ``n_segments`` rows, inside one TPC box."""
    lo, hi = _random_box(rng, (30.0, 30.0, 28.0))
    frac_tracks = rng.uniform(0.2, 0.8)
    n_trk_target = int(frac_tracks * n_segments)
    parts, itrk, ntrk = [], 0, 0
    while ntrk < n_trk_target:
        a, b = _box_chord(rng, lo, hi)
        s, e = _segment_line(a, b, seg_len)
        s, e = s[: n_trk_target - ntrk], e[: n_trk_target - ntrk]
        de = _moyal_de(rng, s.shape[0], np.linalg.norm(e - s, axis=1), seg_len)
        parts.append(_rows(s, e, de, event_id, itrk, 13))
        ntrk += s.shape[0]
        itrk += 1
    n_sh = n_segments - ntrk
    if n_sh > 0:
        s, e, de, which = shower_segments(rng, n_sh, lo, hi)
        parts.append(_rows(s, e, de, event_id, itrk + which, 11))
    return np.concatenate(parts, axis=0)


def batched_events(seed=0, n_events=64, min_segments=1000, max_segments=50000):
    """Events with log-uniform segment counts, local event ids 0..E-1."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(min_segments), np.log(max_segments), size=n_events)).astype(int)
    parts = [mixed_event(rng, int(c), ev) for ev, c in enumerate(counts)]
    return np.concatenate(parts, axis=0), SEGMENT_FIELDS


def large_shower_event(seed=0, n_segments=500_000, n_subtracks=40):
    """One shower-like event of many segments clustered around sub-tracks."""
    rng = np.random.default_rng(seed)
    lo, hi = _random_box(rng, (60.0, 120.0, 29.0))
    s, e, de, which = shower_segments(rng, n_segments, lo, hi, n_subtracks, spread=3.0)
    return _rows(s, e, de, 0, which, 11), SEGMENT_FIELDS


def pad_tracks(tracks, fields, target_len):
    """Pad with invalid rows the way the reference's loader does (dataio.py:340-373)."""
    n = tracks.shape[0]
    if target_len <= n:
        return tracks
    out = np.zeros((target_len, tracks.shape[1]), dtype=np.float32)
    out[:n] = tracks
    col = {f: i for i, f in enumerate(fields)}
    out[n:, col["eventID"]] = -1
    for f in ("trackID", "pixel_plane"):
        if f in col:
            out[n:, col[f]] = -1
    return out


def synthetic_response(seed=0, nx=45, ny=45, nt=1950, t_sampling=0.1):
    """Seeded smooth unipolar current LUT ``response[cx, cy, t]`` (float32).

    ``(cx, cy)`` is the drift position in tenths of a pixel pitch from the
    pixel centre.  The pad collects charge for positions on the pad (cx, cy
    below 5), with a weaker unipolar induction beyond.  The pulse rises
    exponentially while the charge approaches the anode and ends near tick
    ``nt - 20``; the rise time grows with distance, so far positions put a
    sizeable part of their signal before the last 150 ticks.  Each row
    integrates (sum x t_sampling) to its collection amplitude.
    """
    rng = np.random.default_rng(seed)
    cx = np.arange(nx)[:, None].astype(np.float64)
    cy = np.arange(ny)[None, :].astype(np.float64)
    dmax = np.maximum(cx, cy)
    dist = np.sqrt(cx ** 2 + cy ** 2)
    amp = np.where(dmax <= 3, 1.0, np.where(dmax <= 4, 0.5, 0.03 * np.exp(-(dmax - 5.0) / 6.0)))
    amp = amp * (1.0 + 0.05 * rng.uniform(-1, 1, size=(nx, ny)))
    tau_rise = 12.0 + 0.45 * dist + rng.uniform(0, 2, size=(nx, ny))
    t_peak = (nt - 20) - 0.08 * dist
    t = np.arange(nt, dtype=np.float64)[None, None, :]
    dt = t - t_peak[..., None]
    shape = np.where(dt <= 0, np.exp(np.minimum(dt, 0) / tau_rise[..., None]), np.exp(-np.maximum(dt, 0) / 2.0))
    # seeded smooth modulation, a few low-frequency sinusoids
    phase = rng.uniform(0, 2 * np.pi, size=(3,))
    mod = 1.0 + 0.03 * sum(np.sin(2 * np.pi * (k + 1) * t / nt + phase[k]) for k in range(3))
    shape = shape * mod
    # light Gaussian smoothing (sigma 1.5 ticks) to keep the pulse smooth
    kern = np.exp(-0.5 * (np.arange(-6, 7) / 1.5) ** 2)
    kern /= kern.sum()
    sm = np.apply_along_axis(lambda r: np.convolve(r, kern, mode="same"), -1, shape.reshape(-1, nt)).reshape(nx, ny, nt)
    norm = sm.sum(axis=-1, keepdims=True) * t_sampling
    resp = amp[..., None] * sm / norm
    return resp.astype(np.float32)
