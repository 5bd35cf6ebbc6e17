"""Shared helpers of the GPU parity tests (CUDA path vs the CPU oracle)."""

from __future__ import annotations

import numpy as np

WFS_RTOL = 1e-5     # per valid row, relative to the row's max |w| (the spec waveform tolerance)
ADC_RTOL = 1e-5     # ADC values of hits whose crossing tick agrees


def small_params(n_neighbors=1, n_templates=10, **kw):
    from larndsim_gb300 import consts
    base = dict(number_pix_neighbors=n_neighbors, RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0,
                long_diff_template=consts.jax_linspace_f32(0.001, 10, n_templates))
    base.update(kw)
    return consts.Params(**base)


def compare_wfs(wfs_gpu, unique_gpu, wfs_ref, unique_ref):
    """Max relative error over valid rows (pixel id >= 0); rows must align."""
    u = np.asarray(unique_gpu)
    assert np.array_equal(u, np.asarray(unique_ref)), "unique_pixels differ"
    v = u >= 0
    w = np.asarray(wfs_gpu)[v]
    r = np.asarray(wfs_ref)[v]
    scale = np.abs(r).max(axis=1, keepdims=True)
    scale = np.where(scale > 0, scale, 1.0)
    return float((np.abs(w - r) / scale).max()) if w.size else 0.0


def compare_fee(adc_gpu, ticks_gpu, adc_ref, ticks_ref, params=None):
    """(fraction of hit slots whose tick differs, max rel ADC error where ticks agree).

    With ``params`` the inputs are raw integrated charges and are digitised
    first: the raw integral after a reset is a difference of two large
    cumulative sums, so its float32 rounding depends on the summation order
    in both implementations; the contract is on the ADC."""
    tg, tr = np.asarray(ticks_gpu), np.asarray(ticks_ref)
    ag, ar = np.asarray(adc_gpu), np.asarray(adc_ref)
    if params is not None:
        from oracle import reference_np as R
        ag, ar = R.digitize(params, ag), R.digitize(params, ar)
    # a row whose tick differs at hit h differs afterwards as well: compare
    # rows up to their first disagreement
    same_row = np.cumprod(tg == tr, axis=1).astype(bool)
    frac = 1.0 - same_row.mean()
    rel = np.abs(ag - ar) / np.maximum(np.abs(ar), 1e-6)
    err = float(rel[same_row].max()) if same_row.any() else 0.0
    return float(frac), err
