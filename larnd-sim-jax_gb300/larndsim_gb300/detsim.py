"""Host-side event-id checks of the simulate driver (reference:
src/larndsim/detsim_jax.py:26-154, called by optimize/simulate.py:111-113).

Pixel and sub-pixel-bin ids pack the event id above the TPC plane and the
pixel (or bin) coordinates.  These checks run on the host before a batch is
simulated and raise the reference's exceptions: ValueError for event ids
below -1 or a local namespace with gaps, OverflowError when the packed ids
would not fit in int64.  The simulation kernels themselves pack ids in
int32, as the reference does in practice (JAX without x64), and report
event ids outside the batch through their status word.
"""

from __future__ import annotations

import numpy as np

_INT64_MAX = int(np.iinfo(np.int64).max)


def _n_planes(params) -> int:
    return int(np.asarray(params.tpc_borders).shape[0])


def _pixel_id_stride(params) -> int:
    return int(params.n_pixels_x) * int(params.n_pixels_y) * _n_planes(params)


def _bin_id_stride(params) -> int:
    nb = int(params.nb_sampling_bins_per_pixel)
    return int(params.n_pixels_x) * nb * int(params.n_pixels_y) * nb * _n_planes(params)


def max_safe_event_id_for_pixel_packing(params) -> int:
    """Largest event id whose packed pixel ids fit in int64."""
    stride = _pixel_id_stride(params)
    return (_INT64_MAX - (stride - 1)) // stride


def max_safe_event_id_for_bin_packing(params) -> int:
    """Largest event id whose packed bin ids fit in int64."""
    stride = _bin_id_stride(params)
    return (_INT64_MAX - (stride - 1)) // stride


def max_possible_pixel_id(params, max_event_id) -> int:
    """Packed id of the last pixel of the last plane of event max_event_id."""
    nx, ny, nt = int(params.n_pixels_x), int(params.n_pixels_y), _n_planes(params)
    return ((int(max_event_id) * nt + (nt - 1)) * ny + (ny - 1)) * nx + (nx - 1)


def max_possible_bin_id(params, max_event_id) -> int:
    """Packed id of the last sub-pixel bin of the last plane of event max_event_id."""
    nb = int(params.nb_sampling_bins_per_pixel)
    nbx, nby, nt = int(params.n_pixels_x) * nb, int(params.n_pixels_y) * nb, _n_planes(params)
    return ((int(max_event_id) * nt + (nt - 1)) * nby + (nby - 1)) * nbx + (nbx - 1)


def _below_minus_one(ids, what, context):
    bad = ids < -1
    if np.any(bad):
        raise ValueError(f"{context} found {what} below -1: {np.unique(ids[bad])[:16].tolist()}")


def validate_event_ids_for_packing(params, event_ids, kind="pixel", context=""):
    """Event ids >= -1 whose packed pixel (or bin) ids fit in int64
    (detsim_jax.py:54-85)."""
    ids = np.asarray(event_ids, dtype=np.int64)
    if ids.size == 0:
        return
    _below_minus_one(ids, "eventID values", context)
    valid = ids >= 0
    if not np.any(valid):
        return
    top = int(np.max(ids[valid]))
    if kind == "pixel":
        safe, largest = max_safe_event_id_for_pixel_packing(params), max_possible_pixel_id(params, top)
    elif kind == "bin":
        safe, largest = max_safe_event_id_for_bin_packing(params), max_possible_bin_id(params, top)
    else:
        raise ValueError(f"Unknown packing kind '{kind}'")
    if top > safe:
        raise OverflowError(f"{context} eventID {top} exceeds the int64-safe limit {safe} for {kind} packing")
    if largest > _INT64_MAX:
        raise OverflowError(f"{context} maximum packed {kind} id {largest} exceeds int64 max {_INT64_MAX}")


def validate_packed_ids_for_decoding(params, packed_ids, kind="pixel", context=""):
    """Packed ids >= -1 whose decoded event ids are int64-safe
    (detsim_jax.py:87-115)."""
    ids = np.asarray(packed_ids, dtype=np.int64)
    if ids.size == 0:
        return
    _below_minus_one(ids, "packed ids", context)
    valid = ids >= 0
    if not np.any(valid):
        return
    if kind == "pixel":
        stride, safe = _pixel_id_stride(params), max_safe_event_id_for_pixel_packing(params)
    elif kind == "bin":
        stride, safe = _bin_id_stride(params), max_safe_event_id_for_bin_packing(params)
    else:
        raise ValueError(f"Unknown decoding kind '{kind}'")
    top = int(np.max(ids[valid] // stride))
    if top > safe:
        raise OverflowError(f"{context} decoded eventID {top} exceeds the int64-safe limit {safe} for {kind} packing")


def validate_local_event_ids(event_ids, context=""):
    """Event ids that form a local namespace: -1 (padding) and exactly
    0..N-1 with no gaps (detsim_jax.py:117-152)."""
    ids = np.asarray(event_ids, dtype=np.int64)
    if ids.size == 0:
        return
    bad = ids < -1
    if np.any(bad):
        raise ValueError(f"{context} found eventID values below -1 (non-local namespace): "
                         f"{np.unique(ids[bad])[:16].tolist()}")
    valid = ids >= 0
    if not np.any(valid):
        return
    present = np.unique(ids[valid])
    expected = np.arange(len(present), dtype=np.int64)
    if not np.array_equal(present, expected):
        raise ValueError(f"{context} eventID values do not form contiguous local namespace [0, {len(present) - 1}]. "
                         f"Found unique IDs: {present.tolist()}, expected: {expected.tolist()}")
