"""Simulation parameters, detector geometry and derived constants.

Mirrors the parameter object of the reference (``Params_template`` and
``build_params_class`` in src/larndsim/consts_jax.py:25-190) with the same
field names and defaults, ``get_vdrift`` (consts_jax.py:192-217) and
``load_detector_properties`` (consts_jax.py:220-385).

Numerics convention.  In the reference, non-differentiable parameters are
static Python floats, so every expression built only from parameters is
evaluated in float64 on the host and rounded to float32 when it meets a
float32 array.  The helpers here (``DerivedScalars``) reproduce exactly that:
they evaluate such expressions in float64 and round once.
"""

from __future__ import annotations

import dataclasses
import math
from collections import defaultdict
from enum import Enum
from typing import Any

import numpy as np

from . import yaml_lite


class RecombinationMode(Enum):
    """Recombination models (consts_jax.py:20-23)."""

    BOX = 1
    BIRKS = 2
    ELLIPSOID = 3


def jax_linspace_f32(start: float, stop: float, num: int) -> np.ndarray:
    """float32 ``linspace`` with the arithmetic of ``jax.numpy.linspace``.

    JAX (x64 disabled) evaluates ``start * (1 - i/div) + stop * (i/div)`` in
    float32 and appends ``stop`` exactly; numpy's float64 formula can differ
    in the last bit, which matters for searchsorted on the template grid
    (sim_jax.py:163) and for the transverse bin edges (sim_jax.py:401).
    """
    s = np.float32(start)
    e = np.float32(stop)
    if num == 1:
        return np.array([s], dtype=np.float32)
    div = num - 1
    step = (np.arange(div, dtype=np.float32) / np.float32(div)).astype(np.float32)
    out = (s * (np.float32(1) - step) + e * step).astype(np.float32)
    return np.concatenate([out, np.array([e], dtype=np.float32)])


# Geometry of the 2x(2x4)-tile module of pixel layout 2.4.16 (v4) with the
# module0 detector properties: TPC borders (cm, float64 exactly as the
# reference's loader computes them before its float32 conversion).
_MODULE0_TPC_BORDERS_F64 = np.array(
    [[[-31.038, 31.038], [-62.076, 62.076], [30.58975, 0.15874999999999773]],
     [[-31.038, 31.038], [-62.076, 62.076], [-30.58975, -0.15874999999999773]]],
    dtype=np.float64)


@dataclasses.dataclass(frozen=True, eq=False)
class Params:
    """Simulation parameters (field names and meaning as consts_jax.py:80-160).

    Default values are the reference's defaults (consts_jax.py:244-298)
    overridden by the module0 detector properties and the 2.4.16_v4 pixel
    layout, i.e. what ``load_detector_properties(Params, module0.yaml,
    multi_tile_layout-2.4.16_v4.yaml)`` returns.
    """

    eField: float = 0.50
    Ab: float = 0.8
    kb: float = 0.0486
    lifetime: float = 2.2e3
    vdrift: float = 0.1587
    vdrift_static: float = 0.159645
    long_diff: float = 4.0e-6
    tran_diff: float = 8.8e-6
    tpc_borders: Any = dataclasses.field(
        default_factory=lambda: _MODULE0_TPC_BORDERS_F64.astype(np.float32))
    recombination_mode: RecombinationMode = RecombinationMode.BIRKS
    lArDensity: float = 1.38
    alpha: float = 0.93
    beta: float = 0.212
    R_param: float = 1.25
    MeVToElectrons: float = 4.237e4
    pixel_pitch: float = 4.434 * 0.1
    n_pixels_x: int = 140
    n_pixels_y: int = 280
    max_radius: int = 0
    max_active_pixels: int = 0
    drift_length: float = 304.31 * 0.1
    t_sampling: float = 0.1
    time_interval: Any = (0, 200.0)
    time_padding: float = 190
    min_step_size: float = 0.001
    time_max: float = 0
    time_window: float = 189.1
    e_charge: float = 1.602e-19
    temperature: float = 87.17
    response_bin_size: float = 0.04434
    number_pix_neighbors: int = 1
    electron_sampling_resolution: float = 0.001
    signal_length: int = 150
    response_full_drift_t: float = 190.61638
    MAX_ADC_VALUES: int = 10
    DISCRIMINATION_THRESHOLD: float = 5000
    ADC_HOLD_DELAY: int = 15
    CLOCK_CYCLE: float = 0.1
    GAIN: float = 4e-3
    V_CM: float = 284.27734375
    V_REF: float = 1282.71484375
    V_PEDESTAL: float = 580
    ADC_COUNTS: int = 2 ** 8
    RESET_NOISE_CHARGE: float = 900
    UNCORRELATED_NOISE_CHARGE: float = 500
    ELECTRON_MOBILITY_PARAMS: tuple = (551.6, 7158.3, 4440.43, 4.29, 43.63, 0.2053)
    shift_x: float = 0.0
    shift_y: float = 0.0
    shift_z: float = 0.0
    size_margin: float = 2e-2
    diffusion_in_current_sim: bool = True
    mc_diff: bool = False
    nb_sampling_bins_per_pixel: int = 10
    long_diff_template: Any = dataclasses.field(
        default_factory=lambda: jax_linspace_f32(0.001, 10, 100))
    long_diff_extent: int = 20
    roi_threshold: float = 0.01
    roi_split_length: int = 400
    fee_paths_scaling: int = 20
    nb_tran_diff_bins: int = 5
    hit_prob_threshold: float = 1e-5
    tran_diff_bin_edges: Any = None

    # differentiable field names of this class (set by build_params_class)
    _grad_fields = ()

    def replace(self, **updates) -> "Params":
        """Functional update, like ``flax.struct.dataclass.replace``."""
        return dataclasses.replace(self, **updates)

    def __getitem__(self, key):
        return getattr(self, key)


def build_params_class(params_with_grad):
    """Return a ``Params`` subclass whose listed fields are differentiable.

    Mirrors consts_jax.py:162-190.  Differentiability here is bookkeeping
    used by the autograd wrappers; the class otherwise behaves like
    ``Params``.
    """
    unknown = [p for p in params_with_grad if p not in {f.name for f in dataclasses.fields(Params)}]
    if unknown:
        raise ValueError(f"unknown parameter(s) {unknown}")
    cls = type("Params", (Params,), {"_grad_fields": tuple(params_with_grad)})
    return dataclasses.dataclass(frozen=True, eq=False)(cls)


def get_vdrift(params) -> float:
    """Electron drift velocity in cm/us (consts_jax.py:192-217).

    Evaluated in float64 exactly as the reference does for static params;
    callers round to float32 where the reference meets float32 arrays.
    """
    a0, a1, a2, a3, a4, a5 = params.ELECTRON_MOBILITY_PARAMS
    e = params.eField
    num = a0 + a1 * e + a2 * pow(e, 1.5) + a3 * pow(e, 2.5)
    denom = 1 + (a1 / a0) * e + a4 * pow(e, 2) + a5 * pow(e, 3)
    temp_corr = pow(params.temperature / 89, -1.5)
    mu = num / denom * temp_corr / 1000
    return mu * e


def get_vdrift_derivative(params) -> float:
    """d(vdrift)/d(eField) in float64, the analytic derivative of get_vdrift."""
    a0, a1, a2, a3, a4, a5 = params.ELECTRON_MOBILITY_PARAMS
    e = params.eField
    num = a0 + a1 * e + a2 * e ** 1.5 + a3 * e ** 2.5
    dnum = a1 + 1.5 * a2 * e ** 0.5 + 2.5 * a3 * e ** 1.5
    den = 1 + (a1 / a0) * e + a4 * e ** 2 + a5 * e ** 3
    dden = (a1 / a0) + 2 * a4 * e + 3 * a5 * e ** 2
    tc = pow(params.temperature / 89, -1.5) / 1000
    mu = num / den * tc
    dmu = (dnum * den - num * dden) / den ** 2 * tc
    return dmu * e + mu


def n_ticks(params) -> int:
    """Waveform length including the leading garbage tick (sim_jax.py:147)."""
    return int(params.time_interval[1] / params.t_sampling) + 1


def fee_interval(params) -> int:
    """Integration window of the self-trigger, in ticks (fee_jax.py:216)."""
    return round((3 * params.CLOCK_CYCLE + params.ADC_HOLD_DELAY * params.CLOCK_CYCLE) / params.t_sampling)


def tran_diff_bin_edges(params) -> np.ndarray:
    """Sub-pixel bin edges of the 5x5 transverse-diffusion grid (sim_jax.py:398-403)."""
    nb = params.nb_tran_diff_bins
    sym = (nb - 1) // 2
    width = params.pixel_pitch / params.nb_sampling_bins_per_pixel
    return jax_linspace_f32(-sym * width, (sym + 1) * width, nb + 1)


def load_detector_properties(params_cls, detprop_file, pixel_file):
    """Build parameters from a detector-properties and a pixel-layout YAML.

    Same inputs, validation and derived geometry as consts_jax.py:220-385
    (unknown keys raise ``ValueError``; TPC borders from tile positions,
    tile extent, drift length and cathode direction; pixel counts per axis).
    """
    defaults = {f.name: (f.default if f.default is not dataclasses.MISSING else f.default_factory())
                for f in dataclasses.fields(Params)}
    d = dict(defaults)
    d["tpc_centers"] = np.array([[0, 0, 0], [0, 0, 0]])
    d["long_diff_template"] = jax_linspace_f32(0.001, 10, 100)
    d["time_interval"] = [0, 200]
    allowed = set(defaults) | {"tpc_centers"}
    detprop = yaml_lite.load(detprop_file) or {}
    for key, value in detprop.items():
        if key not in allowed:
            raise ValueError(f"Key '{key}' in detector properties file is not recognized.")
        d[key] = np.array(value) if isinstance(value, list) else value
    if isinstance(d.get("ELECTRON_MOBILITY_PARAMS"), np.ndarray):
        d["ELECTRON_MOBILITY_PARAMS"] = tuple(float(v) for v in d["ELECTRON_MOBILITY_PARAMS"])
    tpc_centers = np.array(d["tpc_centers"])
    tpc_centers[:, [2, 0]] = tpc_centers[:, [0, 2]]

    layout = yaml_lite.load(pixel_file)
    mm2cm = 0.1
    pitch = layout["pixel_pitch"] * mm2cm
    pos = np.array(list(layout["chip_channel_to_position"].values()))
    xs = pos[:, 0] * pitch
    ys = pos[:, 1] * pitch
    tile_borders = np.zeros((2, 2))
    tile_borders[0] = [-(max(xs) + pitch) / 2, (max(xs) + pitch) / 2]
    tile_borders[1] = [-(max(ys) + pitch) / 2, (max(ys) + pitch) / 2]
    tile_indeces = layout["tile_indeces"]
    tpc_ids = np.unique(np.array(list(tile_indeces.values()))[:, 0], axis=0)
    anodes = defaultdict(list)
    cathode_dir = {}
    for tpc_id in tpc_ids:
        dirs = []
        for tile in tile_indeces:
            if tile_indeces[tile][0] == tpc_id:
                anodes[tpc_id].append(layout["tile_positions"][tile])
                dirs.append(layout["tile_orientations"][tile][0])
        if len(set(dirs)) != 1:
            raise ValueError("Tiles in same anode plane have different drift directions.")
        if dirs[0] not in (1, -1):
            raise ValueError("Cathode direction should be either 1 or -1.")
        cathode_dir[tpc_id] = dirs[0]
    if "drift_length" in layout:
        drift_length = layout["drift_length"] * mm2cm
    else:
        tp = np.array(list(layout["tile_positions"].values())) * mm2cm
        drift_length = 0.5 * (max(tp[:, 0]) - min(tp[:, 0])) * mm2cm
    borders = np.zeros((len(anodes), 3, 2))
    for itpc, tpc_id in enumerate(anodes):
        tiles = np.vstack(anodes[tpc_id]) * mm2cm
        borders[itpc] = (
            (min(tiles[:, 2]) + tile_borders[0][0] + tpc_centers[itpc][0],
             max(tiles[:, 2]) + tile_borders[0][1] + tpc_centers[itpc][0]),
            (min(tiles[:, 1]) + tile_borders[1][0] + tpc_centers[itpc][1],
             max(tiles[:, 1]) + tile_borders[1][1] + tpc_centers[itpc][1]),
            (min(tiles[:, 0]) + tpc_centers[itpc][2],
             max(tiles[:, 0]) + drift_length * cathode_dir[tpc_id] + tpc_centers[itpc][2]))
    d["pixel_pitch"] = pitch
    d["drift_length"] = drift_length
    d["n_pixels_x"] = len(np.unique(xs)) * 2
    d["n_pixels_y"] = len(np.unique(ys)) * 4
    d["tpc_borders"] = borders.astype(np.float32)
    names = {f.name for f in dataclasses.fields(params_cls)}
    return params_cls(**{k: v for k, v in d.items() if k in names})


def default_params(params_cls=Params, **updates):
    """module0 detector + 2.4.16_v4 layout parameters, with optional updates."""
    return params_cls().replace(**updates) if updates else params_cls()
