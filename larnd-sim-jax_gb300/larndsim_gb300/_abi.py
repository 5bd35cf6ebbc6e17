"""ctypes binding of ``liblsim.so`` (declarations in include/lsim.h).

``load()`` opens the in-tree library once and checks the ABI version and
structure sizes; it raises when the library is missing -- the simulate
path has no CPU fallback.  ``make_params`` converts a ``Params`` object into
the ``LsimParams`` block, evaluating parameter-only expressions in float64
and rounding once, the way the reference's static parameters behave.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

from . import consts

LIB_PATH = Path(__file__).resolve().parent / "liblsim.so"
ABI_VERSION = 2
MAX_TPC, MAX_TEMPLATES, MAX_HITS, NPARAM = 2, 128, 16, 8
GRAD_PARAMS = ("Ab", "kb", "eField", "lifetime", "vdrift", "long_diff", "tran_diff", "lArDensity")

LSIM_OK, LSIM_ERR_INVALID, LSIM_ERR_CAPACITY, LSIM_ERR_CUDA, LSIM_ERR_UNSUPPORTED = 0, 1, 2, 3, 4


class LsimFieldMap(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "n_fields", "eventID", "x", "y", "z", "x_start", "y_start", "z_start", "x_end", "y_end", "z_end",
        "dx", "dE", "dEdx")]


class LsimHitColumns(C.Structure):
    """Device pointers of the 8 hit columns (NULL = column not used)."""
    _fields_ = [(n, C.c_void_p) for n in ("adc", "pixel_x", "pixel_y", "pixel_z", "ticks", "hit_prob", "event",
                                         "pixels")]


NORM_SCHEMES = {"sigmoid": 0, "exp_log": 1, "divide": 2}
FIT_STATE = 32


class LsimFitOptions(C.Structure):
    """Options of lsim_fit_init / lsim_fit_step (arrays in GRAD_PARAMS order)."""
    _fields_ = [("scheme", C.c_int32), ("fit_mask", C.c_int32), ("clip_from_range", C.c_int32),
                ("norm_scale", C.c_float), ("max_clip_norm", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float),
                ("eps", C.c_float)] + [(n, C.c_float * NPARAM) for n in ("lr", "lo", "hi", "nom", "norm", "down", "up")]


class LsimParams(C.Structure):
    _fields_ = [
        ("recombination_mode", C.c_int32),
        ("Ab", C.c_float), ("kb", C.c_float), ("alpha", C.c_float), ("beta", C.c_float), ("r_inv2", C.c_float),
        ("erho", C.c_float), ("mev_to_electrons", C.c_float),
        ("vdrift", C.c_float), ("lifetime", C.c_float), ("long_diff", C.c_float), ("tran_diff", C.c_float),
        ("size_margin", C.c_float),
        ("shift_x", C.c_float), ("shift_y", C.c_float), ("shift_z", C.c_float),
        ("n_tpc", C.c_int32),
        ("tpc_borders", C.c_float * (MAX_TPC * 6)),
        ("pixel_pitch", C.c_float), ("half_pitch", C.c_float), ("bin_width", C.c_float),
        ("n_pixels_x", C.c_int32), ("n_pixels_y", C.c_int32), ("nb_bins_per_pixel", C.c_int32),
        ("n_tran_bins", C.c_int32), ("n_neighbors", C.c_int32),
        ("tran_edges", C.c_float * 8),
        ("t_sampling", C.c_float),
        ("n_ticks", C.c_int32), ("signal_length", C.c_int32),
        ("lut_nx", C.c_int32), ("lut_ny", C.c_int32), ("lut_nt", C.c_int32), ("n_templates", C.c_int32),
        ("long_diff_template", C.c_float * MAX_TEMPLATES),
        ("threshold", C.c_float), ("gain", C.c_float), ("v_pedestal", C.c_float), ("v_cm", C.c_float),
        ("vref_minus_cm", C.c_float), ("adc_counts", C.c_float),
        ("reset_noise", C.c_float), ("uncorr_noise", C.c_float), ("hit_prob_threshold", C.c_float),
        ("max_adc_values", C.c_int32), ("fee_interval", C.c_int32),
        ("diffusion_in_current_sim", C.c_int32), ("param_nticks", C.c_int32),
        ("param_dt", C.c_float), ("param_ticks", C.c_float * 64),
        ("eField", C.c_float), ("lArDensity", C.c_float), ("dvdrift_deField", C.c_float),
        ("reserved", C.c_int32 * 8),
        ("mobility", C.c_double * 6), ("mobility_temp", C.c_double),
    ]


class LsimCounts(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("n_valid", "n_em1", "any_m1", "status", "max_slot", "bad_row", "work",
                                         "n_main_rec", "n_main_seg", "n_big_slots", "n_heavy")] + [("reserved", C.c_int32 * 5)]


_vp, _i64, _i32, _sz = C.c_void_p, C.c_int64, C.c_int32, C.c_size_t
_PP, _PF = C.POINTER(LsimParams), C.POINTER(LsimFieldMap)

_SIGNATURES = {
    "lsim_abi_version": (C.c_int, []),
    "lsim_last_error": (C.c_char_p, []),
    "lsim_struct_sizes": (None, [C.POINTER(_sz)] * 3),
    "lsim_set_kernel_events": (None, [_vp, _vp]),
    "lsim_set_tuning": (None, [_vp]),
    "lsim_lut_build_templates": (C.c_int, [_vp, _i32, _i32, _i32, _vp, _i32, _i32, _vp, _vp]),
    "lsim_lut_tables_bytes": (_sz, [_PP]),
    "lsim_lut_prepare": (C.c_int, [_PP, _vp, _vp, _sz, _vp]),
    "lsim_workspace_bytes": (_sz, [_PP, _i64, _i32]),
    "lsim_lut_stage1": (C.c_int, [_PP, _PF, _vp, _i64, _i32, _vp, _sz, _vp, _vp]),
    "lsim_lut_stage1_theta": (C.c_int, [_PP, _PF, _vp, _i64, _i32, _vp, _vp, _sz, _vp, _vp]),
    "lsim_adam_step": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_float, C.c_float, C.c_float, _vp]),
    "lsim_fit_init": (C.c_int, [_vp, C.POINTER(LsimFitOptions), _vp, _vp]),
    "lsim_fit_step": (C.c_int, [_vp, _vp, C.POINTER(LsimFitOptions), _vp, _vp]),
    "lsim_lut_stage2": (C.c_int, [_PP, _vp, _vp, _i64, _i32, _i64, _i32, _i32, _vp, _vp, _vp]),
    "lsim_valid_pixels": (C.c_int, [_PP, _vp, _i64, _i32, _i32, _vp, _vp]),
    "lsim_lut_adc": (C.c_int, [_PP, _vp, _vp, _i64, _i32, _i32, _vp, _vp, _vp, _vp]),
    "lsim_lut_grad": (C.c_int, [_PP, _vp, _vp, _i64, _i32, _i32, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp]),
    "lsim_lut_grad_stored": (C.c_int, [_PP, _vp, _vp, _i64, _i32, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp]),
    "lsim_lut_wfs_vjp": (C.c_int, [_PP, _vp, _vp, _i64, _i32, _vp, _i64, _i32, _vp, _vp]),
    "lsim_fee": (C.c_int, [_PP, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _vp]),
    "lsim_fee_vjp_workspace_bytes": (_sz, [_i64]),
    "lsim_fee_vjp": (C.c_int, [_PP, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _sz, _vp]),
    "lsim_hits_workspace_bytes": (_sz, [_i64, _i32]),
    "lsim_hits": (C.c_int, [_PP, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz,
                            _vp]),
    "lsim_hits_noalloc_max_slots": (_i64, []),
    "lsim_hits_noalloc": (C.c_int, [_PP, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                    _vp]),
    "lsim_pixel_coords": (C.c_int, [_PP, _vp, _i64, _vp, _vp, _vp, _vp, _vp]),
    "lsim_fee_prob_workspace_bytes": (_sz, [_PP]),
    "lsim_fee_prob": (C.c_int, [_PP, _vp, _i64, _i32, _i32, C.c_float, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "lsim_fee_prob_vjp_workspace_bytes": (_sz, [_PP, _i64, _i32]),
    "lsim_fee_prob_vjp": (C.c_int, [_PP, _vp, _i64, _i32, _i32, C.c_float, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz,
                                    _vp]),
    "lsim_mse_adc_workspace_bytes": (_sz, [_i64, _i64]),
    "lsim_mse_adc": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _i64, C.c_float, C.c_float,
                               _vp, _vp, _vp, _vp, _sz, _vp]),
    "lsim_nll_workspace_bytes": (_sz, [_i64, _i64]),
    "lsim_nll_loss": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _i64, C.c_float,
                                _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "lsim_chamfer_workspace_bytes": (_sz, [_i64, _i64]),
    "lsim_chamfer_3d": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp,
                                  _sz, _vp]),
    "lsim_prob_llhd_workspace_bytes": (_sz, [_i64]),
    "lsim_prob_llhd": (C.c_int, [_PP, _vp, _i64, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _i64, C.c_double, C.c_double,
                                 _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "lsim_llhd_workspace_bytes": (_sz, [_i64]),
    "lsim_llhd_loss": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _i64, _i32, C.c_double, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                 _sz, _vp]),
    "lsim_occurrence_workspace_bytes": (_sz, [_i64]),
    "lsim_occurrence_indices": (C.c_int, [_vp, _i64, _vp, _vp, _sz, _vp]),
    "lsim_hit_records_workspace_bytes": (_sz, [_i64]),
    "lsim_hit_records": (C.c_int, [_PP, C.c_float, C.POINTER(LsimHitColumns), _i64, C.POINTER(LsimHitColumns), _vp,
                                   _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "lsim_gather_tracks": (C.c_int, [_vp, _i64, _i32, _vp, _i64, _i32, _vp, _vp, _vp, _vp]),
    "lsim_pad_tracks": (C.c_int, [_vp, _i64, _i64, _i32, _i32, _vp, _i64, _vp]),
    "lsim_chop_workspace_bytes": (_sz, [_i64]),
    "lsim_chop_tracks": (C.c_int, [_PF, _vp, _i64, C.c_double, _vp, _i64, _vp, _vp, _sz, _vp]),
    "lsim_param_stage1": (C.c_int, [_PP, _PF, _vp, _i64, _i32, _vp, _vp, _sz, _vp, _vp]),
    "lsim_param_wfs_vjp": (C.c_int, [_PP, _vp, _i64, _i32, _vp, _i64, _i32, _vp, _vp]),
    "lsim_param_stage2": (C.c_int, [_PP, _vp, _i64, _i32, _i64, _i32, _i32, _vp, _vp, _vp]),
}

EXPORTED = tuple(_SIGNATURES)

_lock = threading.Lock()
_lib = None


class LsimError(RuntimeError):
    """A non-zero status returned by liblsim."""

    def __init__(self, code, msg):
        super().__init__(f"liblsim error {code}: {msg}")
        self.code = code


def load(path: Path | None = None):
    """Open liblsim.so once; raise if it is missing or does not match."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise RuntimeError(f"{p} is missing: build it with `python -m larndsim_gb300.build` "
                               "(the simulate path has no CPU fallback)")
        lib = C.CDLL(str(p))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.lsim_abi_version() != ABI_VERSION:
            raise RuntimeError(f"liblsim ABI {lib.lsim_abi_version()} != {ABI_VERSION}")
        sp, sf, sc = _sz(), _sz(), _sz()
        lib.lsim_struct_sizes(C.byref(sp), C.byref(sf), C.byref(sc))
        if (sp.value, sf.value, sc.value) != (C.sizeof(LsimParams), C.sizeof(LsimFieldMap), C.sizeof(LsimCounts)):
            raise RuntimeError("liblsim structure layout does not match the binding")
        if path is None:
            _lib = lib
        return lib


def set_kernel_events(start=None, stop=None):
    """Record torch.cuda.Event ``start``/``stop`` around the pixel
    accumulation kernel of every following LUT call on this thread
    (``None`` turns it off).  The events are recorded once here first so
    that their CUDA handles exist."""
    lib = load()
    if start is None or stop is None:
        lib.lsim_set_kernel_events(None, None)
        return
    start.record()
    stop.record()
    lib.lsim_set_kernel_events(C.c_void_p(start.cuda_event), C.c_void_p(stop.cuda_event))


def check(lib, rc: int):
    if rc != LSIM_OK:
        raise LsimError(rc, lib.lsim_last_error().decode(errors="replace"))


_FIELD_NAMES = ("eventID", "x", "y", "z", "x_start", "y_start", "z_start", "x_end", "y_end", "z_end", "dx", "dE",
                "dEdx")


def field_map(fields, n_fields=None) -> LsimFieldMap:
    """Resolve the reference's column names to indices (dataio.py:130-141)."""
    fields = tuple(fields)
    fm = LsimFieldMap()
    fm.n_fields = len(fields) if n_fields is None else n_fields
    for name in _FIELD_NAMES:
        if name not in fields:
            raise ValueError(f"track array has no '{name}' column")
        setattr(fm, name, fields.index(name))
    return fm


def _f32(x) -> float:
    return float(np.float32(x))


def make_params(params, lut_shape=None) -> LsimParams:
    """Fill an LsimParams block from a Params object.

    ``lut_shape`` = (n_templates, nx, ny, nt) of the template bank (LUT
    mode); omitted in parametrised mode.
    """
    lp = LsimParams()
    mode = getattr(params.recombination_mode, "value", params.recombination_mode)
    if mode not in (1, 2, 3):
        raise ValueError(f"Invalid recombination mode {params.recombination_mode}: "
                         "must be RecombinationMode.BOX, RecombinationMode.BIRKS, or RecombinationMode.ELLIPSOID")
    lp.recombination_mode = int(mode)
    lp.Ab, lp.kb = _f32(params.Ab), _f32(params.kb)
    lp.alpha, lp.beta = _f32(params.alpha), _f32(params.beta)
    lp.r_inv2 = _f32(1.0 / params.R_param ** 2)
    lp.erho = _f32(params.eField * params.lArDensity)
    lp.mev_to_electrons = _f32(params.MeVToElectrons)
    lp.vdrift = _f32(consts.get_vdrift(params))
    lp.lifetime, lp.long_diff, lp.tran_diff = _f32(params.lifetime), _f32(params.long_diff), _f32(params.tran_diff)
    lp.size_margin = _f32(params.size_margin)
    lp.shift_x, lp.shift_y, lp.shift_z = _f32(params.shift_x), _f32(params.shift_y), _f32(params.shift_z)
    b = np.asarray(params.tpc_borders, np.float32)
    if b.shape[0] > MAX_TPC or b.shape[1:] != (3, 2):
        raise ValueError(f"tpc_borders of shape {b.shape} not supported")
    lp.n_tpc = b.shape[0]
    for i, v in enumerate(b.ravel()):
        lp.tpc_borders[i] = float(v)
    nb = int(params.nb_sampling_bins_per_pixel)
    lp.pixel_pitch = _f32(params.pixel_pitch)
    lp.half_pitch = _f32(params.pixel_pitch / 2)
    lp.bin_width = _f32(params.pixel_pitch / nb)
    lp.n_pixels_x, lp.n_pixels_y = int(params.n_pixels_x), int(params.n_pixels_y)
    lp.nb_bins_per_pixel = nb
    lp.n_tran_bins = int(params.nb_tran_diff_bins)
    lp.n_neighbors = int(params.number_pix_neighbors)
    edges = consts.tran_diff_bin_edges(params)
    for i, v in enumerate(edges[:8]):
        lp.tran_edges[i] = float(v)
    lp.t_sampling = _f32(params.t_sampling)
    lp.n_ticks = consts.n_ticks(params)
    lp.signal_length = int(params.signal_length)
    tmpl = np.asarray(params.long_diff_template, np.float32)
    if tmpl.shape[0] > MAX_TEMPLATES:
        raise ValueError(f"{tmpl.shape[0]} long-diffusion templates > {MAX_TEMPLATES}")
    lp.n_templates = tmpl.shape[0]
    for i, v in enumerate(tmpl):
        lp.long_diff_template[i] = float(v)
    if lut_shape is not None:
        nt_, nx, ny, nt = (int(v) for v in lut_shape)
        if nt_ != tmpl.shape[0]:
            raise ValueError(f"template bank has {nt_} templates but long_diff_template has {tmpl.shape[0]}")
        need = nb * int(params.number_pix_neighbors) + nb // 2
        if nx < need or ny < need:
            raise ValueError(f"a {nx}x{ny} LUT covers fewer than the {need} sub-pixel positions that "
                             f"number_pix_neighbors={params.number_pix_neighbors} reads")
        lp.lut_nx, lp.lut_ny, lp.lut_nt = nx, ny, nt
    lp.threshold = _f32(params.DISCRIMINATION_THRESHOLD)
    lp.gain = _f32(params.GAIN)
    lp.v_pedestal = _f32(params.V_PEDESTAL)
    lp.v_cm = _f32(params.V_CM)
    lp.vref_minus_cm = _f32(params.V_REF - params.V_CM)
    lp.adc_counts = _f32(params.ADC_COUNTS)
    lp.reset_noise = _f32(params.RESET_NOISE_CHARGE)
    lp.uncorr_noise = _f32(params.UNCORRELATED_NOISE_CHARGE)
    lp.hit_prob_threshold = _f32(params.hit_prob_threshold)
    lp.max_adc_values = int(params.MAX_ADC_VALUES)
    if not 1 <= lp.max_adc_values <= MAX_HITS:
        raise ValueError(f"MAX_ADC_VALUES {lp.max_adc_values} not in [1, {MAX_HITS}]")
    lp.fee_interval = int(consts.fee_interval(params))
    lp.diffusion_in_current_sim = 1 if params.diffusion_in_current_sim else 0
    npt = int(5 / params.t_sampling) + 1
    if npt > 64:
        raise ValueError("parametrised current window longer than 64 ticks")
    lp.param_nticks = npt
    lp.param_dt = _f32(5.0 / (npt - 1))
    for i, v in enumerate(consts.jax_linspace_f32(0, 5, npt)):
        lp.param_ticks[i] = float(v)
    lp.eField, lp.lArDensity = _f32(params.eField), _f32(params.lArDensity)
    lp.dvdrift_deField = _f32(consts.get_vdrift_derivative(params))
    for i, v in enumerate(params.ELECTRON_MOBILITY_PARAMS):
        lp.mobility[i] = float(v)
    lp.mobility_temp = pow(params.temperature / 89, -1.5) / 1000
    return lp
