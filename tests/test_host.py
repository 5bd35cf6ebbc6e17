"""Host-side logic: parameters, YAML loading, the parameter block, and the
C-ABI library's exported symbols (no GPU needed)."""

import ctypes
import os
import re
from pathlib import Path

import numpy as np
import pytest

from larndsim_gb300 import _abi, consts, yaml_lite

ROOT = Path(__file__).resolve().parent.parent
# the larnd-sim-jax source tree, when one is at hand (its own YAML files)
REF = Path(os.environ.get("LARNDSIM_JAX_SRC", "/nonexistent"))

DETPROP = """
tpc_centers: # cm
  - [0, 0, 0]
  - [0, 0, 0]
time_interval: [0, 200.] # us
drift_length: 30.27225 # cm
eField: 0.50 #kV/cm
lifetime: 2.2e+3 # us
vdrift: 0.1587 # cm / us
MeVToElectrons: 4.237e+04
Ab: 0.8
kb: 0.0486
long_diff: 4.0e-6  # cm * cm / us
tran_diff: 8.8e-6  # cm * cm / us
DISCRIMINATION_THRESHOLD: 5000
V_CM: 284.27734375
V_REF: 1282.71484375
"""


def _layout_text():
    """A 2-TPC, 16-tile layout of 70x70 pixels in the reference's format."""
    lines = ["chip_channel_to_position:"]
    k = 0
    for x in range(70):
        for y in range(70):
            lines += [f"  {1000 + k}:", f"  - {x}", f"  - {y}"]
            k += 1
    lines += ["drift_length: 304.31", "pixel_pitch: 4.434", "tile_indeces:"]
    for t in range(1, 17):
        lines += [f"  {t}:", f"  - {1 if t <= 8 else 2}", f"  - {(t - 1) % 8 + 1}"]
    lines.append("tile_orientations:")
    for t in range(1, 17):
        lines += [f"  {t}:", f"  - {-1 if t <= 8 else 1}", "  - 1", "  - 1"]
    ys = [465.57, 465.57, 155.19, 155.19, -155.19, -155.19, -465.57, -465.57]
    zs = [-155.19, 155.19] * 4
    lines.append("tile_positions:")
    for t in range(1, 17):
        x = 305.8975 if t <= 8 else -305.8975
        lines += [f"  {t}:", f"  - {x}", f"  - {ys[(t - 1) % 8]}", f"  - {zs[(t - 1) % 8]}"]
    return "\n".join(lines) + "\n"


def test_yaml_lite_subset():
    d = yaml_lite.loads(DETPROP)
    assert d["tpc_centers"] == [[0, 0, 0], [0, 0, 0]]
    assert d["time_interval"] == [0, 200.0]
    assert d["lifetime"] == 2200.0 and d["DISCRIMINATION_THRESHOLD"] == 5000
    lay = yaml_lite.loads(_layout_text())
    assert lay["chip_channel_to_position"][1000] == [0, 0]
    assert lay["tile_positions"][16] == [-305.8975, -465.57, 155.19]


def test_load_detector_properties_matches_defaults(tmp_path):
    (tmp_path / "det.yaml").write_text(DETPROP)
    (tmp_path / "lay.yaml").write_text(_layout_text())
    p = consts.load_detector_properties(consts.Params, tmp_path / "det.yaml", tmp_path / "lay.yaml")
    d = consts.Params()
    np.testing.assert_array_equal(p.tpc_borders, d.tpc_borders)
    assert p.n_pixels_x == 140 and p.n_pixels_y == 280
    assert p.pixel_pitch == d.pixel_pitch and p.drift_length == d.drift_length
    assert p.DISCRIMINATION_THRESHOLD == 5000 and p.V_CM == 284.27734375


def test_unknown_detector_key_raises(tmp_path):
    (tmp_path / "det.yaml").write_text(DETPROP + "bogus_key: 1\n")
    (tmp_path / "lay.yaml").write_text(_layout_text())
    with pytest.raises(ValueError):
        consts.load_detector_properties(consts.Params, tmp_path / "det.yaml", tmp_path / "lay.yaml")


@pytest.mark.skipif(not REF.exists(), reason="set LARNDSIM_JAX_SRC to the larnd-sim-jax source tree")
def test_reference_yaml_files_give_the_embedded_geometry():
    p = consts.load_detector_properties(
        consts.Params, REF / "src/larndsim/detector_properties/module0.yaml",
        REF / "src/larndsim/pixel_layouts/multi_tile_layout-2.4.16_v4.yaml")
    d = consts.Params()
    np.testing.assert_array_equal(p.tpc_borders, d.tpc_borders)
    assert (p.n_pixels_x, p.n_pixels_y, p.pixel_pitch, p.drift_length) == (140, 280, d.pixel_pitch, d.drift_length)


def test_build_params_class_and_replace():
    P = consts.build_params_class(["Ab", "eField"])
    p = P()
    assert P._grad_fields == ("Ab", "eField")
    q = p.replace(Ab=0.9)
    assert q.Ab == 0.9 and p.Ab == 0.8 and isinstance(q, P)
    with pytest.raises(ValueError):
        consts.build_params_class(["nope"])


def test_vdrift_derivative_matches_finite_difference():
    p = consts.Params()
    h = 1e-6
    fd = (consts.get_vdrift(p.replace(eField=0.5 + h)) - consts.get_vdrift(p.replace(eField=0.5 - h))) / (2 * h)
    assert abs(consts.get_vdrift_derivative(p) - fd) < 1e-8


def test_parameter_block_rounding():
    p = consts.Params()
    lp = _abi.make_params(p, (100, 45, 45, 1950))
    f = np.float32
    assert lp.vdrift == float(f(consts.get_vdrift(p)))
    assert lp.erho == float(f(0.5 * 1.38))
    assert lp.vref_minus_cm == 998.4375
    assert lp.bin_width == float(f(p.pixel_pitch / 10))
    assert lp.n_ticks == 2001 and lp.fee_interval == 18 and lp.param_nticks == 51
    assert [lp.tran_edges[i] for i in range(6)] == [float(v) for v in consts.tran_diff_bin_edges(p)]
    with pytest.raises(ValueError):
        _abi.make_params(p, (99, 45, 45, 1950))
    with pytest.raises(ValueError):
        _abi.make_params(p.replace(recombination_mode=7))


def test_field_map():
    from larndsim_gb300.workloads import SEGMENT_FIELDS
    fm = _abi.field_map(SEGMENT_FIELDS)
    assert fm.x == SEGMENT_FIELDS.index("x") and fm.n_fields == len(SEGMENT_FIELDS)
    with pytest.raises(ValueError):
        _abi.field_map(("x", "y"))


def test_jax_linspace_endpoints():
    t = consts.jax_linspace_f32(0.001, 10, 100)
    assert t.dtype == np.float32 and t[0] == np.float32(0.001) and t[-1] == np.float32(10)
    assert np.all(np.diff(t) > 0)


@pytest.fixture(scope="module")
def lib():
    from larndsim_gb300 import build
    if not _abi.LIB_PATH.exists():
        build.build()
    return _abi.load()


def test_library_exports_every_declared_symbol(lib):
    header = (ROOT / "include" / "lsim.h").read_text()
    names = set(re.findall(r"^\s*(?:int64_t|int|size_t|void|const char \*)\s*(lsim_\w+)\s*\(", header, re.M))
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(_abi.EXPORTED) <= names | {"lsim_valid_pixels"}


def test_library_abi_and_sizes(lib):
    assert lib.lsim_abi_version() == _abi.ABI_VERSION == 2
    p = _abi.make_params(consts.Params(number_pix_neighbors=4), (100, 45, 45, 1950))
    assert lib.lsim_lut_tables_bytes(p) > 40e6
    assert lib.lsim_workspace_bytes(p, 1000, 2) > 1000 * 192
    assert lib.lsim_hits_workspace_bytes(10, 10) >= 4


def test_library_rejects_bad_arguments_without_gpu(lib):
    p = _abi.make_params(consts.Params(number_pix_neighbors=4), (100, 45, 45, 1950))
    rc = lib.lsim_lut_prepare(p, None, None, 0, None)
    assert rc == _abi.LSIM_ERR_INVALID
    assert b"null" in lib.lsim_last_error()
    p.n_neighbors = 7
    assert lib.lsim_lut_prepare(p, ctypes.c_void_p(16), ctypes.c_void_p(16), 1 << 40, None) == _abi.LSIM_ERR_UNSUPPORTED


def test_next_row_entry_points_reject_bad_arguments_without_gpu(lib):
    """The probabilistic front end, the fit losses, the waveform VJP and the
    pixel coordinates validate their arguments before any launch."""
    V = ctypes.c_void_p
    p = _abi.make_params(consts.Params(number_pix_neighbors=4), (100, 45, 45, 1950))
    ws = V(256)
    big = 1 << 30
    # probabilistic front end
    assert lib.lsim_fee_prob_workspace_bytes(p) >= 4 * int(p.max_adc_values)
    assert lib.lsim_fee_prob(p, V(16), 4, 2000, 20, 1e-9, V(16), V(16), V(16), None, None, ws, big,
                             None) == _abi.LSIM_ERR_INVALID            # reductions: all three or none
    assert lib.lsim_fee_prob(p, V(16), 4, 2000, 20, 0.0, None, None, None, None, None, ws, big,
                             None) == _abi.LSIM_ERR_INVALID            # stop threshold
    assert lib.lsim_fee_prob(p, V(16), 4, 2000, 20, 1e-9, None, None, None, None, None, ws, 0,
                             None) == _abi.LSIM_ERR_CAPACITY
    assert lib.lsim_fee_prob(p, V(16), 4, 4096, 20, 1e-9, None, None, None, None, None, ws, big,
                             None) == _abi.LSIM_ERR_UNSUPPORTED        # n_t > 2048
    assert lib.lsim_fee_prob(p, V(16), 4, 2000, 40, 1e-9, None, None, None, None, None, ws, big,
                             None) == _abi.LSIM_ERR_UNSUPPORTED        # more than 32 paths
    p0 = _abi.make_params(consts.Params(RESET_NOISE_CHARGE=0))
    assert lib.lsim_fee_prob(p0, V(16), 4, 2000, 20, 1e-9, None, None, None, None, None, ws, big,
                             None) == _abi.LSIM_ERR_INVALID            # noise width 0
    assert lib.lsim_fee_prob_vjp(p, V(16), 4, 2000, 20, 1e-9, None, None, V(16), None, None, V(16), ws, big,
                                 None) == _abi.LSIM_ERR_INVALID       # reduction cotangents: all three or none
    assert lib.lsim_fee_prob_vjp(p, V(16), 4, 2000, 20, 1e-9, None, None, None, None, None, V(16), ws, 16,
                                 None) == _abi.LSIM_ERR_CAPACITY
    assert lib.lsim_fee_prob_vjp_workspace_bytes(p, 10, 20) >= 10 * int(p.max_adc_values) * 20 * 12
    # losses
    out = V(64)
    assert lib.lsim_mse_adc_workspace_bytes(1000, 900) > 4 * 1900
    assert lib.lsim_mse_adc(V(16), V(16), V(16), V(16), V(16), 10, V(16), V(16), V(16), V(16), V(16), 10, 0.0, 1.0,
                            out, None, None, ws, big, None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_mse_adc(V(16), V(16), V(16), V(16), V(16), 10, V(16), V(16), V(16), V(16), V(16), 10, 1.0, 1.0,
                            out, None, None, ws, 8, None) == _abi.LSIM_ERR_CAPACITY
    assert lib.lsim_mse_adc(None, V(16), V(16), V(16), V(16), 10, V(16), V(16), V(16), V(16), V(16), 10, 1.0, 1.0,
                            out, None, None, ws, big, None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_nll_loss(V(16), V(16), V(16), V(16), V(16), V(16), 10, V(16), V(16), V(16), V(16), V(16), V(16),
                             10, -1.0, out, None, None, None, ws, big, None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_nll_loss(V(16), V(16), V(16), V(16), V(16), V(16), 10, V(16), V(16), V(16), V(16), V(16), V(16),
                             10, 1.0, out, None, None, None, ws, 8, None) == _abi.LSIM_ERR_CAPACITY
    assert lib.lsim_chamfer_3d(V(16), V(16), V(16), V(16), V(16), 10, None, V(16), V(16), V(16), V(16), 10, out,
                               None, None, ws, big, None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_chamfer_3d(V(16), V(16), V(16), V(16), V(16), 1 << 32, V(16), V(16), V(16), V(16), V(16), 10,
                               out, None, None, ws, big, None) == _abi.LSIM_ERR_INVALID   # int32 neighbour indices
    # waveform VJP and pixel coordinates
    assert lib.lsim_lut_wfs_vjp(p, None, ws, 10, 1, V(16), 8, 4, V(16), None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_lut_wfs_vjp(p, V(16), ws, 10, 1, V(16), 2, 4, V(16), None) == _abi.LSIM_ERR_CAPACITY
    assert lib.lsim_pixel_coords(p, None, 5, None, None, None, None, None) == _abi.LSIM_ERR_INVALID
    # parametrised mode implements the default current model with longitudinal smearing only
    pn = _abi.make_params(consts.Params(number_pix_neighbors=0, mc_diff=True, diffusion_in_current_sim=False))
    fm = _abi.field_map(("eventID", "x", "y", "z", "x_start", "y_start", "z_start", "x_end", "y_end", "z_end",
                         "dx", "dE", "dEdx"))
    assert lib.lsim_param_stage1(pn, fm, V(16), 10, 1, None, ws, big, V(64), None) == _abi.LSIM_ERR_UNSUPPORTED
    assert lib.lsim_param_wfs_vjp(p, None, 10, 1, V(16), 8, 4, V(16), None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_param_wfs_vjp(p, ws, 10, 1, V(16), 2, 4, V(16), None) == _abi.LSIM_ERR_CAPACITY
    assert lib.lsim_fee_vjp_workspace_bytes(100) >= 100 * 4 * 1024
    assert lib.lsim_fee_vjp(p, V(16), 4, 2002, None, V(16), V(16), ws, big, None) == _abi.LSIM_ERR_UNSUPPORTED
    assert lib.lsim_fee_vjp(p, V(16), 4, 2000, None, None, V(16), ws, big, None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_fee_vjp(p, V(16), 4, 2000, None, V(16), V(16), ws, 16, None) == _abi.LSIM_ERR_CAPACITY


def test_hit_records_rejects_bad_arguments_without_gpu(lib):
    V = ctypes.c_void_p
    p = _abi.make_params(consts.Params())
    cols = _abi.LsimHitColumns(16, 16, 16, 16, 16, 16, 16, 16)
    no_pix = _abi.LsimHitColumns(16, 16, 16, 16, 16, 16, 16, None)
    counts = V(64)
    # a 16-byte summary and a 24-byte offset record per tile of 4096 hits
    assert lib.lsim_hit_records_workspace_bytes(3_000_000) >= 40 * (3_000_000 // 4096)
    assert lib.lsim_hit_records(None, 80.0, cols, 10, cols, None, None, None, None, counts, V(256), 1 << 20,
                                None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_hit_records(p, 80.0, cols, 10, cols, None, None, None, None, None, V(256), 1 << 20,
                                None) == _abi.LSIM_ERR_INVALID                  # counts required
    assert lib.lsim_hit_records(p, 80.0, no_pix, 10, cols, None, None, None, None, counts, V(256), 1 << 20,
                                None) == _abi.LSIM_ERR_INVALID                  # output column without input
    assert lib.lsim_hit_records(p, 80.0, cols, 10, cols, None, None, V(16), None, counts, V(256), 1 << 20,
                                None) == _abi.LSIM_ERR_INVALID                  # run_event without run_start
    assert lib.lsim_hit_records(p, 80.0, cols, 10, cols, None, None, None, None, counts, V(256), 8,
                                None) == _abi.LSIM_ERR_CAPACITY
    assert b"workspace" in lib.lsim_last_error()


def test_track_batch_entry_points_reject_bad_arguments_without_gpu(lib):
    V = ctypes.c_void_p
    assert lib.lsim_gather_tracks(V(16), 10, 0, V(16), 4, 0, None, V(16), V(16), None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_gather_tracks(V(16), 10, 120, V(16), 4, 0, None, V(16), V(16), None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_gather_tracks(V(16), 10, 26, V(16), 4, 30, V(16), V(16), V(16), None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_gather_tracks(V(16), 10, 26, V(16), 4, 0, None, V(16), None, None) == _abi.LSIM_ERR_INVALID
    roles = (ctypes.c_int8 * 3)(0, 1, 5)
    assert lib.lsim_pad_tracks(V(16), 4, 8, 3, 0, roles, -1, None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_pad_tracks(V(16), 4, 8, 3, 3, None, -1, None) == _abi.LSIM_ERR_INVALID


def test_noalloc_refuses_sizes_beyond_its_scratch_before_any_cuda_call(lib):
    """The size checks of lsim_hits_noalloc come before any CUDA call, so the
    refusals are tested here without a GPU.  On a machine with a visible GPU
    the test is skipped: its pointers are host placeholders that must never
    reach a kernel."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("placeholder pointers are only passed where no GPU is visible")
    cap = lib.lsim_hits_noalloc_max_slots()
    assert cap == 16384 * 1024
    p = _abi.make_params(consts.Params())
    H = int(p.max_adc_values)
    buf = np.zeros(16, np.float32)
    ph = ctypes.c_void_p(buf.ctypes.data)
    for n_pix in (cap // H + 1, 1 << 62):          # just past the limit, and a count whose product would wrap
        rc = lib.lsim_hits_noalloc(p, ph, ph, ph, n_pix, 1997, *([ph] * 8), ph, None)
        assert rc == _abi.LSIM_ERR_CAPACITY
        assert b"fixed scratch limit" in lib.lsim_last_error()
    p.max_adc_values = 0
    assert lib.lsim_hits_noalloc(p, ph, ph, ph, 4, 1997, *([ph] * 8), ph, None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_hits(p, ph, ph, ph, 4, 1997, *([ph] * 8), ph, ph, 1 << 20, None) == _abi.LSIM_ERR_INVALID


def test_fit_options_follow_the_reference_checks():
    from larndsim_gb300 import fit
    init = {k: v["nom"] for k, v in fit.RANGES.items()}
    with pytest.raises(ValueError, match="Unknown normalization_scheme"):
        fit.fit_options(("Ab",), 0.1, init, "linear")
    with pytest.raises(ValueError, match="must be > 0"):
        fit.fit_options(("Ab",), 0.1, init, "sigmoid", 0.0)
    with pytest.raises(ValueError, match="cannot fit"):
        fit.fit_options(("shift_x",), 0.1, init)


def test_likelihood_loss_entry_points_reject_bad_arguments_without_gpu(lib):
    """lsim_prob_llhd, lsim_llhd_loss and lsim_occurrence_indices validate
    their arguments before any launch."""
    V = ctypes.c_void_p
    p = _abi.make_params(consts.Params())
    big = 1 << 30
    assert lib.lsim_prob_llhd_workspace_bytes(1000) >= 8 * 3 * 4
    assert lib.lsim_prob_llhd_workspace_bytes(-1) == 0
    assert lib.lsim_prob_llhd(p, V(16), 0, 10, 2000, V(16), V(16), V(16), V(16), V(16), 5, 500.0, 1e-10, None,
                              V(16), None, None, V(256), big, None) == _abi.LSIM_ERR_INVALID   # hits, no pixels
    assert b"no simulated pixels" in lib.lsim_last_error()
    assert lib.lsim_prob_llhd(p, V(16), 4, 0, 2000, V(16), V(16), V(16), V(16), V(16), 5, 500.0, 1e-10, None,
                              V(16), None, None, V(256), big, None) == _abi.LSIM_ERR_INVALID   # n_values
    assert lib.lsim_prob_llhd(p, V(16), 4, 10, 2000, V(16), V(16), V(16), V(16), V(16), 5, 0.0, 1e-10, None,
                              V(16), None, None, V(256), big, None) == _abi.LSIM_ERR_INVALID   # sigma
    assert lib.lsim_prob_llhd(p, V(16), 4, 10, 2000, None, V(16), V(16), V(16), V(16), 5, 500.0, 1e-10, None,
                              V(16), None, None, V(256), big, None) == _abi.LSIM_ERR_INVALID   # null ids
    assert lib.lsim_prob_llhd(p, V(16), 4, 10, 2000, V(16), V(16), V(16), V(16), V(16), 5, 500.0, 1e-10, None,
                              V(16), None, None, V(256), 8, None) == _abi.LSIM_ERR_CAPACITY
    assert lib.lsim_llhd_loss(V(16), V(16), V(16), V(16), V(16), 4, 0, 500.0, None, V(16), None, None, None, None,
                              V(256), big, None) == _abi.LSIM_ERR_INVALID                     # n_ticks
    assert lib.lsim_llhd_loss(V(16), None, V(16), V(16), V(16), 4, 100, 500.0, None, V(16), None, None, None, None,
                              V(256), big, None) == _abi.LSIM_ERR_INVALID                     # null ticks
    assert lib.lsim_llhd_loss(V(16), V(16), V(16), V(16), V(16), 4, 100, 500.0, None, V(16), None, None, None, None,
                              V(256), 0, None) == _abi.LSIM_ERR_CAPACITY
    assert lib.lsim_occurrence_indices(V(16), -1, V(16), V(256), big, None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_occurrence_indices(V(16), 1 << 31, V(16), V(256), big, None) == _abi.LSIM_ERR_INVALID
    assert lib.lsim_occurrence_indices(V(16), 5000, V(16), V(256), 16, None) == _abi.LSIM_ERR_CAPACITY
