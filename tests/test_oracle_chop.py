"""Pin the oracle's chop_tracks (optimize/dataio.py:63-106) to the
reference's own outputs (tests/golden/chop_ref.npz, made by running the
reference's chop_tracks with tests/golden/make_chop_golden.py), and check
the C ABI's argument handling without a GPU."""

import ctypes
from pathlib import Path

import numpy as np
import pytest

from oracle import reference_np as R

GOLD = Path(__file__).resolve().parent / "golden" / "chop_ref.npz"
CASES = ("p0p04", "p0p001", "p0p1")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("case", CASES)
def test_oracle_chop_matches_reference_bitwise(gold, case):
    fields = tuple(gold["fields"])
    out = R.chop_tracks(gold[f"{case}_in"], fields, float(gold[f"{case}_precision"]))
    ref = gold[f"{case}_out"]
    assert out.shape == ref.shape
    np.testing.assert_array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_oracle_chop_steps_chain(gold):
    """Every step starts where the previous step of its track ends."""
    fields = tuple(gold["fields"])
    t = gold["p0p04_in"]
    out = R.chop_tracks(t, fields, 0.04)
    ids = out[:, fields.index("trackID")]
    same = ids[1:] == ids[:-1]
    for a, b in (("x_start", "x_end"), ("y_start", "y_end"), ("z_start", "z_end")):
        np.testing.assert_array_equal(out[1:, fields.index(a)][same], out[:-1, fields.index(b)][same])
    assert out.shape[0] > t.shape[0]


def test_oracle_chop_rejects_non_finite_length(gold):
    fields = tuple(gold["fields"])
    t = gold["p0p1_in"].copy()
    t[3, fields.index("x_end")] = np.nan
    with pytest.raises(ValueError):
        R.chop_tracks(t, fields, 0.1)


def test_chop_abi_argument_checks_without_gpu():
    from larndsim_gb300 import _abi
    lib = _abi.load()
    fields = tuple(np.load(GOLD)["fields"])
    fm = _abi.field_map(fields)
    assert lib.lsim_chop_workspace_bytes(1000) >= 16 * 1000
    assert lib.lsim_chop_workspace_bytes(0) > 0
    cnt = ctypes.c_void_p(64)
    ws = ctypes.c_void_p(256)
    # a non-positive precision and a short workspace fail before any launch
    assert lib.lsim_chop_tracks(fm, ctypes.c_void_p(16), 10, 0.0, None, 0, cnt, ws, 1 << 20, None) == _abi.LSIM_ERR_INVALID
    assert b"precision" in lib.lsim_last_error()
    assert lib.lsim_chop_tracks(fm, ctypes.c_void_p(16), 10, 0.1, None, 0, cnt, ws, 8, None) == _abi.LSIM_ERR_CAPACITY
    assert lib.lsim_chop_tracks(fm, ctypes.c_void_p(16), 10, 0.1, None, 5, cnt, ws, 1 << 20, None) == _abi.LSIM_ERR_INVALID
    bad = _abi.field_map(fields)
    bad.dE = len(fields)
    assert lib.lsim_chop_tracks(bad, ctypes.c_void_p(16), 10, 0.1, None, 0, cnt, ws, 1 << 20, None) == _abi.LSIM_ERR_INVALID
