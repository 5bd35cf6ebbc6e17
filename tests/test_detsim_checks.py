"""Host-side event-id checks (src/larndsim/detsim_jax.py:26-154): known
answers for the module0 geometry and the reference's exceptions."""

import numpy as np
import pytest

from larndsim_gb300 import consts, detsim

I64 = int(np.iinfo(np.int64).max)


@pytest.fixture(scope="module")
def params():
    return consts.Params()


def test_strides_and_limits(params):
    assert detsim._pixel_id_stride(params) == 140 * 280 * 2
    assert detsim._bin_id_stride(params) == 1400 * 2800 * 2
    safe = detsim.max_safe_event_id_for_pixel_packing(params)
    assert safe == (I64 - (78400 - 1)) // 78400
    assert detsim.max_possible_pixel_id(params, safe) <= I64 < detsim.max_possible_pixel_id(params, safe + 1)
    safe_b = detsim.max_safe_event_id_for_bin_packing(params)
    assert detsim.max_possible_bin_id(params, safe_b) <= I64 < detsim.max_possible_bin_id(params, safe_b + 1)
    assert detsim.max_possible_pixel_id(params, 0) == 78400 - 1


def test_packing_checks(params):
    detsim.validate_event_ids_for_packing(params, [])
    detsim.validate_event_ids_for_packing(params, [-1, -1])
    detsim.validate_event_ids_for_packing(params, [-1, 0, 5], kind="bin")
    with pytest.raises(ValueError, match=r"below -1: \[-3\]"):
        detsim.validate_event_ids_for_packing(params, [0, -3], context="batch 0")
    with pytest.raises(OverflowError, match="int64-safe limit"):
        detsim.validate_event_ids_for_packing(params, [detsim.max_safe_event_id_for_bin_packing(params) + 1],
                                              kind="bin")
    with pytest.raises(ValueError, match="Unknown packing kind"):
        detsim.validate_event_ids_for_packing(params, [0], kind="voxel")


def test_decoding_checks(params):
    detsim.validate_packed_ids_for_decoding(params, [-1, 0, 78400 * 7 + 3])
    with pytest.raises(ValueError, match="packed ids below -1"):
        detsim.validate_packed_ids_for_decoding(params, [-2])
    with pytest.raises(ValueError, match="Unknown decoding kind"):
        detsim.validate_packed_ids_for_decoding(params, [1], kind="voxel")


def test_local_namespace(params):
    detsim.validate_local_event_ids([-1, 0, 1, 1, 2, -1])
    detsim.validate_local_event_ids([-1, -1])
    with pytest.raises(ValueError, match="contiguous local namespace"):
        detsim.validate_local_event_ids([0, 2])
    with pytest.raises(ValueError, match="non-local namespace"):
        detsim.validate_local_event_ids([0, -5])
