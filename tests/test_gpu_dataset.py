"""TracksDataset batches assembled on the GPU (gather with local event ids,
chop, pad: lsim_gather_tracks, lsim_chop_tracks, lsim_pad_tracks) against
the reference's own batches, bit for bit (tests/golden/dataset_ref.npz)."""

import numpy as np
import pytest
import torch

from larndsim_gb300 import dataio

from test_oracle_dataset import CASES, make

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gold():
    from test_oracle_dataset import GOLD
    return np.load(GOLD)


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


@pytest.mark.parametrize("name", list(CASES))
def test_batches_bitwise(cuda, gold, name):
    ds = make(gold, name)
    for i in range(len(ds)):
        b = ds[i]
        assert b.is_cuda and b.dtype == torch.float32
        np.testing.assert_array_equal(_bits(b.cpu().numpy()), _bits(gold[f"{name}/batch_{i}"]), err_msg=f"batch {i}")
    p = ds.pad_batch(ds[0], ds[0].shape[0] + 37, 0)
    np.testing.assert_array_equal(_bits(p.cpu().numpy()), _bits(gold[f"{name}/pad_batch_0"]))


def test_pad_batch_invalidates_foreign_events(cuda, gold):
    ds = make(gold, "batched")
    b = ds[0].clone()
    n_local = len(ds.get_batch_global_event_ids(0))
    b[3, ds._evt_col] = n_local + 2.0        # not a local event
    b[4, ds._evt_col] = n_local - 0.5        # integer part is a local event: kept
    out = ds.pad_batch(b, b.shape[0], 0).cpu().numpy()
    f = ds.get_track_fields()
    assert out[3, ds._evt_col] == -1 and out[3, f.index("dE")] == 0 and out[3, f.index("trackID")] == -1
    assert out[3, f.index("x")] == b[3, f.index("x")].item()
    assert out[4, ds._evt_col] == np.float32(n_local - 0.5)


def test_data_loader_stacks_padded_batches(cuda, gold):
    ds = make(gold, "batched")
    dl = dataio.DataLoader(ds, 3)
    stacks = list(dl)
    assert len(dl) == len(stacks) == 2 and stacks[0].shape == (3, ds.max_batch_nsteps, len(ds.get_track_fields()))
    np.testing.assert_array_equal(_bits(stacks[1][0].cpu().numpy()), _bits(gold["batched/batch_3"]))
