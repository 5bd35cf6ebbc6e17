"""TracksDataset batches assembled on the GPU (gather with local event ids,
chop, pad: lsim_gather_tracks, lsim_chop_tracks, lsim_pad_tracks): bit for
bit against the same assembly in numpy with the oracle's chop_tracks on the
same batch layout, and against the reference's own batches
(tests/golden/dataset_ref.npz) -- row for row where numpy's unstable argsort
orders the rows of a trajectory as it did when the golden batches were made
(x86-64), else as multisets of rows (not at all for the live-selection case,
whose layout itself follows that order)."""

import numpy as np
import pytest
import torch

from larndsim_gb300 import dataio
from oracle import reference_np as R

from test_oracle_dataset import CASES, SAME_SORT, golden_comparable, make

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gold():
    from test_oracle_dataset import GOLD
    return np.load(GOLD)


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def _pad_np(ds, batch, target, idx):
    """pad_batch / _invalidate_rows of optimize/dataio.py:347-373 in numpy."""
    f = ds.get_track_fields()
    b = np.asarray(batch, np.float32).copy()
    cur = b.shape[0]
    inval = np.zeros(max(cur, target), bool)
    if target > cur:
        b = np.pad(b, ((0, target - cur), (0, 0)))
        inval[cur:] = True
    if idx is not None:
        ev = b[:, ds._evt_col]
        n_local = len(ds.get_batch_global_event_ids(idx))
        inval |= (ev >= 0) & ~np.isin(ev.astype(np.int64), np.arange(n_local))
    b[inval, ds._evt_col] = -1
    for name in ("n_electrons", "dE", "dEdx", "dx", "long_diff", "tran_diff"):
        if name in f:
            b[inval, f.index(name)] = 0
    for name in ("trackID", "pixel_plane"):
        if name in f:
            b[inval, f.index(name)] = -1
    return b


def _assemble_np(ds, i):
    rows = ds.get_batch_row_indices(i)
    arr = dataio.np_from_structured(ds.tracks_struct[rows])
    arr = dataio.remap_event_ids_to_local(arr, ds.tracks_struct[rows]["eventID"], ds.get_batch_global_event_ids(i),
                                          ds.get_track_fields())
    if ds.chopped:
        arr = R.chop_tracks(arr, ds.get_track_fields(), ds.electron_sampling_resolution)
    if ds.pad and ds.max_batch_nsteps > 0 and arr.shape[0] < ds.max_batch_nsteps:
        arr = _pad_np(ds, arr, ds.max_batch_nsteps, i)
    return arr


def _same_rows(a, b):
    ka, kb = _bits(a), _bits(b)
    assert ka.shape == kb.shape
    np.testing.assert_array_equal(ka[np.lexsort(ka.T[::-1])], kb[np.lexsort(kb.T[::-1])])


@pytest.mark.parametrize("name", list(CASES))
def test_batches_bitwise(cuda, gold, name):
    ds = make(gold, name)
    for i in range(len(ds)):
        b = ds[i]
        assert b.is_cuda and b.dtype == torch.float32
        got = b.cpu().numpy()
        np.testing.assert_array_equal(_bits(got), _bits(_assemble_np(ds, i)), err_msg=f"batch {i}")
        want = gold[f"{name}/batch_{i}"]
        if SAME_SORT:
            np.testing.assert_array_equal(_bits(got), _bits(want), err_msg=f"batch {i}")
        elif golden_comparable(name):
            _same_rows(got, want)
    p = ds.pad_batch(ds[0], ds[0].shape[0] + 37, 0).cpu().numpy()
    np.testing.assert_array_equal(_bits(p), _bits(_pad_np(ds, ds[0].cpu().numpy(), ds[0].shape[0] + 37, 0)))
    if SAME_SORT:
        np.testing.assert_array_equal(_bits(p), _bits(gold[f"{name}/pad_batch_0"]))
    elif golden_comparable(name):
        _same_rows(p, gold[f"{name}/pad_batch_0"])


def test_pad_batch_invalidates_foreign_events(cuda, gold):
    ds = make(gold, "batched")
    b = ds[0].clone()
    n_local = len(ds.get_batch_global_event_ids(0))
    b[3, ds._evt_col] = n_local + 2.0        # not a local event
    b[4, ds._evt_col] = n_local - 0.5        # integer part is a local event: kept
    out = ds.pad_batch(b, b.shape[0], 0).cpu().numpy()
    np.testing.assert_array_equal(_bits(out), _bits(_pad_np(ds, b.cpu().numpy(), b.shape[0], 0)))
    f = ds.get_track_fields()
    assert out[3, ds._evt_col] == -1 and out[3, f.index("dE")] == 0 and out[3, f.index("trackID")] == -1
    assert out[4, ds._evt_col] == np.float32(n_local - 0.5)


def test_data_loader_stacks_padded_batches(cuda, gold):
    ds = make(gold, "batched")
    dl = dataio.DataLoader(ds, 3)
    stacks = list(dl)
    assert len(dl) == len(stacks) == 2 and stacks[0].shape == (3, ds.max_batch_nsteps, len(ds.get_track_fields()))
    np.testing.assert_array_equal(_bits(stacks[1][0].cpu().numpy()), _bits(ds[3].cpu().numpy()))


@pytest.mark.parametrize("name", ["tgt_batched", "tgt_unchopped"])
def test_target_batches_bitwise(cuda, gold, name):
    """Target batches (rows found by key and sorted: the same on every
    platform) against the reference's, bit for bit."""
    from test_oracle_dataset import make_target
    ds = make_target(gold, name)
    for i in range(len(ds)):
        got = ds[i].cpu().numpy()
        np.testing.assert_array_equal(_bits(got), _bits(gold[f"{name}/batch_{i}"]), err_msg=f"batch {i}")


def test_driver_loop_end_to_end(cuda, gold, tmp_path):
    """The simulate driver's loop (optimize/simulate.py:91-179) on the GPU:
    dataset batches, the id checks, simulate_wfs + simulate_stochastic, the
    hit records and the --out_np archive, each batch's hits equal to the
    oracle's chain on the same batch."""
    from larndsim_gb300 import consts, detsim, output, sim, workloads
    params = consts.Params(number_pix_neighbors=1, RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0,
                           long_diff_template=consts.jax_linspace_f32(0.001, 10, 10))
    tmpl = R.load_lut_templates(workloads.synthetic_response(seed=0, nx=15, ny=15), params)
    ds = make(gold, "batched")
    fields = ds.get_track_fields()
    recs = []
    sim.reset_size_history()
    hist = {}                                   # the oracle's pad_size history, in step with the GPU's
    for i in range(len(ds)):
        batch = ds[i]
        ev = batch[:, fields.index("eventID")].cpu().numpy()
        detsim.validate_local_event_ids(ev, context=f"batch {i}")
        detsim.validate_event_ids_for_packing(params, ev, kind="pixel")
        wfs, unique = sim.simulate_wfs(params, torch.from_numpy(tmpl).cuda(), batch, fields)
        out = sim.simulate_stochastic(params, wfs, unique, i)
        rec = output.hit_records(params, out)
        recs.append(rec)
        wo, uo = R.simulate_wfs(params, tmpl, batch.cpu().numpy(), fields, history=hist)
        ref = R.simulate_stochastic(params, wo, uo)
        assert rec["adc"].numel() <= ref["nb_valid"]
        np.testing.assert_array_equal(unique.cpu().numpy(), uo)
    path = tmp_path / "hits.npz"
    output.write_hits_npz(path, recs)
    d = np.load(path)
    assert d["adcs"].shape[0] == sum(r["adc"].numel() for r in recs)
