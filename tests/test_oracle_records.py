"""Output side (optimize/simulate.py:129-176) on the CPU: the oracle's hit
records pinned to the reference's committed outputs, and the host-side
per-event split and writers of larndsim_gb300.output run on CPU tensors."""

from pathlib import Path

import numpy as np
import pytest
import torch

from larndsim_gb300 import consts, output
from oracle import reference_np as R

F = np.float32
GOLD = Path(__file__).resolve().parent / "golden" / "jax_ref_hits.npz"


@pytest.fixture(scope="module")
def params():
    return consts.Params()


@pytest.mark.parametrize("tag", ["lut_rows", "parametrized_rows"])
def test_records_of_committed_outputs_are_idempotent(params, tag):
    """The committed --out_np rows are records already: every row is kept,
    and the recomputed charge equals the committed one bit for bit."""
    d = np.load(GOLD)[tag]
    adc, q, x, y, z, ticks = (d[:, i].view(F) for i in range(6))
    ev = d[:, 6].view(np.int32)
    rec = R.hit_records(params, adc, x, y, z, ticks, np.ones_like(adc), ev, np.arange(adc.size, dtype=np.int32))
    assert rec["adc"].size == adc.size
    np.testing.assert_array_equal(rec["Q"].view(np.uint32), q.view(np.uint32))
    np.testing.assert_array_equal(rec["event"], ev)


def test_adc_lowest_is_digitized_threshold(params):
    lo = output.adc_lowest(params)
    assert F(lo) == R.digitize(params, F(params.DISCRIMINATION_THRESHOLD))
    assert F(lo) == F(80.951485)
    p7 = params.replace(DISCRIMINATION_THRESHOLD=7000)
    assert F(output.adc_lowest(p7)) == R.digitize(p7, F(7000))


def _random_hits(rng, n, n_events, contiguous=True):
    ev = np.sort(rng.integers(-1, n_events, n)).astype(np.int32) if contiguous else \
        rng.integers(-1, n_events, n).astype(np.int32)
    adc = rng.uniform(75, 256, n).astype(F)
    return [adc, rng.normal(size=n).astype(F), rng.normal(size=n).astype(F), rng.normal(size=n).astype(F),
            rng.uniform(0, 2000, n).astype(F), np.ones(n, F), ev, rng.integers(0, 10 ** 6, n).astype(np.int32)]


def _runs(ev):
    head = np.ones(ev.size, bool)
    head[1:] = ev[1:] != ev[:-1]
    starts = np.flatnonzero(head)
    return ev[starts], np.append(starts, ev.size)


def _records_on_cpu(params, cols):
    """What lsim_hit_records returns, assembled from the oracle on CPU
    tensors, so the host-side split can be tested without a GPU."""
    r = R.hit_records(params, *cols)
    run_event, run_start = _runs(r["event"])
    rec = output.HitRecords({k: torch.from_numpy(v) for k, v in r.items()})
    rec["run_event"] = torch.from_numpy(run_event)
    rec["run_start"] = torch.from_numpy(run_start)
    return r, rec


@pytest.mark.parametrize("contiguous", [True, False])
def test_by_event_matches_reference_grouping(params, contiguous):
    rng = np.random.default_rng(5)
    cols = _random_hits(rng, 5000, 12, contiguous)
    r, rec = _records_on_cpu(params, cols)
    gids = list(range(100, 112))
    got = rec.by_event(gids)
    ref = R.hit_records_by_event(r, {i: g for i, g in enumerate(gids)})
    assert list(got) == list(ref)
    for g in ref:
        assert set(got[g]) == set(output.GROUP_FIELDS)
        for k in output.GROUP_FIELDS:
            np.testing.assert_array_equal(got[g][k], ref[g][k])
            assert got[g][k].dtype == ref[g][k].dtype
        assert got[g]["eventID"].dtype == np.int64 and np.all(got[g]["eventID"] == g)


def test_writers_round_trip(params, tmp_path):
    rng = np.random.default_rng(6)
    batches, refs = [], []
    for b in range(2):
        r, rec = _records_on_cpu(params, _random_hits(rng, 800, 4))
        batches.append(rec)
        refs.append(r)
    flat = tmp_path / "hits.npz"
    output.write_hits_npz(flat, batches)
    d = np.load(flat)
    assert sorted(d.files) == sorted(["adcs", "Q", "x", "y", "z", "ticks", "hit_prob", "event_id"])
    np.testing.assert_array_equal(d["adcs"], np.concatenate([r["adc"] for r in refs]))
    np.testing.assert_array_equal(d["event_id"], np.concatenate([r["event"] for r in refs]))
    grp = tmp_path / "groups.npz"
    output.write_hits_groups_npz(grp, batches, [[10, 11, 12, 13], [20, 21, 22, 23]])
    g = np.load(grp)
    for b, r in enumerate(refs):
        ref = R.hit_records_by_event(r, {i: (10 if b == 0 else 20) + i for i in range(4)})
        for gid, fields in ref.items():
            for k, v in fields.items():
                np.testing.assert_array_equal(g[f"batch_{b}/event_{gid}/{k}"], v)


def test_h5_writer_needs_h5py(params, tmp_path):
    try:
        import h5py  # noqa: F401
        pytest.skip("h5py present")
    except ImportError:
        pass
    with pytest.raises(ImportError, match="h5py"):
        output.write_hits_h5(tmp_path / "x.h5", [])


def test_by_event_needs_runs(params):
    rec = output.HitRecords({"adc": torch.zeros(0)})
    with pytest.raises(ValueError, match="runs=False"):
        rec.by_event()
