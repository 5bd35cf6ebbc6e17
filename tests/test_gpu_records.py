"""Hit records on the GPU (lsim_hit_records through output.hit_records)
against the oracle's restatement of optimize/simulate.py:129-176: every
column bit for bit, the event runs, the per-event groups, and the charges
of the reference's committed outputs."""

from pathlib import Path

import numpy as np
import pytest
import torch

from larndsim_gb300 import consts, output, sim, workloads
from oracle import reference_np as R

from gpu_common import small_params

pytestmark = pytest.mark.gpu
F = np.float32
GOLD = Path(__file__).resolve().parent / "golden" / "jax_ref_hits.npz"
COLS = ("adc", "adc_clean", "Q", "pix_x", "pix_y", "pix_z", "ticks", "hit_prob", "event", "pixels")


def _random_hits(rng, n, n_events, contiguous=True):
    ev = rng.integers(-1, n_events, n).astype(np.int32)
    if contiguous:
        ev.sort()
    adc = rng.uniform(75, 256, n).astype(F)
    return [adc, rng.normal(size=n).astype(F), rng.normal(size=n).astype(F), rng.normal(size=n).astype(F),
            rng.uniform(0, 2000, n).astype(F), rng.uniform(0, 1, n).astype(F), ev,
            rng.integers(-5, 10 ** 6, n).astype(np.int32)]


def _same(got, want, name):
    """Bit-identical, except that any NaN matches any NaN (the GPU returns
    the canonical NaN, numpy keeps the input's payload)."""
    assert got.dtype == want.dtype, name
    if got.dtype != F:
        np.testing.assert_array_equal(got, want, err_msg=name)
        return
    nan = np.isnan(want)
    np.testing.assert_array_equal(np.isnan(got), nan, err_msg=name)
    np.testing.assert_array_equal(got[~nan].view(np.uint32), want[~nan].view(np.uint32), err_msg=name)


def _check(params, cols, rec):
    ref = R.hit_records(params, *cols)
    for k in COLS:
        _same(rec[k].cpu().numpy(), ref[k], k)
    ev = ref["event"]
    head = np.ones(ev.size, bool)
    head[1:] = ev[1:] != ev[:-1]
    starts = np.flatnonzero(head)
    np.testing.assert_array_equal(rec["run_event"].cpu().numpy(), ev[starts])
    np.testing.assert_array_equal(rec["run_start"].cpu().numpy(), np.append(starts, ev.size))
    return ref


@pytest.mark.parametrize("n,contiguous", [(1, True), (1000, True), (3_000_000, True), (200_000, False)])
def test_records_match_oracle(cuda, n, contiguous):
    params = consts.Params()
    rng = np.random.default_rng(n)
    cols = _random_hits(rng, n, 40, contiguous)
    lo = F(output.adc_lowest(params))
    # rows whose ADC is exactly the lowest ADC are dropped; NaN ADCs are kept
    k = min(n, 50)
    cols[0][rng.choice(n, k, replace=False)] = lo
    if n > 10:
        cols[0][3] = np.nan
    rec = output.hit_records(params, cols)
    ref = _check(params, cols, rec)
    if contiguous and n > 10:
        gids = list(range(1000, 1040))
        got = rec.by_event(gids)
        want = R.hit_records_by_event(ref, {i: g for i, g in enumerate(gids)})
        assert list(got) == list(want)
        for g in want:
            for f in output.GROUP_FIELDS:
                _same(got[g][f], want[g][f], f)


def test_records_of_non_contiguous_events_group_like_the_reference(cuda):
    params = consts.Params()
    cols = _random_hits(np.random.default_rng(9), 20_000, 7, contiguous=False)
    rec = output.hit_records(params, cols)
    ref = _check(params, cols, rec)
    got, want = rec.by_event(), R.hit_records_by_event(ref)
    assert list(got) == list(want)
    for g in want:
        for f in output.GROUP_FIELDS:
            np.testing.assert_array_equal(got[g][f], want[g][f])


def test_empty_and_all_dropped(cuda):
    params = consts.Params()
    rec = output.hit_records(params, [np.zeros(0, F)] * 6 + [np.zeros(0, np.int32)] * 2)
    assert rec["adc"].numel() == 0 and rec["run_start"].cpu().tolist() == [0]
    cols = _random_hits(np.random.default_rng(1), 3000, 3)
    cols[6][:] = -1
    rec = output.hit_records(params, cols)
    assert rec["adc"].numel() == 0 and rec["run_event"].numel() == 0
    assert rec["run_start"].cpu().tolist() == [0] and rec.by_event() == {}


@pytest.mark.parametrize("tag", ["lut_rows", "parametrized_rows"])
def test_committed_charges_bitwise(cuda, tag):
    d = np.load(GOLD)[tag]
    adc, q = d[:, 0].view(F), d[:, 1].view(F)
    ev = d[:, 6].view(np.int32)
    n = adc.size
    cols = [adc] + [np.zeros(n, F)] * 5 + [ev, np.zeros(n, np.int32)]
    rec = output.hit_records(consts.Params(), cols)
    assert rec["Q"].numel() == n
    np.testing.assert_array_equal(rec["Q"].cpu().numpy().view(np.uint32), q.view(np.uint32))


def test_records_of_a_simulated_batch(cuda):
    """The driver's chain: simulate_wfs + simulate_stochastic, then the
    records, on two muon events."""
    params = small_params(n_neighbors=1)
    t0, fields = workloads.muon_event(seed=21, n_tracks=4, event_id=0)
    t1, _ = workloads.muon_event(seed=22, n_tracks=4, event_id=1)
    tracks = np.concatenate([t0, t1])
    resp = workloads.synthetic_response(seed=0, nx=15, ny=15)
    tmpl = torch.from_numpy(R.load_lut_templates(resp, params)).cuda()
    wfs, unique = sim.simulate_wfs(params, tmpl, tracks, fields)
    out = sim.simulate_stochastic(params, wfs, unique, 0)
    cols = [t.cpu().numpy() for t in out]
    rec = output.hit_records(params, out)
    ref = _check(params, cols, rec)
    assert ref["adc"].size > 0
    groups = rec.by_event([7, 9])
    assert set(groups) <= {7, 9} and sum(g["adc"].size for g in groups.values()) == ref["adc"].size
