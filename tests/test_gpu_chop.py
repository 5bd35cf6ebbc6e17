"""Track chopping on the GPU (lsim_chop_tracks through larndsim_gb300.dataio)
against the reference's outputs (tests/golden/chop_ref.npz) and the oracle,
bit for bit, plus size-independent properties on a large input."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "chop_ref.npz"


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("case", ("p0p04", "p0p001", "p0p1"))
def test_chop_matches_reference_golden(cuda, case):
    from larndsim_gb300 import dataio
    g = np.load(GOLD)
    out = dataio.chop_tracks(g[f"{case}_in"], tuple(g["fields"]), float(g[f"{case}_precision"]))
    assert out.is_cuda and out.dtype == torch.float32
    np.testing.assert_array_equal(_bits(out.cpu().numpy()), _bits(g[f"{case}_out"]))


def test_chop_large_batch_matches_oracle(cuda):
    """40k tracks of the batched workload (muon segments and shower steps)
    cut at 0.01 cm: ~0.8M output rows, bit-identical to the oracle."""
    from larndsim_gb300 import dataio, workloads
    from oracle import reference_np as R
    tracks, fields = workloads.batched_events(seed=3, n_events=6, min_segments=3000, max_segments=12000)
    tracks = tracks[:40000]
    out = dataio.chop_tracks(tracks, fields, 0.01).cpu().numpy()
    ref = R.chop_tracks(tracks, fields, 0.01)
    assert out.shape == ref.shape and out.shape[0] > 10 * tracks.shape[0]
    np.testing.assert_array_equal(_bits(out), _bits(ref))


def test_chop_properties_at_full_size(cuda):
    """500k-segment shower event at the reference default 0.001 cm: the
    row count, the chain of step boundaries, each track's last step ending
    at the track end, and dE conserved per track to float32 rounding."""
    from larndsim_gb300 import dataio, workloads
    tracks, fields = workloads.large_shower_event(seed=2, n_segments=500_000, n_subtracks=40)
    col = {k: fields.index(k) for k in fields}
    t = torch.from_numpy(tracks).cuda()
    out = dataio.chop_tracks(t, fields, 0.001)
    seg = (tracks[:, [col["x_end"], col["y_end"], col["z_end"]]]
           - tracks[:, [col["x_start"], col["y_start"], col["z_start"]]]).astype(np.float32)
    sq = seg * seg
    length = np.sqrt((sq[:, 0] + sq[:, 1]) + sq[:, 2]).astype(np.float32)
    nsteps = np.maximum(np.ceil(length / np.float32(0.001)), 1).astype(np.int64)
    nsteps = torch.from_numpy(nsteps).cuda()
    assert out.shape[0] == int(nsteps.sum())
    src = torch.repeat_interleave(torch.arange(t.shape[0], device="cuda"), nsteps)
    last = torch.ones(out.shape[0], dtype=torch.bool, device="cuda")
    last[:-1] = src[1:] != src[:-1]
    for a, b in (("x_start", "x_end"), ("y_start", "y_end"), ("z_start", "z_end")):
        same = ~last[:-1]
        assert torch.equal(out[1:, col[a]][same], out[:-1, col[b]][same])
        assert torch.equal(out[last, col[b]], t[:, col[b]])
    de = torch.zeros(t.shape[0], dtype=torch.float64, device="cuda").index_add_(0, src, out[:, col["dE"]].double())
    ref = t[:, col["dE"]].double()
    assert torch.all((de - ref).abs() <= 1e-5 * ref.abs() + 1e-6)
    for c in ("eventID", "trackID", "dEdx", "pdgId"):
        assert torch.equal(out[:, col[c]], t[src, col[c]])


def test_chop_edge_cases(cuda):
    from larndsim_gb300 import _abi, dataio, sim
    g = np.load(GOLD)
    fields = tuple(g["fields"])
    empty = dataio.chop_tracks(np.zeros((0, len(fields)), np.float32), fields, 0.1)
    assert empty.shape == (0, len(fields))
    bad = g["p0p1_in"].copy()
    bad[5, fields.index("y_start")] = np.inf
    with pytest.raises(ValueError):
        dataio.chop_tracks(bad, fields, 0.1)
    # a capacity smaller than the row count writes only the leading rows
    lib = _abi.load()
    t = sim.as_tracks(g["p0p04_in"])
    n_ref = g["p0p04_out"].shape[0]
    guard = torch.full((n_ref, len(fields)), -7.0, device="cuda")
    ws = torch.empty(lib.lsim_chop_workspace_bytes(t.shape[0]), dtype=torch.uint8, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    cap = 300
    _abi.check(lib, lib.lsim_chop_tracks(_abi.field_map(fields), t.data_ptr(), t.shape[0], 0.04, guard.data_ptr(),
                                         cap, cnt.data_ptr(), ws.data_ptr(), ws.numel(), sim._stream()))
    assert int(cnt.item()) == n_ref
    got = guard.cpu().numpy()
    np.testing.assert_array_equal(_bits(got[:cap]), _bits(g["p0p04_out"][:cap]))
    assert np.all(got[cap:] == -7.0)
