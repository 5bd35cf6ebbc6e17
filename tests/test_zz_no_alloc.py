"""lsim_hits_noalloc: hit assembly and compaction for callers that cannot
allocate device memory (a plug-in inside a framework that has already
reserved the GPU's memory for its own pool, or code under a fixed
device-memory budget).  It must give exactly what lsim_hits gives with a
caller-allocated workspace, call after call, and refuse sizes beyond its
fixed scratch.  This file is collected last on purpose."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from gpu_common import small_params

MAX_SLOTS = 16384 * 1024


def _grids(seed, n_tracks):
    """A simulated event's digitised ADC / tick grids and pixel ids."""
    from larndsim_gb300 import _abi, sim, workloads
    from oracle import reference_np as R
    p = small_params()
    resp = workloads.synthetic_response(seed=0, nx=15, ny=15)
    tmpl = torch.from_numpy(R.load_lut_templates(resp, p)).cuda()
    tracks, fields = workloads.muon_event(seed=seed, n_tracks=n_tracks)
    wfs, unique = sim.simulate_wfs(p, tmpl, tracks, fields)
    lib = _abi.load()
    lp = _abi.make_params(p)
    P, T = wfs.shape
    H = int(p.MAX_ADC_VALUES)
    adc = torch.empty((P, H), dtype=torch.float32, device="cuda")
    ticks = torch.empty((P, H), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    _abi.check(lib, lib.lsim_fee(lp, wfs.data_ptr(), P, T, None, adc.data_ptr(), ticks.data_ptr(), None, s))
    return lib, lp, adc, ticks, unique, T - 3


def _call(lib, lp, adc, ticks, unique, tick_limit, noalloc):
    from larndsim_gb300 import _abi
    P, H = adc.shape
    n = P * H
    f = [torch.full((n,), -7.0, dtype=torch.float32, device="cuda") for _ in range(6)]
    ev = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    pix = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    nb = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    args = [lp, adc.data_ptr(), ticks.data_ptr(), unique.data_ptr(), P, tick_limit] + [t.data_ptr() for t in f] + \
        [ev.data_ptr(), pix.data_ptr(), nb.data_ptr()]
    if noalloc:
        rc = lib.lsim_hits_noalloc(*args, s)
    else:
        wb = lib.lsim_hits_workspace_bytes(P, H)
        ws = torch.empty(wb, dtype=torch.uint8, device="cuda")
        rc = lib.lsim_hits(*args, ws.data_ptr(), wb, s)
    _abi.check(lib, rc)
    k = int(nb.item())
    return [t[:k].cpu().numpy() for t in f + [ev, pix]]


@pytest.mark.gpu
def test_noalloc_matches_workspace_entry_point_on_consecutive_calls(cuda):
    for seed, n_tracks in ((31, 4), (32, 7)):      # two calls in a row, different sizes
        lib, lp, adc, ticks, unique, limit = _grids(seed, n_tracks)
        ref = _call(lib, lp, adc, ticks, unique, limit, noalloc=False)
        got = _call(lib, lp, adc, ticks, unique, limit, noalloc=True)
        assert ref[0].shape[0] > 0
        for a, b in zip(got, ref):
            np.testing.assert_array_equal(a, b)


def _synthetic_grids(n_pix, H, seed=5):
    """Random ADC and tick grids over n_pix sorted pixel ids (a few -1 rows
    first, as simulate_wfs orders them), on the device."""
    rng = np.random.default_rng(seed)
    adc = torch.from_numpy(rng.uniform(70.0, 130.0, (n_pix, H)).astype(np.float32)).cuda()
    ticks = torch.from_numpy(rng.integers(0, 2000, (n_pix, H)).astype(np.float32)).cuda()
    pids = np.sort(rng.integers(0, 1 << 30, n_pix).astype(np.int32))
    pids[:3] = -1
    return adc, ticks, torch.from_numpy(pids).cuda()


@pytest.mark.gpu
def test_noalloc_at_its_slot_limit_matches_workspace_entry_point(cuda):
    """The largest accepted size, compared bit for bit with lsim_hits; one
    pixel more is refused.  Every buffer is sized for the refused call too,
    so no call can reach past an allocation."""
    from larndsim_gb300 import _abi
    lib = _abi.load()
    lp = _abi.make_params(small_params())
    H = int(lp.max_adc_values)
    cap = int(lib.lsim_hits_noalloc_max_slots())
    assert cap == MAX_SLOTS
    n_pix = cap // H
    adc, ticks, unique = _synthetic_grids(n_pix + 1, H)
    ref = _call(lib, lp, adc[:n_pix], ticks[:n_pix], unique[:n_pix], 1997, noalloc=False)
    got = _call(lib, lp, adc[:n_pix], ticks[:n_pix], unique[:n_pix], 1997, noalloc=True)
    assert ref[0].shape[0] > 0.9 * (n_pix - 3) * H
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)
    n = (n_pix + 1) * H
    outs = [torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(6)] + \
        [torch.empty(n, dtype=torch.int32, device="cuda") for _ in range(2)]
    nb = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.lsim_hits_noalloc(lp, adc.data_ptr(), ticks.data_ptr(), unique.data_ptr(), n_pix + 1, 1997,
                               *[t.data_ptr() for t in outs], nb.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == _abi.LSIM_ERR_CAPACITY
    assert b"fixed scratch limit" in lib.lsim_last_error()
