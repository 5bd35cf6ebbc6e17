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


@pytest.mark.gpu
def test_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    from larndsim_gb300 import _abi
    lib = _abi.load()
    lp = _abi.make_params(small_params())
    n_pix = MAX_SLOTS // int(lp.max_adc_values) + 1
    fake = ctypes.c_void_p(256)        # never dereferenced: the size check comes first
    rc = lib.lsim_hits_noalloc(lp, fake, fake, fake, n_pix, 1997, *([fake] * 8), fake, None)
    assert rc == _abi.LSIM_ERR_CAPACITY
    assert b"fixed scratch limit" in lib.lsim_last_error()
