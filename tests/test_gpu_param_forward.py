"""Parametrised-mode forward parity (reference sim_jax.py:339-372): GPU vs
the CPU oracle with the same Monte-Carlo diffusion draws supplied."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_common import ADC_RTOL, WFS_RTOL, compare_fee, compare_wfs, small_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["muon", "shower"])
def test_param_waveforms_and_hits(cuda, kind):
    from larndsim_gb300 import sim, workloads
    from oracle import reference_np as R
    p = small_params(n_neighbors=0, mc_diff=True)
    if kind == "muon":
        tracks, fields = workloads.muon_event(seed=21)
    else:
        tracks, fields = workloads.shower_event(seed=22, n_segments=1500)
    tracks = workloads.pad_tracks(tracks, fields, tracks.shape[0] + 17)
    rng = np.random.default_rng(5)
    offsets = rng.standard_normal((tracks.shape[0], 3)).astype(np.float32)
    sim.reset_size_history()
    out, wfs, unique = sim.simulate_parametrized(p, tracks, fields, offsets=torch.from_numpy(offsets).cuda(),
                                                 return_wfs=True)
    ref = R.simulate_parametrized(p, tracks, fields, offsets, history={})
    assert compare_wfs(wfs.cpu().numpy(), unique.cpu().numpy(), ref["wfs"], ref["unique_pixels"]) < WFS_RTOL
    integral, ticks = sim.get_adc_values(p, wfs)
    ai, ti = R.get_adc_values(p, wfs.cpu().numpy())
    frac, err = compare_fee(integral.cpu().numpy(), ticks.cpu().numpy(), ai, ti, p)
    assert frac < 0.005 and err < ADC_RTOL
    assert out[0].shape[0] > 0
