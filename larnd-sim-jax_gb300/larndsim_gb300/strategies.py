"""Simulation strategies: the fitters' plug point (reference:
optimize/strategies.py:80-149).  ``predict(params, tracks, fields, rngkey)``
returns the same dictionary keys as the reference's strategies."""

from __future__ import annotations

import torch

from . import sim


class SimulationStrategy:
    def predict(self, params, tracks, fields, rngkey):
        raise NotImplementedError


class LUTSimulation(SimulationStrategy):
    """LUT mode: simulate_wfs + simulate_stochastic (strategies.py:87-105)."""

    def __init__(self, response):
        self.response = response

    def predict(self, params, tracks, fields, rngkey):
        wfs, unique_pixels = sim.simulate_wfs(params, self.response, tracks, fields)
        adcs, x, y, z, ticks, hit_prob, event, hit_pixels = sim.simulate_stochastic(
            params, wfs, unique_pixels, rngseed=0 if rngkey is None else rngkey)
        return {"adcs": adcs, "pixel_x": x, "pixel_y": y, "pixel_z": z, "ticks": ticks, "hit_prob": hit_prob,
                "event": event, "hit_pixels": hit_pixels, "unique_pixels": unique_pixels, "wfs": wfs}


def pad_to_closest_multiple(x, dims_to_pad=None, multiple=128, pad_value=0, pad_front=False):
    """Pad the given dimensions of x up to a multiple of ``multiple``
    (strategies.py:41-77), at the front when ``pad_front``."""
    x = torch.as_tensor(x)
    dims = range(x.dim()) if dims_to_pad is None else dims_to_pad
    shape = list(x.shape)
    for d in dims:
        shape[d] = (x.shape[d] + multiple - 1) // multiple * multiple
    out = torch.full(shape, pad_value, dtype=x.dtype, device=x.device)
    sl = tuple(slice(t - n, None) if pad_front else slice(0, n) for t, n in zip(shape, x.shape))
    out[sl] = x
    return out


class LUTProbabilisticSimulation(SimulationStrategy):
    """LUT mode with the probabilistic front end (strategies.py:107-134):
    simulate_wfs, rows padded at the front to a multiple of 128, then
    simulate_probabilistic."""

    def __init__(self, response):
        self.response = response

    def predict(self, params, tracks, fields, rngkey):
        wfs, unique_pixels = sim.simulate_wfs(params, self.response, tracks, fields)
        unique_pixels = pad_to_closest_multiple(unique_pixels, multiple=128, pad_value=-1, pad_front=True)
        wfs = pad_to_closest_multiple(wfs, dims_to_pad=(0,), multiple=128, pad_value=0.0, pad_front=True)
        adcs_distrib, x, y, ticks_prob, event = sim.simulate_probabilistic(params, wfs, unique_pixels)
        _, _, plane, _ = sim.pixel_coordinates(params, unique_pixels)
        return {"adcs_distrib": adcs_distrib, "hit_prob": ticks_prob, "pixel_x": x, "pixel_y": y,
                "pixel_plane": plane, "event": event, "unique_pixels": unique_pixels, "hit_pixels": unique_pixels,
                "wfs": wfs}


class ParametrizedSimulation(SimulationStrategy):
    """Parametrised-current mode (strategies.py:136-149)."""

    def predict(self, params, tracks, fields, rngkey):
        adcs, x, y, z, ticks, hit_prob, event, unique_pixels = sim.simulate_parametrized(
            params, tracks, fields, rngseed=0 if rngkey is None else rngkey)
        return {"adcs": adcs, "pixel_x": x, "pixel_y": y, "pixel_z": z, "ticks": ticks, "hit_prob": hit_prob,
                "event": event, "unique_pixels": unique_pixels}
