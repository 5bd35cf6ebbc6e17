"""Simulation strategies: the fitters' plug point (reference:
optimize/strategies.py:80-149).  ``predict(params, tracks, fields, rngkey)``
returns the same dictionary keys as the reference's strategies."""

from __future__ import annotations

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


class ParametrizedSimulation(SimulationStrategy):
    """Parametrised-current mode (strategies.py:136-149)."""

    def predict(self, params, tracks, fields, rngkey):
        adcs, x, y, z, ticks, hit_prob, event, unique_pixels = sim.simulate_parametrized(
            params, tracks, fields, rngseed=0 if rngkey is None else rngkey)
        return {"adcs": adcs, "pixel_x": x, "pixel_y": y, "pixel_z": z, "ticks": ticks, "hit_prob": hit_prob,
                "event": event, "unique_pixels": unique_pixels}
