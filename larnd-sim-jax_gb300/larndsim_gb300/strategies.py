"""Simulation and loss strategies: the fitters' plug points (reference:
optimize/strategies.py).  ``predict(params, tracks, fields, rngkey)``
returns the same dictionary keys as the reference's simulation strategies
(:80-149); ``compute(params, prediction, target)`` returns (loss, aux) like
its loss strategies (:150-567)."""

from __future__ import annotations

import numpy as np
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


# ---------------------------------------------------------------- loss strategies

def compute_occurrence_indices(ids):
    """strategies.py:14-40: the index of each element within its run of
    equal consecutive ids ([100, 100, 100, 200, 200, 300] -> [0, 1, 2, 0,
    1, 0]), by a max-scan of run starts on the device
    (lsim_occurrence_indices)."""
    from . import _abi
    lib = _abi.load()
    t = torch.as_tensor(ids)
    dev = t.device if t.is_cuda else sim._device()
    t = t.to(device=dev, dtype=torch.int32).reshape(-1).contiguous()
    n = t.shape[0]
    out = torch.empty(n, dtype=torch.int32, device=dev)
    ws = torch.empty(max(lib.lsim_occurrence_workspace_bytes(n), 1), dtype=torch.uint8, device=dev)
    _abi.check(lib, lib.lsim_occurrence_indices(sim._ptr(t), n, sim._ptr(out), sim._ptr(ws), ws.numel(),
                                                sim._stream()))
    return out


def _dev_tensor(x, dtype, dev):
    return torch.as_tensor(x).to(device=dev, dtype=dtype).contiguous()


def _hit_z(params, ticks, plane, theta=None):
    """get_hit_z (detsim_jax.py:309-319); with ``theta`` (the 8 parameter
    values) differentiable in eField through the drift velocity."""
    from . import grad
    from .consts import get_vdrift
    if theta is not None:
        return grad._hit_z(params, theta, ticks, plane)
    v = np.float32(get_vdrift(params))
    b = torch.as_tensor(np.asarray(params.tpc_borders, np.float32), device=ticks.device)[plane.long()]
    za, zh = b[..., 2, 0], b[..., 2, 1]
    return za + ((ticks * np.float32(params.t_sampling)) * v) * torch.sign(zh - za)


class LossStrategy:
    """strategies.py:150-159: ``compute(params, prediction, target)`` ->
    (loss, aux) with the prediction and target as dictionaries."""

    def __init__(self, **kwargs):
        self.kwargs = kwargs

    def compute(self, params, prediction, target):
        raise NotImplementedError


class GenericLossStrategy(LossStrategy):
    """strategies.py:161-180: a hit-level loss (mse_adc, chamfer_3d,
    nll_loss, ...) on the predicted and target hits, charges from
    adc2charge."""

    def __init__(self, loss_fn, **kwargs):
        super().__init__(**kwargs)
        self.loss_fn = loss_fn

    def compute(self, params, prediction, target):
        from .losses import adc2charge
        Q = adc2charge(prediction["adcs"], params)
        ref_Q = adc2charge(target["adcs"], params)
        return self.loss_fn(params, Q, prediction["pixel_x"], prediction["pixel_y"], prediction["pixel_z"],
                            prediction["ticks"], prediction["hit_prob"], prediction["event"], ref_Q,
                            target["pixel_x"], target["pixel_y"], target["pixel_z"], target["ticks"],
                            target["hit_prob"], target["event"], **self.kwargs)


class CollapsedProbabilisticLossStrategy(LossStrategy):
    """strategies.py:182-335: the probabilistic front end's distributions
    collapsed into pseudo-hits and scored with a hit-level loss.  With
    ``collapsed`` (default) one pseudo-hit per (pixel, hit) at the expected
    tick and ADC of get_average_hit_values over the prediction's
    ``hit_prob``; otherwise one per (pixel, hit, tick) entry above
    ``hit_threshold``.  As in the reference, ``hit_prob`` is passed to these
    as it comes (the front end's log-probabilities).  A ``theta`` entry in
    the prediction (the 8 parameter values) makes the pseudo-hits' z
    differentiable in eField."""

    def __init__(self, loss_fn, hit_threshold=1e-8, collapsed=True, prob_target=False, **kwargs):
        super().__init__(**kwargs)
        self.loss_fn = loss_fn
        self.hit_threshold = hit_threshold
        self.collapsed = collapsed
        self.prob_target = prob_target

    def _generate_distribution_hits(self, params, output):
        from .losses import adc2charge
        tp = torch.as_tensor(output["hit_prob"])
        ad = torch.as_tensor(output["adcs_distrib"]).to(tp.device)
        P, H, T = tp.shape
        mask = tp > self.hit_threshold
        hit_prob = tp[mask]
        Q = adc2charge(ad[mask], params)
        ticks = torch.arange(T, dtype=torch.float32, device=tp.device).expand(P, H, T)[mask]
        if "pixel_z" in output:
            pred_z = output["pixel_z"]
        else:
            plane = _dev_tensor(output.get("pixel_plane"), torch.int32, tp.device)
            pred_z = _hit_z(params, ticks, plane[:, None, None].expand(P, H, T)[mask], output.get("theta"))
        ev = _dev_tensor(output["event"], torch.int32, tp.device)[:, None, None].expand(P, H, T)[mask]
        x = _dev_tensor(output["pixel_x"], torch.float32, tp.device)[:, None, None].expand(P, H, T)[mask]
        y = _dev_tensor(output["pixel_y"], torch.float32, tp.device)[:, None, None].expand(P, H, T)[mask]
        return Q, x, y, pred_z, ticks, hit_prob, ev

    def _prepare_probabilistic_output(self, params, output):
        from .losses import adc2charge
        tp = torch.as_tensor(output["hit_prob"])
        ad = torch.as_tensor(output["adcs_distrib"]).to(tp.device)
        e_tick, e_adc, hit_prob = sim.get_average_hit_values(tp, ad)
        P, H, _ = tp.shape
        Q = adc2charge(e_adc, params)
        if "pixel_z" in output:
            pred_z = output["pixel_z"]
        else:
            plane = _dev_tensor(output.get("pixel_plane"), torch.int32, tp.device)
            pred_z = _hit_z(params, e_tick, plane[:, None].expand(P, H), output.get("theta"))
        ev = _dev_tensor(output["event"], torch.int32, tp.device)[:, None].expand(P, H)
        x = _dev_tensor(output["pixel_x"], torch.float32, tp.device)[:, None].expand(P, H)
        y = _dev_tensor(output["pixel_y"], torch.float32, tp.device)[:, None].expand(P, H)
        return Q, x, y, pred_z, e_tick, hit_prob, ev

    def compute(self, params, prediction, target):
        from .losses import adc2charge
        if self.prob_target:
            ref = self._prepare_probabilistic_output(params, target)
        else:
            ticks = torch.as_tensor(target["ticks"])
            ref_event = target.get("event", torch.zeros_like(ticks, dtype=torch.int32))
            ref_hp = target.get("hit_prob", torch.ones_like(ticks))
            ref = (adc2charge(target["adcs"], params), target["pixel_x"], target["pixel_y"], target["pixel_z"],
                   ticks, ref_hp, ref_event)
        if self.collapsed:
            pred = self._prepare_probabilistic_output(params, prediction)
        else:
            pred = self._generate_distribution_hits(params, prediction)
        flat = lambda t: torch.as_tensor(t).reshape(-1)   # noqa: E731
        return self.loss_fn(params, *(flat(t) for t in pred), *(flat(t) for t in ref), **self.kwargs)


class _ProbLlhdFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, log_prob, adcs, lp, sim_pixels, tgt_pix, tgt_tick, tgt_adc, sigma_charge, eps):
        from . import _abi
        lib = _abi.load()
        P, H, T = log_prob.shape
        n = tgt_pix.shape[0]
        ws = torch.empty(max(lib.lsim_prob_llhd_workspace_bytes(n), 1), dtype=torch.uint8, device=log_prob.device)
        out = torch.empty(4, dtype=torch.float32, device=log_prob.device)
        p = sim._ptr
        _abi.check(lib, lib.lsim_prob_llhd(lp, p(sim_pixels), P, H, T, p(log_prob), p(adcs), p(tgt_pix),
                                           p(tgt_tick), p(tgt_adc), n, float(sigma_charge), float(eps), None,
                                           p(out), None, None, p(ws), ws.numel(), sim._stream()))
        ctx.save_for_backward(log_prob, adcs, sim_pixels, tgt_pix, tgt_tick, tgt_adc)
        ctx.lp, ctx.sigma, ctx.eps = lp, sigma_charge, eps
        aux = out[1:].clone()
        ctx.mark_non_differentiable(aux)
        return out[0].clone(), aux

    @staticmethod
    def backward(ctx, g, _g_aux):
        from . import _abi
        lib = _abi.load()
        log_prob, adcs, sim_pixels, tgt_pix, tgt_tick, tgt_adc = ctx.saved_tensors
        P, H, T = log_prob.shape
        n = tgt_pix.shape[0]
        ws = torch.empty(max(lib.lsim_prob_llhd_workspace_bytes(n), 1), dtype=torch.uint8, device=log_prob.device)
        out = torch.empty(4, dtype=torch.float32, device=log_prob.device)
        g_lp = torch.empty_like(log_prob) if ctx.needs_input_grad[0] else None
        g_ad = torch.empty_like(adcs) if ctx.needs_input_grad[1] else None
        gl = g.detach().to(torch.float32).reshape(1).contiguous()
        p = sim._ptr
        _abi.check(lib, lib.lsim_prob_llhd(ctx.lp, p(sim_pixels), P, H, T, p(log_prob), p(adcs), p(tgt_pix),
                                           p(tgt_tick), p(tgt_adc), n, float(ctx.sigma), float(ctx.eps), p(gl),
                                           p(out), p(g_lp), p(g_ad), p(ws), ws.numel(), sim._stream()))
        return g_lp, g_ad, *(None,) * 7


class ProbabilisticLossStrategy(LossStrategy):
    """strategies.py:338-567: the negative log-likelihood of the target hits
    under the probabilistic front end's distributions.  Target hits
    (``pixel_id``, ``ticks``, ``adcs``) are matched to the prediction's
    sorted ``unique_pixels``; the k-th hit of a pixel reads hit row k of
    ``hit_prob`` (log-probabilities) and ``adcs_distrib`` at its tick.
    loss = sqrt(T * C) with T the tick log-likelihood (clamped at log(eps),
    log(eps) per unmatched hit) and C the Gaussian charge log-likelihood of
    width sigma_charge / 1000 ke-.  Returns (loss, aux) with the reference's
    aux keys; the loss is differentiable with respect to both distributions
    (lsim_prob_llhd)."""

    def __init__(self, sigma_charge=500.0, eps=1e-10, **kwargs):
        super().__init__(**kwargs)
        self.sigma_charge = sigma_charge
        self.eps = eps

    def compute(self, params, prediction, target):
        from . import _abi
        lp_dist = torch.as_tensor(prediction["hit_prob"], dtype=torch.float32)
        dev = lp_dist.device if lp_dist.is_cuda else sim._device()
        lp_dist = lp_dist.to(dev).contiguous()
        ad = torch.as_tensor(prediction["adcs_distrib"], dtype=torch.float32).to(dev).contiguous()
        if lp_dist.dim() != 3 or ad.shape != lp_dist.shape:
            raise ValueError(f"hit_prob {tuple(lp_dist.shape)} and adcs_distrib {tuple(ad.shape)} must be the "
                             "same (pixels, hits, ticks) shape")
        sim_pixels = _dev_tensor(prediction["unique_pixels"], torch.int32, dev).reshape(-1)
        if sim_pixels.shape[0] != lp_dist.shape[0]:
            raise ValueError("unique_pixels needs one id per distribution row")
        tgt_pix = _dev_tensor(target["pixel_id"], torch.int32, dev).reshape(-1)
        tgt_tick = _dev_tensor(target["ticks"], torch.int32, dev).reshape(-1)   # .astype(int): truncation
        tgt_adc = _dev_tensor(target["adcs"], torch.float32, dev).reshape(-1)
        if not (tgt_pix.shape[0] == tgt_tick.shape[0] == tgt_adc.shape[0]):
            raise ValueError("target pixel_id, ticks and adcs need one entry per hit")
        loss, aux = _ProbLlhdFn.apply(lp_dist, ad, _abi.make_params(params), sim_pixels, tgt_pix, tgt_tick, tgt_adc,
                                      self.sigma_charge, self.eps)
        return loss, {"log_likelihood_charge": aux[0], "log_likelihood_tick": aux[1], "no_match_penalty": aux[2]}
