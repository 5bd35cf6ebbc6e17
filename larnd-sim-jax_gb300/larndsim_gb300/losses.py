"""Loss-side helpers (reference: src/larndsim/losses_jax.py)."""

from __future__ import annotations

import numpy as np
import torch


def adc2charge(dw, params):
    """Charge in ke- from ADC counts (losses_jax.py:380-383)."""
    x = torch.as_tensor(dw, dtype=torch.float32)
    return ((((x / np.float32(params.ADC_COUNTS)) * np.float32(params.V_REF - params.V_CM))
             + np.float32(params.V_CM)) - np.float32(params.V_PEDESTAL)) / np.float32(params.GAIN) * np.float32(1e-3)


def _f32(t, device):
    return torch.as_tensor(t).to(device=device, dtype=torch.float32).contiguous()


def _i32(t, device):
    return torch.as_tensor(t).to(device=device, dtype=torch.int32).contiguous()


class _MseAdcFn(torch.autograd.Function):
    """mse_adc on weights and z with the gradient from lsim_mse_adc."""

    @staticmethod
    def forward(ctx, w, z, x, y, event, rw, rx, ry, rz, revent, sigma, lambda_q):
        from . import _abi, sim
        lib = _abi.load()
        dev = w.device
        n, m = w.shape[0], rw.shape[0]
        ws = torch.empty(max(lib.lsim_mse_adc_workspace_bytes(n, m), 1), dtype=torch.uint8, device=dev)
        out = torch.empty(4, dtype=torch.float32, device=dev)
        need = ctx.needs_input_grad[0] or ctx.needs_input_grad[1]
        gw = torch.empty(n, dtype=torch.float32, device=dev) if need else None
        gz = torch.empty(n, dtype=torch.float32, device=dev) if need else None
        p = sim._ptr
        _abi.check(lib, lib.lsim_mse_adc(p(x), p(y), p(z), p(event), p(w), n, p(rx), p(ry), p(rz), p(revent), p(rw), m,
                                         float(sigma), float(lambda_q), p(out), p(gw), p(gz), p(ws), ws.numel(),
                                         sim._stream()))
        ctx.save_for_backward(*(t for t in (gw, gz) if t is not None))
        ctx.has_grad = need
        ctx.mark_non_differentiable(out)
        return out[0].clone(), out

    @staticmethod
    def backward(ctx, g, _g_out):
        if not ctx.has_grad or g is None:
            return (None,) * 12
        gw, gz = ctx.saved_tensors
        return g * gw, g * gz, *(None,) * 10


def mse_adc(params, Q, x, y, z, ticks, hit_prob, event, ref_Q, ref_x, ref_y, ref_z, ref_ticks, ref_hit_prob,
            ref_event, sigma=1, lambda_Q=1):
    """losses_jax.py:60-79: the weighted RBF maximum mean discrepancy between
    predicted and reference hits on (x + event * 1e5, y, z), weights
    Q * hit_prob, plus lambda_Q times the squared relative difference of the
    total weights.  Returns (loss, aux) like the reference; the loss is a
    0-d CUDA tensor, differentiable with respect to Q, hit_prob and z."""
    Q = torch.as_tensor(Q, dtype=torch.float32)
    dev = Q.device if Q.is_cuda else torch.device("cuda", torch.cuda.current_device())
    Q = Q.to(dev)
    hp = torch.as_tensor(hit_prob, dtype=torch.float32).to(dev)
    rQ, rhp = _f32(ref_Q, dev), _f32(ref_hit_prob, dev)
    w = (Q * hp).contiguous()
    v = (rQ * rhp).contiguous()
    zt = torch.as_tensor(z, dtype=torch.float32).to(dev).contiguous()
    loss, parts = _MseAdcFn.apply(w, zt, _f32(x, dev), _f32(y, dev), _i32(event, dev), v, _f32(ref_x, dev),
                                  _f32(ref_y, dev), _f32(ref_z, dev), _i32(ref_event, dev), float(sigma),
                                  float(lambda_Q))
    aux = {"charge_loss": parts[2], "mmd_loss_term": parts[1], "Q": Q, "ref_Q": rQ, "ref_hit_prob": rhp,
           "hit_prob": hp}
    return loss, aux


class _NllFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q, z, hp, x, y, event, rq, rx, ry, rz, revent, rhp, sigma):
        from . import _abi, sim
        lib = _abi.load()
        dev = q.device
        n, m = q.shape[0], rq.shape[0]
        ws = torch.empty(max(lib.lsim_nll_workspace_bytes(n, m), 1), dtype=torch.uint8, device=dev)
        out = torch.empty(4, dtype=torch.float32, device=dev)
        grads = [torch.empty(n, dtype=torch.float32, device=dev) for _ in range(3)]
        p = sim._ptr
        _abi.check(lib, lib.lsim_nll_loss(p(x), p(y), p(z), p(q), p(event), p(hp), n, p(rx), p(ry), p(rz), p(rq),
                                          p(revent), p(rhp), m, float(sigma), p(out), *(p(g) for g in grads), p(ws),
                                          ws.numel(), sim._stream()))
        ctx.save_for_backward(*grads)
        ctx.mark_non_differentiable(out)
        return out[0].clone(), out

    @staticmethod
    def backward(ctx, g, _g_out):
        gq, gz, ghp = ctx.saved_tensors
        return g * gq, g * gz, g * ghp, *(None,) * 10


def nll_loss(params, Q, x, y, z, ticks, hit_prob, event, ref_Q, ref_x, ref_y, ref_z, ref_ticks, ref_hit_prob,
             ref_event, adc_norm=10., sigma=1., match_z=False):
    """losses_jax.py:329-359: negative log-likelihood of the reference hits
    under the Gaussian intensity of the predicted hits on
    (x + event * 1e9, y, z, Q / adc_norm).  Returns (loss, {}); the loss is
    differentiable with respect to Q, z and hit_prob."""
    from .sim import pad_size
    Q = torch.as_tensor(Q, dtype=torch.float32)
    dev = Q.device if Q.is_cuda else torch.device("cuda", torch.cuda.current_device())
    Q = Q.to(dev)
    pad_size((len(ref_Q), Q.shape[0]), "nll_loss")   # the reference's size history (padding adds nothing)
    q = (Q / np.float32(adc_norm)).contiguous()
    rq = (_f32(ref_Q, dev) / np.float32(adc_norm)).contiguous()
    hp = torch.as_tensor(hit_prob, dtype=torch.float32).to(dev).contiguous()
    zt = torch.as_tensor(z, dtype=torch.float32).to(dev).contiguous()
    loss, _ = _NllFn.apply(q, zt, hp, _f32(x, dev), _f32(y, dev), _i32(event, dev), rq, _f32(ref_x, dev),
                           _f32(ref_y, dev), _f32(ref_z, dev), _i32(ref_event, dev), _f32(ref_hit_prob, dev),
                           float(sigma))
    return loss, dict()


class _ChamferFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, w, z, x, y, event, rw, rx, ry, rz, revent):
        from . import _abi, sim
        lib = _abi.load()
        dev = w.device
        n, m = w.shape[0], rw.shape[0]
        ws = torch.empty(max(lib.lsim_chamfer_workspace_bytes(n, m), 1), dtype=torch.uint8, device=dev)
        out = torch.empty(4, dtype=torch.float32, device=dev)
        gw = torch.empty(n, dtype=torch.float32, device=dev)
        gz = torch.empty(n, dtype=torch.float32, device=dev)
        p = sim._ptr
        _abi.check(lib, lib.lsim_chamfer_3d(p(x), p(y), p(z), p(event), p(w), n, p(rx), p(ry), p(rz), p(revent),
                                            p(rw), m, p(out), p(gw), p(gz), p(ws), ws.numel(), sim._stream()))
        ctx.save_for_backward(gw, gz)
        ctx.mark_non_differentiable(out)
        return out[0].clone(), out

    @staticmethod
    def backward(ctx, g, _g_out):
        gw, gz = ctx.saved_tensors
        return g * gw, g * gz, *(None,) * 8


def _pad(t, n, value=0):
    if t.shape[0] >= n:
        return t
    return torch.cat([t, torch.full((n - t.shape[0],), value, dtype=t.dtype, device=t.device)])


def chamfer_3d(params, Q, x, y, z, ticks, hit_prob, event, ref_Q, ref_x, ref_y, ref_z, ref_ticks, ref_hit_prob,
               ref_event, adc_norm=10., match_z=False):
    """losses_jax.py:213-229: nearest-neighbour (Chamfer) distance between
    predicted and reference hits on (x + event * 1e9, y, z), weighted by
    Q / adc_norm, with both sets zero-padded to pad_size's buckets as the
    reference pads them.  Returns (loss, {}); differentiable with respect
    to Q and z."""
    from .sim import pad_size
    Q = torch.as_tensor(Q, dtype=torch.float32)
    dev = Q.device if Q.is_cuda else torch.device("cuda", torch.cuda.current_device())
    Q = Q.to(dev)
    n, m = Q.shape[0], len(ref_Q)
    new_ref, new_cur = pad_size((m, n), "chamfer_3d")
    w = _pad(Q / np.float32(adc_norm), new_cur).contiguous()
    rw = _pad(_f32(ref_Q, dev) / np.float32(adc_norm), new_ref).contiguous()
    zt = _pad(torch.as_tensor(z, dtype=torch.float32).to(dev), new_cur).contiguous()
    loss, _ = _ChamferFn.apply(w, zt, _pad(_f32(x, dev), new_cur).contiguous(), _pad(_f32(y, dev), new_cur).contiguous(),
                               _pad(_i32(event, dev), new_cur).contiguous(), rw,
                               _pad(_f32(ref_x, dev), new_ref).contiguous(), _pad(_f32(ref_y, dev), new_ref).contiguous(),
                               _pad(_f32(ref_z, dev), new_ref).contiguous(),
                               _pad(_i32(ref_event, dev), new_ref).contiguous())
    return loss, dict()


class _LlhdFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, tpd, nohit, cd, cm, ticks, sigma):
        from . import _abi, sim
        lib = _abi.load()
        n, t = tpd.shape
        ws = torch.empty(max(lib.lsim_llhd_workspace_bytes(n), 1), dtype=torch.uint8, device=tpd.device)
        out = torch.empty(1, dtype=torch.float32, device=tpd.device)
        p = sim._ptr
        _abi.check(lib, lib.lsim_llhd_loss(p(tpd), p(ticks), p(nohit), p(cd), p(cm), n, t, float(sigma), None,
                                           p(out), None, None, None, None, p(ws), ws.numel(), sim._stream()))
        ctx.save_for_backward(tpd, nohit, cd, cm, ticks)
        ctx.sigma = sigma
        return out[0]

    @staticmethod
    def backward(ctx, g):
        from . import _abi, sim
        lib = _abi.load()
        tpd, nohit, cd, cm, ticks = ctx.saved_tensors
        n, t = tpd.shape
        ws = torch.empty(max(lib.lsim_llhd_workspace_bytes(n), 1), dtype=torch.uint8, device=tpd.device)
        out = torch.empty(1, dtype=torch.float32, device=tpd.device)
        g_t, g_c = torch.empty_like(tpd), torch.empty_like(cd)
        g_nh, g_cm = torch.empty_like(nohit), torch.empty_like(cm)
        gl = g.detach().to(torch.float32).reshape(1).contiguous()
        p = sim._ptr
        _abi.check(lib, lib.lsim_llhd_loss(p(tpd), p(ticks), p(nohit), p(cd), p(cm), n, t, float(ctx.sigma), p(gl),
                                           p(out), p(g_t), p(g_nh), p(g_c), p(g_cm), p(ws), ws.numel(),
                                           sim._stream()))
        return g_t, g_nh, g_c, g_cm, None, None


def llhd_loss(ticks_prob_distrib, ticks_mc, no_hit_prob, charge_distrib, charge_mc, sigma=500):
    """losses_jax.py:414-441: the negative log-likelihood of observed hit
    ticks and charges under per-row tick distributions (N, T): log(p[tick]
    + 1e-10), or log(no_hit_prob + 1e-10) where tick >= T - 3, plus a
    Gaussian charge term of width ``sigma`` at the distribution's charge.
    Returns (loss, {}); the loss is differentiable with respect to the four
    float inputs (lsim_llhd_loss)."""
    tpd = torch.as_tensor(ticks_prob_distrib, dtype=torch.float32)
    dev = tpd.device if tpd.is_cuda else torch.device("cuda", torch.cuda.current_device())
    tpd = tpd.to(dev).contiguous()
    if tpd.dim() != 2:
        raise ValueError(f"ticks_prob_distrib must be (rows, ticks), got {tuple(tpd.shape)}")
    cd = torch.as_tensor(charge_distrib, dtype=torch.float32).to(dev).contiguous()
    if cd.shape != tpd.shape:
        raise ValueError(f"charge_distrib {tuple(cd.shape)} does not match ticks_prob_distrib {tuple(tpd.shape)}")
    nohit = torch.as_tensor(no_hit_prob, dtype=torch.float32).to(dev).reshape(-1).contiguous()
    cm = torch.as_tensor(charge_mc, dtype=torch.float32).to(dev).reshape(-1).contiguous()
    ticks = _i32(torch.as_tensor(ticks_mc), dev)
    if not (nohit.shape[0] == cm.shape[0] == ticks.shape[0] == tpd.shape[0]):
        raise ValueError("ticks_mc, no_hit_prob and charge_mc need one entry per row")
    return _LlhdFn.apply(tpd, nohit, cd, cm, ticks, sigma), dict()
