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
