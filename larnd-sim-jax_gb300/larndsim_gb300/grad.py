"""Forward + adjoint of the LUT-mode chain with respect to the physics
parameters (Ab, kb, eField, lifetime, vdrift, long_diff, tran_diff,
lArDensity).

The reference differentiates ``simulate_wfs`` + ``simulate_stochastic`` with
``jax.value_and_grad`` (optimize/fit_params.py:704, :731).  Here the adjoint
is hand-written: the backward kernel recomputes each pixel's waveform and
front-end state instead of storing waveforms, then pushes dL/dADC back
through the self-trigger (crossing indices and clamps carry no gradient,
exactly as in JAX), the sub-tick split, the long-diffusion template
interpolation, the transverse bin weights, lifetime, recombination and the
drift velocity.  ``d/d vdrift`` is identically zero, as in the reference,
where ``params.vdrift`` is never read (drift velocity is
``get_vdrift(eField, temperature)``).

``LUTChain`` holds one batch of tracks; ``loss_and_grad`` evaluates the
sum-of-squared-ADC loss against a target on the (pixel id x hit) grid
(pixels absent from one side count as no-hit, i.e. digitize(0)).
``adc_fn`` wraps the chain as a ``torch.autograd.Function``.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _abi, sim

GRAD_PARAMS = _abi.GRAD_PARAMS


class Target:
    """ADC grid of a reference simulation: ascending pixel ids + (P, H) ADCs."""

    def __init__(self, pids: torch.Tensor, adc: torch.Tensor):
        self.pids = pids.to(torch.int32).contiguous()
        self.adc = adc.to(torch.float32).contiguous()


class LUTChain:
    """Fused LUT-mode forward/adjoint over one batch of tracks."""

    def __init__(self, params, response_template, tracks, fields, n_events=None):
        self.lut = sim.prepare_lut(response_template, params)
        self.fields = tuple(fields)
        self.tracks = sim.as_tracks(tracks)
        ev = self.tracks[:, self.fields.index("eventID")]
        self.n_events = int(ev.max().item()) + 1 if n_events is None else int(n_events)
        self.H = int(params.MAX_ADC_VALUES)
        self.lib = _abi.load()
        self._stage = None

    def stage1(self, params):
        lp = _abi.make_params(params, self.lut.shape)
        st = sim.run_stage1(params, self.tracks, self.fields, lp, n_events=self.n_events)
        self._stage = st
        return st

    def _check(self, st):
        st.raise_status()
        return st.n_valid

    def adc(self, params, normals=None):
        """ADC and tick grids (n_valid, H) and the valid pixel ids."""
        st = self.stage1(params)
        n_valid = self._check(st)
        dev = self.tracks.device
        adc = torch.empty((n_valid, self.H), dtype=torch.float32, device=dev)
        ticks = torch.empty((n_valid, self.H), dtype=torch.float32, device=dev)
        pids = torch.empty((n_valid,), dtype=torch.int32, device=dev)
        s = sim._stream()
        _abi.check(self.lib, self.lib.lsim_valid_pixels(st.lp, sim._ptr(st.ws), st.n_rows, st.n_events, n_valid,
                                                        sim._ptr(pids), s))
        _abi.check(self.lib, self.lib.lsim_lut_adc(st.lp, sim._ptr(self.lut.tables), sim._ptr(st.ws), st.n_rows,
                                                   st.n_events, n_valid, sim._ptr(normals), sim._ptr(adc),
                                                   sim._ptr(ticks), s))
        return adc, ticks, pids

    def target(self, params, normals=None) -> Target:
        adc, _, pids = self.adc(params, normals)
        return Target(pids, adc)

    def _grad(self, params, g_adc=None, target=None, normals=None, adc_out=None, sync=True, events=None):
        st = self.stage1(params)
        n_valid = self._check(st) if sync else None
        dev = self.tracks.device
        out = torch.empty(1 + _abi.NPARAM, dtype=torch.float32, device=dev)
        tp = target.pids if target is not None else None
        ta = target.adc if target is not None else None
        nt = target.pids.shape[0] if target is not None else 0
        if events is not None:
            events[0].record()
        _abi.check(self.lib, self.lib.lsim_lut_grad(
            st.lp, sim._ptr(self.lut.tables), sim._ptr(st.ws), st.n_rows, st.n_events,
            n_valid if n_valid is not None else 0, sim._ptr(normals), sim._ptr(g_adc), sim._ptr(tp), sim._ptr(ta), nt,
            sim._ptr(out), sim._ptr(out[1:]), sim._ptr(adc_out), sim._stream()))
        if events is not None:
            events[1].record()
        return out

    def loss_and_grad(self, params, target: Target, normals=None):
        """SSE loss against ``target`` and its gradient (dict by parameter)."""
        out = self._grad(params, target=target, normals=normals)
        vals = out.cpu().numpy()
        return float(vals[0]), dict(zip(GRAD_PARAMS, vals[1:].tolist()))

    def loss_and_grad_stored(self, params, target: Target, normals=None):
        """``loss_and_grad`` through the store-the-waveforms variant: a
        simulate_wfs pass writes the (n_valid, n_ticks - 1) waveforms, and
        the adjoint reads them back instead of recomputing them.  Returns
        (loss, gradient dict, waveforms)."""
        st = self.stage1(params)
        n_valid = self._check(st)
        dev = self.tracks.device
        T = int(st.lp.n_ticks) - 1
        wfs = torch.empty((n_valid, T), dtype=torch.float32, device=dev)
        unique = torch.empty((n_valid,), dtype=torch.int32, device=dev)
        s = sim._stream()
        _abi.check(self.lib, self.lib.lsim_lut_stage2(st.lp, sim._ptr(self.lut.tables), sim._ptr(st.ws), st.n_rows,
                                                      st.n_events, n_valid, 0, n_valid, sim._ptr(wfs),
                                                      sim._ptr(unique), s))
        out = torch.empty(1 + _abi.NPARAM, dtype=torch.float32, device=dev)
        _abi.check(self.lib, self.lib.lsim_lut_grad_stored(
            st.lp, sim._ptr(self.lut.tables), sim._ptr(st.ws), st.n_rows, st.n_events, sim._ptr(wfs), n_valid,
            n_valid, sim._ptr(normals), None, sim._ptr(target.pids), sim._ptr(target.adc), target.pids.shape[0],
            sim._ptr(out), sim._ptr(out[1:]), None, s))
        vals = out.cpu().numpy()
        return float(vals[0]), dict(zip(GRAD_PARAMS, vals[1:].tolist())), wfs

    def loss_and_grad_device(self, params, target: Target, normals=None, events=None):
        """Like ``loss_and_grad`` but returns the device tensor [loss, grads...]
        without a host synchronisation.  ``events`` (start, end) CUDA events,
        if given, bracket the lsim_lut_grad call (all gradient kernels)."""
        return self._grad(params, target=target, normals=normals, sync=False, events=events)

    def capture(self, params, target: Target, normals=None):
        """One loss-and-gradient step at fixed ``params`` (stage 1, forward,
        adjoint) captured in a CUDA graph; returns (graph, output tensor
        [loss, grads...] that every replay rewrites).  Nothing in the step
        waits for the host, so replays run back to back."""
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.loss_and_grad_device(params, target, normals=normals)
        torch.cuda.current_stream().wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            out = self.loss_and_grad_device(params, target, normals=normals)
        return g, out

    def set_tracks(self, tracks):
        """Replace the batch (same shape); host tensors are copied asynchronously."""
        src = torch.as_tensor(tracks)
        if tuple(src.shape) != tuple(self.tracks.shape):
            raise ValueError("set_tracks needs the shape of the original batch")
        self.tracks.copy_(src, non_blocking=True)

    def wfs(self, params):
        """simulate_wfs at params on this chain's tracks: (wfs (P_pad, T),
        unique_pixels (P_pad,)), rows as the reference orders them."""
        st = self.stage1(params)
        st.raise_status()
        p_unique = st.n_em1 + st.n_valid + st.any_m1 + 1
        p_pad = sim.pad_size(p_unique, "unique_pixels", 0.2)
        T = int(st.lp.n_ticks) - 1
        dev = self.tracks.device
        wfs = torch.empty((p_pad, T), dtype=torch.float32, device=dev)
        unique = torch.empty((p_pad,), dtype=torch.int32, device=dev)
        _abi.check(self.lib, self.lib.lsim_lut_stage2(st.lp, sim._ptr(self.lut.tables), sim._ptr(st.ws), st.n_rows,
                                                      st.n_events, p_pad, st.n_em1, st.n_valid, sim._ptr(wfs),
                                                      sim._ptr(unique), sim._stream()))
        return wfs, unique

    def wfs_vjp(self, params, g_wfs: torch.Tensor):
        """dL/dtheta for a cotangent on the waveforms ``wfs`` returns (same
        shape; rows with a negative pixel id carry no gradient)."""
        st = self.stage1(params)
        n_valid = self._check(st)
        g = g_wfs.to(device=self.tracks.device, dtype=torch.float32).contiguous()
        out = torch.empty(_abi.NPARAM, dtype=torch.float32, device=self.tracks.device)
        _abi.check(self.lib, self.lib.lsim_lut_wfs_vjp(st.lp, sim._ptr(self.lut.tables), sim._ptr(st.ws), st.n_rows,
                                                       st.n_events, sim._ptr(g), g.shape[0], n_valid, sim._ptr(out),
                                                       sim._stream()))
        return out

    def vjp(self, params, g_adc: torch.Tensor, normals=None):
        """dL/dtheta for a given cotangent on the (n_valid, H) ADC grid."""
        g = g_adc.to(torch.float32).contiguous()
        out = self._grad(params, g_adc=g, normals=normals)
        return out[1:]


class _AdcFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, chain, params, normals):
        vals = theta.detach().cpu().numpy().astype(np.float64)
        p = params.replace(**{k: float(v) for k, v in zip(GRAD_PARAMS, vals)})
        adc, ticks, pids = chain.adc(p, normals)
        ctx.chain, ctx.params, ctx.normals = chain, p, normals
        ctx.theta_device, ctx.theta_dtype = theta.device, theta.dtype
        ctx.mark_non_differentiable(ticks, pids)
        return adc, ticks, pids

    @staticmethod
    def backward(ctx, g_adc, g_ticks, g_pids):
        if g_adc is None:
            return None, None, None, None
        grad = ctx.chain.vjp(ctx.params, g_adc, ctx.normals)
        return grad.to(device=ctx.theta_device, dtype=ctx.theta_dtype), None, None, None


class _WfsFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, chain, params):
        vals = theta.detach().cpu().numpy().astype(np.float64)
        p = params.replace(**{k: float(v) for k, v in zip(GRAD_PARAMS, vals)})
        wfs, unique = chain.wfs(p)
        ctx.chain, ctx.params = chain, p
        ctx.theta_device, ctx.theta_dtype = theta.device, theta.dtype
        ctx.mark_non_differentiable(unique)
        return wfs, unique

    @staticmethod
    def backward(ctx, g_wfs, g_unique):
        if g_wfs is None:
            return None, None, None
        grad = ctx.chain.wfs_vjp(ctx.params, g_wfs)
        return grad.to(device=ctx.theta_device, dtype=ctx.theta_dtype), None, None


def wfs_fn(theta: torch.Tensor, chain: LUTChain, params):
    """Differentiable simulate_wfs (sim_jax.py:689-736) as a function of
    ``theta`` = the 8 parameter values (order ``GRAD_PARAMS``): returns
    (wfs, unique_pixels); backward runs lsim_lut_wfs_vjp."""
    return _WfsFn.apply(theta, chain, params)


def lut_value_and_grad(params, response_template, tracks, fields, target: Target, n_events=None):
    """Loss and gradient of one fit step through the public API.

    Mirrors the reference's ``value_and_grad(loss_wrapper)`` over
    LUTSimulation.predict (optimize/fit_params.py:704-731) for the SSE-ADC
    loss: ``tracks`` may live on the host (copied to the device here); the
    result comes back to the host.  Returns (loss, {param: dL/dparam}).
    """
    chain = LUTChain(params, response_template, tracks, fields, n_events=n_events)
    return chain.loss_and_grad(params, target)


def theta_of(params, device=None) -> torch.Tensor:
    """The 8 differentiable parameter values as a float64 tensor."""
    return torch.tensor([float(getattr(params, k)) for k in GRAD_PARAMS], dtype=torch.float64, device=device)


def adc_fn(theta: torch.Tensor, chain: LUTChain, params, normals=None):
    """Differentiable (ADC, ticks, pixel ids) of the LUT chain as a function
    of ``theta`` = the 8 parameter values (order ``GRAD_PARAMS``)."""
    return _AdcFn.apply(theta, chain, params, normals)


def _hit_z(params, theta, ticks, plane):
    """get_hit_z (detsim_jax.py:309-319) with the drift velocity of theta's
    eField: z_anode + tick * t_sampling * v * sign(z_high - z_anode); the
    value uses get_vdrift in float64 rounded to float32, the derivative
    d v / d eField (the reference differentiates get_vdrift)."""
    from .consts import get_vdrift, get_vdrift_derivative
    e = theta[GRAD_PARAMS.index("eField")]
    pe = params.replace(eField=float(e.detach()))
    v = torch.tensor(np.float32(get_vdrift(pe)), dtype=torch.float32, device=ticks.device)
    v = v + (e - e.detach()).to(torch.float32) * float(get_vdrift_derivative(pe))
    b = torch.as_tensor(np.asarray(params.tpc_borders, np.float32), device=ticks.device)[plane.long()]
    za, zh = b[..., 2, 0], b[..., 2, 1]
    return za + ticks * (np.float32(params.t_sampling) * v) * torch.sign(zh - za)


def predicted_hits(theta, chain, params, normals=None):
    """The accepted hits of the LUT chain at theta (simulate_stochastic's
    compaction, sim_jax.py:757-769 and :619-647), differentiable in theta:
    (Q, x, y, z, ticks, hit_prob, event)."""
    from . import losses
    from .consts import n_ticks
    adc, ticks, pids = adc_fn(theta, chain, params, normals)
    T = n_ticks(params) - 1
    keep = (ticks < T - 3).reshape(-1)
    H = adc.shape[1]
    x, y, plane, event = sim.pixel_coordinates(params, pids)
    rep = lambda t: t.repeat_interleave(H)[keep]   # noqa: E731
    t_k = ticks.reshape(-1)[keep]
    z = _hit_z(params, theta, t_k, rep(plane))
    Q = losses.adc2charge(adc.reshape(-1)[keep], params)
    return Q, rep(x), rep(y), z, t_k, torch.ones_like(t_k), rep(event)


def params_loss(params, chain, ref, loss_fn=None, theta=None, normals=None, **loss_kwargs):
    """params_loss (losses_jax.py:385-398) for the LUT chain with a hit-level
    loss: simulate at ``theta`` (default: params' values), build the hits,
    and evaluate ``loss_fn`` (default mse_adc) against ``ref`` = (ref_Q,
    ref_x, ref_y, ref_z, ref_ticks, ref_hit_prob, ref_event).  Returns
    (loss, aux, theta); ``loss.backward()`` fills theta.grad through the
    loss kernel, the hit z and the LUT adjoint."""
    from . import losses
    loss_fn = losses.mse_adc if loss_fn is None else loss_fn
    if theta is None:
        theta = theta_of(params, device=chain.tracks.device).requires_grad_(True)
    Q, x, y, z, t, hp, ev = predicted_hits(theta, chain, params, normals)
    loss, aux = loss_fn(params, Q, x, y, z, t, hp, ev, *ref, **loss_kwargs)
    return loss, aux, theta
