"""Device-resident fit of the physics parameters: the reference's
GradientDescentFitter step (optimize/fit_params.py:704-731 the loss and its
gradient with respect to the normalised parameters, :781-895 the optax
chain and process_grads, :168-199 the normalisation schemes).

One step is: the segment stage with the fit parameters read from device
memory (``lsim_lut_stage1_theta``), the forward + adjoint of the SSE-ADC
loss (``lsim_lut_grad``) and the optimiser update of the parameters in place
(``lsim_fit_step``: chain rule to the normalised parameters, NaN skip,
optional clip_by_global_norm, Adam, optional clip_values_from_range, map
back).  Nothing in a step needs the host, so the step is captured once in a
CUDA graph and replayed; the loss and the parameters of every step are
appended to device-side histories inside the graph.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _abi, sim
from .grad import GRAD_PARAMS, Target

# The reference's parameter ranges (optimize/ranges.py) for the parameters
# the gradient covers: nominal value, the soft range (down, up) used by
# clip_values_from_range, and the hard limits (min, max) of the sigmoid map.
RANGES = {
    "Ab": dict(nom=0.8, down=0.78, up=0.88, min=0.75, max=0.9),
    "kb": dict(nom=0.0486, down=0.04, up=0.07, min=0.03, max=0.08),
    "eField": dict(nom=0.5, down=0.45, up=0.55, min=0.4, max=0.6),
    "lifetime": dict(nom=2.2e3, down=500.0, up=5000.0, min=400.0, max=6000.0),
    "vdrift": dict(nom=0.1596, down=0.1400, up=0.1800, min=0.13, max=0.19),
    "long_diff": dict(nom=4.0e-6, down=2e-6, up=9e-6, min=1e-6, max=1e-5),
    "tran_diff": dict(nom=8.8e-6, down=4e-6, up=14e-6, min=3e-6, max=15e-6),
    "lArDensity": dict(nom=1.38, down=1.37, up=1.41, min=1.35, max=1.43),
}


def fit_options(fit_params, lr, initial, normalization_scheme="sigmoid", normalization_scale=1.0,
                max_clip_norm_val=None, clip_from_range=False, betas=(0.9, 0.999), eps=1e-8, ranges=None):
    """The LsimFitOptions block of one fit, with the reference's checks
    (fit_params.py:255-264, :168-199).  ``lr`` is one learning rate or a
    dict per parameter; ``initial`` the physical starting values (dict),
    which set the divide scheme's params_normalization (:443)."""
    if normalization_scheme not in _abi.NORM_SCHEMES:
        raise ValueError(f"Unknown normalization_scheme '{normalization_scheme}'. Use one of: sigmoid, exp_log, divide")
    scale = 1.0 if normalization_scheme == "divide" else float(normalization_scale)
    if scale <= 0:
        raise ValueError(f"normalization_scale_{normalization_scheme} must be > 0, got {normalization_scale}")
    unknown = set(fit_params) - set(GRAD_PARAMS)
    if unknown:
        raise ValueError(f"cannot fit {sorted(unknown)}; fit parameters are {GRAD_PARAMS}")
    rg = dict(RANGES, **(ranges or {}))
    o = _abi.LsimFitOptions()
    o.scheme = _abi.NORM_SCHEMES[normalization_scheme]
    o.fit_mask = sum(1 << GRAD_PARAMS.index(k) for k in fit_params)
    o.clip_from_range = int(bool(clip_from_range))
    o.norm_scale = scale
    o.max_clip_norm = float(max_clip_norm_val) if max_clip_norm_val is not None else 0.0
    o.beta1, o.beta2, o.eps = float(betas[0]), float(betas[1]), float(eps)
    for i, k in enumerate(GRAD_PARAMS):
        r = rg[k]
        o.lr[i] = (float(lr[k]) if isinstance(lr, dict) else float(lr)) if k in fit_params else 0.0
        o.lo[i], o.hi[i], o.nom[i], o.down[i], o.up[i] = r["min"], r["max"], r["nom"], r["down"], r["up"]
        v = float(initial[k])
        o.norm[i] = v if v != 0.0 else 1.0
        if k in fit_params and normalization_scheme == "exp_log" and r["nom"] <= 0:
            raise ValueError(f"exp_log normalization requires positive nominal value for '{k}', got {r['nom']}")
    return o


class DeviceFit:
    """The reference's gradient-descent fit (Adam) of ``fit_params`` (a
    subset of GRAD_PARAMS) against ``target``, with its normalisation
    schemes ("sigmoid", the reference's default; "exp_log"; "divide"),
    optional clip_by_global_norm (``max_clip_norm_val``) and
    clip_values_from_range (``clip_from_range``, divide scheme).  ``lr`` is
    the learning rate in normalised units, one value or a dict per
    parameter; ``normalization_scale`` is normalization_scale_sigmoid or
    normalization_scale_exp_log.

    The loss is the SSE of the ADC grids against ``target`` (the whole step
    on the device, capturable in one CUDA graph), or, with ``loss_fn`` (a
    hit-level loss of ``larndsim_gb300.losses`` such as ``mse_adc``, the
    reference fitter's default) and ``ref_hits`` = (ref_Q, ref_x, ref_y,
    ref_z, ref_ticks, ref_hit_prob, ref_event), that loss of the predicted
    hits as GenericLossStrategy forms them (strategies.py:161-180): the
    step then runs eagerly (the number of hits is read on the host), the
    gradient through the loss kernel, the hit z and the LUT adjoint.
    """

    def __init__(self, params, response_template, tracks, fields, target: Target = None, fit_params=None, lr=1e-2,
                 normalization_scheme="sigmoid", normalization_scale=1.0, max_clip_norm_val=None,
                 clip_from_range=False, betas=(0.9, 0.999), eps=1e-8, n_events=None, max_steps=1000, ranges=None,
                 loss_fn=None, ref_hits=None, loss_kwargs=None):
        if loss_fn is None and target is None:
            raise ValueError("DeviceFit needs a target (SSE loss) or loss_fn with ref_hits")
        if loss_fn is not None and ref_hits is None:
            raise ValueError("a hit-level loss_fn needs ref_hits")
        self.lib = _abi.load()
        self.lut = sim.prepare_lut(response_template, params)
        self.fields = tuple(fields)
        self.tracks = sim.as_tracks(tracks)
        dev = self.tracks.device
        ev = self.tracks[:, self.fields.index("eventID")]
        self.n_events = int(ev.max().item()) + 1 if n_events is None else int(n_events)
        self.n_rows = self.tracks.shape[0]
        self.lp = _abi.make_params(params, self.lut.shape)
        self.fm = _abi.field_map(self.fields)
        self.ws_bytes = self.lib.lsim_workspace_bytes(self.lp, self.n_rows, self.n_events)
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=dev)
        self.counts = torch.empty(16, dtype=torch.int32, device=dev)
        fit = tuple(fit_params) if fit_params is not None else tuple(k for k in GRAD_PARAMS if k != "vdrift")
        initial = {k: float(getattr(params, k)) for k in GRAD_PARAMS}
        self.opts = fit_options(fit, lr, initial, normalization_scheme, normalization_scale, max_clip_norm_val,
                                clip_from_range, betas, eps, ranges)
        self.theta = torch.tensor([initial[k] for k in GRAD_PARAMS], dtype=torch.float32, device=dev)
        self.state = torch.zeros(_abi.FIT_STATE, dtype=torch.float32, device=dev)
        self.out = torch.empty(1 + _abi.NPARAM, dtype=torch.float32, device=dev)
        self.target = target
        self.max_steps = int(max_steps)
        self.loss_hist = torch.zeros(self.max_steps, dtype=torch.float32, device=dev)
        self.theta_hist = torch.zeros((self.max_steps, _abi.NPARAM), dtype=torch.float32, device=dev)
        self.step_idx = torch.zeros(1, dtype=torch.int64, device=dev)
        self.graph = None
        self.params0 = params
        self.loss_fn, self.loss_kwargs = loss_fn, dict(loss_kwargs or {})
        self.ref_hits = tuple(ref_hits) if ref_hits is not None else None
        self.chain = None
        if loss_fn is not None:
            from . import grad
            self.chain = grad.LUTChain(params, self.lut, self.tracks, self.fields, n_events=self.n_events)
        _abi.check(self.lib, self.lib.lsim_fit_init(sim._ptr(self.theta), self.opts, sim._ptr(self.state),
                                                    sim._stream()))

    def _launch_hits(self):
        """One step with the hit-level loss: loss and dL/dtheta by autograd
        through the loss kernel and the LUT adjoint, then the update."""
        from . import grad
        theta = self.theta.detach().clone().requires_grad_(True)
        loss, _, _ = grad.params_loss(self.params0, self.chain, self.ref_hits, self.loss_fn, theta=theta,
                                      **self.loss_kwargs)
        loss.backward()
        self.out[0] = loss.detach()
        self.out[1:] = theta.grad
        idx = self.step_idx.clamp(max=self.max_steps - 1)
        self.loss_hist.index_copy_(0, idx, self.out[:1])
        self.theta_hist.index_copy_(0, idx, self.theta.unsqueeze(0))
        self.step_idx.add_(1)
        p = sim._ptr
        _abi.check(self.lib, self.lib.lsim_fit_step(p(self.theta), p(self.out[1:]), self.opts, p(self.state),
                                                    sim._stream()))

    def _launch(self):
        if self.loss_fn is not None:
            self._launch_hits()
            return
        s = sim._stream()
        lib, p = self.lib, sim._ptr
        _abi.check(lib, lib.lsim_lut_stage1_theta(self.lp, self.fm, p(self.tracks), self.n_rows, self.n_events,
                                                  p(self.theta), p(self.ws), self.ws_bytes, p(self.counts), s))
        t = self.target
        _abi.check(lib, lib.lsim_lut_grad(self.lp, p(self.lut.tables), p(self.ws), self.n_rows, self.n_events, 0,
                                          None, None, p(t.pids), p(t.adc), t.pids.shape[0], p(self.out),
                                          p(self.out[1:]), None, s))
        # history of the parameters the loss was evaluated at, then the update
        idx = self.step_idx.clamp(max=self.max_steps - 1)
        self.loss_hist.index_copy_(0, idx, self.out[:1])
        self.theta_hist.index_copy_(0, idx, self.theta.unsqueeze(0))
        self.step_idx.add_(1)
        _abi.check(lib, lib.lsim_fit_step(p(self.theta), p(self.out[1:]), self.opts, p(self.state), s))

    def step(self):
        """One eager step (no graph)."""
        self._launch()

    def capture(self):
        """Capture one step in a CUDA graph (a warm-up step runs first and is
        undone, so the trajectory starts from the current parameters).  The
        SSE loss only: a hit-level loss reads the hit count on the host."""
        if self.loss_fn is not None:
            raise ValueError("a fit with a hit-level loss runs eagerly (run(..., graph=False))")
        saved = [t.clone() for t in (self.theta, self.state, self.loss_hist, self.theta_hist, self.step_idx)]
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self._launch()
        torch.cuda.current_stream().wait_stream(side)
        for t, v in zip((self.theta, self.state, self.loss_hist, self.theta_hist, self.step_idx), saved):
            t.copy_(v)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode="thread_local"):
            self._launch()
        return self.graph

    def run(self, n_steps, graph=True):
        """n_steps optimiser steps; returns (loss history, parameter history)
        of all steps taken so far, as numpy arrays."""
        graph = graph and self.loss_fn is None   # a hit-level loss runs eagerly
        if graph and self.graph is None:
            self.capture()
        for _ in range(n_steps):
            if graph:
                self.graph.replay()
            else:
                self._launch()
        return self.history()

    def history(self):
        n = min(int(self.step_idx.item()), self.max_steps)
        return self.loss_hist[:n].cpu().numpy(), self.theta_hist[:n].cpu().numpy()

    def normalised(self):
        """The current normalised parameters u (GRAD_PARAMS order)."""
        return self.state[2 * _abi.NPARAM:3 * _abi.NPARAM].cpu().numpy()

    def params(self, params):
        """``params`` with the current fit values."""
        vals = self.theta.cpu().numpy().astype(np.float64)
        return params.replace(**{k: float(v) for k, v in zip(GRAD_PARAMS, vals)})
