"""Device-resident Adam fit of the physics parameters (the fit loop of
optimize/fit_params.py:704-731, :872-895 with the "divide" normalisation).

One step is: the segment stage with the fit parameters read from device
memory (``lsim_lut_stage1_theta``), the forward + adjoint of the SSE-ADC
loss (``lsim_lut_grad``) and an Adam update of the parameters in place
(``lsim_adam_step``).  Nothing in a step needs the host, so the step is
captured once in a CUDA graph and replayed; the loss and the parameters of
every step are appended to device-side histories inside the graph.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _abi, consts, sim
from .grad import GRAD_PARAMS, Target


class DeviceFit:
    """Adam on ``fit_params`` (a subset of GRAD_PARAMS) against ``target``.

    ``lr`` is the learning rate in normalised units (parameter / scale);
    ``scale`` defaults to the nominal values of the reference's parameters.
    """

    def __init__(self, params, response_template, tracks, fields, target: Target, fit_params=None, lr=1e-2,
                 scale=None, betas=(0.9, 0.999), eps=1e-8, n_events=None, max_steps=1000):
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
        unknown = set(fit) - set(GRAD_PARAMS)
        if unknown:
            raise ValueError(f"cannot fit {sorted(unknown)}; fit parameters are {GRAD_PARAMS}")
        nominal = consts.Params()
        sc = [abs(float(getattr(nominal, k))) if scale is None else float(scale[k]) for k in GRAD_PARAMS]
        self.theta = torch.tensor([float(getattr(params, k)) for k in GRAD_PARAMS], dtype=torch.float32, device=dev)
        self.scale = torch.tensor(sc, dtype=torch.float32, device=dev)
        self.lr = torch.tensor([lr if k in fit else 0.0 for k in GRAD_PARAMS], dtype=torch.float32, device=dev)
        self.state = torch.zeros(2 * _abi.NPARAM + 1, dtype=torch.float32, device=dev)
        self.out = torch.empty(1 + _abi.NPARAM, dtype=torch.float32, device=dev)
        self.betas, self.eps = (float(betas[0]), float(betas[1])), float(eps)
        self.target = target
        self.max_steps = int(max_steps)
        self.loss_hist = torch.zeros(self.max_steps, dtype=torch.float32, device=dev)
        self.theta_hist = torch.zeros((self.max_steps, _abi.NPARAM), dtype=torch.float32, device=dev)
        self.step_idx = torch.zeros(1, dtype=torch.int64, device=dev)
        self.graph = None

    def _launch(self):
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
        _abi.check(lib, lib.lsim_adam_step(p(self.theta), p(self.out[1:]), p(self.scale), p(self.lr), p(self.state),
                                           self.betas[0], self.betas[1], self.eps, s))

    def step(self):
        """One eager step (no graph)."""
        self._launch()

    def capture(self):
        """Capture one step in a CUDA graph (a warm-up step runs first and is
        undone, so the trajectory starts from the current parameters)."""
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
        """n_steps Adam steps; returns (loss history, parameter history) of
        all steps taken so far, as numpy arrays."""
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

    def params(self, params):
        """``params`` with the current fit values."""
        vals = self.theta.cpu().numpy().astype(np.float64)
        return params.replace(**{k: float(v) for k, v in zip(GRAD_PARAMS, vals)})
