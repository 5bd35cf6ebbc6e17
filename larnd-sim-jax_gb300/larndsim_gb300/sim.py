"""Drop-in simulate functions (reference: src/larndsim/sim_jax.py).

Same names, arguments and outputs as the reference's LUT-mode and
parametrised-mode entry points; arrays are torch CUDA tensors (inputs may
also be numpy arrays or CPU tensors).  All device work runs in liblsim's
sm_103a kernels on the current torch stream; there is no CPU fallback.

Behaviour that differs from the reference on purpose:
* Waveform rows whose pixel id is negative (the -1 rows and eventID -1
  rows that ``parse_output`` always drops) are returned as zeros instead of
  the sum of every unmatched neighbour contribution.
* Noise draws (when RESET/UNCORRELATED noise are non-zero) come from
  torch's generator seeded with ``rngseed``, not JAX's threefry stream;
  exact draws can be supplied through ``normals=``.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _abi, consts

_SIZE_HISTORY: dict = {}


def pad_size(cur_size, tag, pad_threshold=0.05):
    """Size buckets that limit the number of distinct shapes (sim_jax.py:61-102)."""
    scalar = isinstance(cur_size, (int, np.integer))
    cur = (int(cur_size),) if scalar else tuple(int(c) for c in cur_size)
    sizes = _SIZE_HISTORY.setdefault(tag, [])
    if cur in sizes:
        return cur[0] if scalar else cur
    for s in sizes:
        if all(c <= q <= c * (1 + pad_threshold) for c, q in zip(cur, s)):
            return s[0] if scalar else s
    new = tuple(int(c * (1 + pad_threshold / 2) + 0.5) for c in cur)
    sizes.append(new)
    sizes.sort()
    return new[0] if scalar else new


def get_size_history():
    return _SIZE_HISTORY


def reset_size_history():
    _SIZE_HISTORY.clear()


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("larndsim_gb300 needs a CUDA device (sm_103a); no CPU fallback exists")
    return torch.device("cuda", torch.cuda.current_device())


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _ptr(t):
    return None if t is None else t.data_ptr()


def as_tracks(tracks) -> torch.Tensor:
    t = torch.as_tensor(np.asarray(tracks) if not isinstance(tracks, torch.Tensor) else tracks)
    return t.to(device=_device(), dtype=torch.float32).contiguous()


def _n_events(tracks_dev: torch.Tensor, fields) -> int:
    ev = tracks_dev[:, fields.index("eventID")]
    return int(ev.max().item()) + 1 if ev.numel() else 0


class PreparedLUT:
    """A template bank on the device plus the tables derived from it.

    The reference recomputes a cumulative sum over the whole bank on every
    call (sim_jax.py:228); here the windows and cumulative sums are derived
    once per bank and reused.
    """

    def __init__(self, response_template, params):
        lib = _abi.load()
        t = torch.as_tensor(response_template) if not isinstance(response_template, torch.Tensor) else response_template
        self.templates = t.to(device=_device(), dtype=torch.float32).contiguous()
        if self.templates.dim() != 4:
            raise ValueError("response_template must have shape (n_templates, nx, ny, nt)")
        self.shape = tuple(self.templates.shape)
        self.signal_length = int(params.signal_length)
        self.n_templates = self.shape[0]
        lp = _abi.make_params(params, self.shape)
        nbytes = lib.lsim_lut_tables_bytes(lp)
        self.tables = torch.empty(nbytes, dtype=torch.uint8, device=self.templates.device)
        _abi.check(lib, lib.lsim_lut_prepare(lp, _ptr(self.templates), _ptr(self.tables), nbytes, _stream()))
        self._key = self.key(self.templates, params)

    @staticmethod
    def key(t, params):
        return (t.data_ptr(), tuple(t.shape), t._version, int(params.signal_length),
                tuple(np.asarray(params.long_diff_template, np.float32).tolist()))


_LUT_CACHE: dict = {}


def prepare_lut(response_template, params) -> PreparedLUT:
    """Prepared tables for a template bank (cached per bank tensor)."""
    if isinstance(response_template, PreparedLUT):
        return response_template
    if isinstance(response_template, torch.Tensor) and response_template.is_cuda:
        k = PreparedLUT.key(response_template.contiguous(), params)
        hit = _LUT_CACHE.get(k)
        if hit is not None:
            return hit
        lut = PreparedLUT(response_template, params)
        _LUT_CACHE.clear()
        _LUT_CACHE[k] = lut
        return lut
    return PreparedLUT(response_template, params)


def load_lut(lut, params):
    """Template bank from a raw response LUT (consts_jax.py:387-449).

    ``lut`` is a path to a .npy/.npz file (key 'response') or an array of
    shape (nx, ny, nt).  Returns (templates on the device, params).
    """
    updated = params
    if isinstance(lut, (str, bytes)) or hasattr(lut, "__fspath__"):
        arr = np.load(lut)
        if isinstance(arr, np.lib.npyio.NpzFile):
            if "response" not in arr:
                raise ValueError("No 'response' key found in the npz file.")
            resp = arr["response"]
            if "drift_length" in arr:
                updated = params.replace(response_full_drift_t=float(arr["drift_length"]) / params.vdrift_static)
        else:
            resp = arr
    else:
        resp = lut
    dev = _device()
    r = torch.as_tensor(np.asarray(resp, np.float32) if not isinstance(resp, torch.Tensor) else resp)
    r = r.to(device=dev, dtype=torch.float32).contiguous()
    if r.dim() != 3:
        raise ValueError("response LUT must have shape (nx, ny, nt)")
    sig = torch.as_tensor(np.asarray(params.long_diff_template, np.float32), device=dev)
    nt_ = sig.shape[0]
    out = torch.empty((nt_,) + tuple(r.shape), dtype=torch.float32, device=dev)
    lib = _abi.load()
    _abi.check(lib, lib.lsim_lut_build_templates(_ptr(r), r.shape[0], r.shape[1], r.shape[2], _ptr(sig), nt_,
                                                 int(params.long_diff_extent), _ptr(out), _stream()))
    return out, updated


class Stage1:
    """Device state after the segment + pixel-map stage."""

    def __init__(self, lp, tracks, n_rows, n_events, ws, counts):
        self.lp, self.tracks, self.n_rows, self.n_events = lp, tracks, n_rows, n_events
        self.ws, self.counts_dev = ws, counts
        self._host = None

    def counts(self):
        if self._host is None:
            self._host = self.counts_dev.cpu().numpy()
        return self._host

    @property
    def n_valid(self):
        return int(self.counts()[0])

    @property
    def n_em1(self):
        return int(self.counts()[1])

    @property
    def any_m1(self):
        return int(self.counts()[2])

    def raise_status(self):
        c = self.counts()
        if c[3] == _abi.LSIM_ERR_CAPACITY:
            raise ValueError(f"{int(c[4])} segments share one principal pixel; at most {(1 << 23) - 1} are supported")
        if c[3] == _abi.LSIM_ERR_UNSUPPORTED:
            raise ValueError(f"segment at row {int(c[5])} lies beyond the supported sub-pixel bin range "
                             "(|bin| < 32768 per axis)")
        if c[3] != 0:
            row = int(c[5])
            raise ValueError(f"invalid track input: eventID outside [-1, {self.n_events}) at row {row} "
                             "(event ids must form a local namespace -1, 0..N-1)")


def run_stage1(params, tracks, fields, lp, param_mode=False, normals=None, n_events=None) -> Stage1:
    lib = _abi.load()
    fields = tuple(fields)
    t = as_tracks(tracks)
    if t.dim() != 2 or t.shape[1] != len(fields):
        raise ValueError(f"tracks must be (N, {len(fields)}) to match fields")
    n = t.shape[0]
    ne = _n_events(t, fields) if n_events is None else int(n_events)
    fm = _abi.field_map(fields)
    ws_bytes = lib.lsim_workspace_bytes(lp, n, ne)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=t.device)
    counts = torch.empty(16, dtype=torch.int32, device=t.device)
    if param_mode:
        nrm = None if normals is None else torch.as_tensor(normals).to(device=t.device, dtype=torch.float32).contiguous()
        if nrm is not None and tuple(nrm.shape) != (n, 3):
            raise ValueError("normals must have shape (N, 3)")
        _abi.check(lib, lib.lsim_param_stage1(lp, fm, _ptr(t), n, ne, _ptr(nrm), _ptr(ws), ws_bytes, _ptr(counts),
                                              _stream()))
        st = Stage1(lp, t, n, ne, ws, counts)
        st.normals = nrm
    else:
        _abi.check(lib, lib.lsim_lut_stage1(lp, fm, _ptr(t), n, ne, _ptr(ws), ws_bytes, _ptr(counts), _stream()))
        st = Stage1(lp, t, n, ne, ws, counts)
    return st


def simulate_wfs(params, response_template, tracks, fields):
    """LUT-mode waveforms (sim_jax.py:689-736).

    Returns ``wfs`` (P_pad, Nticks-1) float32 and ``unique_pixels`` (P_pad,)
    int32, rows ordered as the reference orders them.
    """
    lut = prepare_lut(response_template, params)
    lp = _abi.make_params(params, lut.shape)
    st = run_stage1(params, tracks, fields, lp)
    st.raise_status()
    p_unique = st.n_em1 + st.n_valid + st.any_m1 + 1          # + the appended -1 (sim_jax.py:718)
    p_pad = pad_size(p_unique, "unique_pixels", 0.2)
    lib = _abi.load()
    T = lp.n_ticks - 1
    dev = st.tracks.device
    wfs = torch.empty((p_pad, T), dtype=torch.float32, device=dev)
    unique = torch.empty((p_pad,), dtype=torch.int32, device=dev)
    _abi.check(lib, lib.lsim_lut_stage2(lp, _ptr(lut.tables), _ptr(st.ws), st.n_rows, st.n_events, p_pad, st.n_em1,
                                        st.n_valid, _ptr(wfs), _ptr(unique), _stream()))
    return wfs, unique


def _noise_normals(params, n_pix, rngseed, normals):
    H = int(params.MAX_ADC_VALUES)
    if normals is not None:
        nrm = torch.as_tensor(normals).to(device=_device(), dtype=torch.float32).contiguous()
        if tuple(nrm.shape) != (n_pix, 1 + 3 * H):
            raise ValueError(f"normals must have shape ({n_pix}, {1 + 3 * H})")
        return nrm
    if params.RESET_NOISE_CHARGE == 0 and params.UNCORRELATED_NOISE_CHARGE == 0:
        return None
    g = torch.Generator(device=_device())
    g.manual_seed(int(rngseed) % (2 ** 63))
    return torch.randn((n_pix, 1 + 3 * H), generator=g, device=_device(), dtype=torch.float32)


def get_adc_values(params, pixels_signals, rngseed=0, normals=None):
    """Self-trigger FEE (fee_jax.py:168-279): (integral, ticks), each (P, H)."""
    lib = _abi.load()
    w = torch.as_tensor(pixels_signals).to(device=_device(), dtype=torch.float32).contiguous()
    P, T = w.shape
    H = int(params.MAX_ADC_VALUES)
    lp = _abi.make_params(params)
    nrm = _noise_normals(params, P, rngseed, normals)
    adc = torch.empty((P, H), dtype=torch.float32, device=w.device)
    ticks = torch.empty((P, H), dtype=torch.float32, device=w.device)
    integral = torch.empty((P, H), dtype=torch.float32, device=w.device)
    _abi.check(lib, lib.lsim_fee(lp, _ptr(w), P, T, _ptr(nrm), _ptr(adc), _ptr(ticks), _ptr(integral), _stream()))
    return integral, ticks


def _fee_and_hits(params, wfs, unique_pixels, tick_limit, rngseed, normals):
    lib = _abi.load()
    w = torch.as_tensor(wfs).to(device=_device(), dtype=torch.float32).contiguous()
    u = torch.as_tensor(unique_pixels).to(device=w.device, dtype=torch.int32).contiguous()
    P, T = w.shape
    H = int(params.MAX_ADC_VALUES)
    lp = _abi.make_params(params)
    nrm = _noise_normals(params, P, rngseed, normals)
    adc = torch.empty((P, H), dtype=torch.float32, device=w.device)
    ticks = torch.empty((P, H), dtype=torch.float32, device=w.device)
    _abi.check(lib, lib.lsim_fee(lp, _ptr(w), P, T, _ptr(nrm), _ptr(adc), _ptr(ticks), None, _stream()))
    n = P * H
    outs_f = [torch.empty(n, dtype=torch.float32, device=w.device) for _ in range(6)]
    out_event = torch.empty(n, dtype=torch.int32, device=w.device)
    out_pix = torch.empty(n, dtype=torch.int32, device=w.device)
    nb = torch.empty(1, dtype=torch.int32, device=w.device)
    hb = lib.lsim_hits_workspace_bytes(P, H)
    hws = torch.empty(hb, dtype=torch.uint8, device=w.device)
    o_adc, o_x, o_y, o_z, o_t, o_hp = outs_f
    _abi.check(lib, lib.lsim_hits(lp, _ptr(adc), _ptr(ticks), _ptr(u), P, int(tick_limit), _ptr(o_adc), _ptr(o_x),
                                  _ptr(o_y), _ptr(o_z), _ptr(o_t), _ptr(o_hp), _ptr(out_event), _ptr(out_pix),
                                  _ptr(nb), _ptr(hws), hb, _stream()))
    k = int(nb.item())
    return (o_adc[:k], o_x[:k], o_y[:k], o_z[:k], o_t[:k], o_hp[:k], out_event[:k], out_pix[:k]), (adc, ticks)


def simulate_stochastic(params, wfs, unique_pixels, rngseed=0, normals=None, return_grids=False):
    """FEE, hit coordinates and compaction (sim_jax.py:738-769).

    Returns (adcs, pixel_x, pixel_y, pixel_z, ticks, hit_prob, event,
    hit_pixels), 1-D of the number of accepted hits.
    """
    T = torch.as_tensor(wfs).shape[1]
    out, grids = _fee_and_hits(params, wfs, unique_pixels, T - 3, rngseed, normals)
    return (out, grids) if return_grids else out


def draw_offsets(n, rngseed=0, device=None):
    """Standard normals (n, 3) for the Monte-Carlo diffusion offsets."""
    g = torch.Generator(device=device or _device())
    g.manual_seed(int(rngseed) % (2 ** 63))
    return torch.randn((n, 3), generator=g, device=device or _device(), dtype=torch.float32)


def simulate_parametrized_wfs(params, tracks, fields, rngseed=0, offsets=None):
    """Waveforms and unique pixels of parametrised mode (sim_jax.py:339-368)."""
    if int(params.number_pix_neighbors) != 0:
        raise ValueError("parametrised mode requires number_pix_neighbors == 0")
    lp = _abi.make_params(params)
    t = as_tracks(tracks)
    nrm = offsets if offsets is not None else draw_offsets(t.shape[0], rngseed, t.device)
    if not params.mc_diff:
        raise ValueError("parametrised mode needs mc_diff=True: the reference's deterministic branch "
                         "(apply_tran_diff) requires tran_diff_bin_edges, which it never sets")
    if not params.diffusion_in_current_sim:
        raise NotImplementedError("diffusion_in_current_sim=False (current_model, detsim_jax.py:545-579) is not "
                                  "implemented; the default True (current_model_diff) is")
    st = run_stage1(params, t, fields, lp, param_mode=True, normals=nrm)
    st.raise_status()
    p_unique = st.n_em1 + st.n_valid + st.any_m1
    p_pad = pad_size(p_unique, "unique_pixels")
    lib = _abi.load()
    T = lp.n_ticks - 1
    wfs = torch.empty((p_pad, T), dtype=torch.float32, device=t.device)
    unique = torch.empty((p_pad,), dtype=torch.int32, device=t.device)
    _abi.check(lib, lib.lsim_param_stage2(lp, _ptr(st.ws), st.n_rows, st.n_events, p_pad, st.n_em1, st.n_valid,
                                          _ptr(wfs), _ptr(unique), _stream()))
    return wfs, unique


def simulate_parametrized(params, tracks, fields, rngseed=0, offsets=None, normals=None, return_wfs=False):
    """Parametrised-current simulation (sim_jax.py:339-372).

    ``offsets`` (N, 3) standard normals for the diffusion draws (drawn
    from ``rngseed`` when omitted).  Returns the same 8-tuple as the
    reference (last element: pixel ids).
    """
    wfs, unique = simulate_parametrized_wfs(params, tracks, fields, rngseed, offsets)
    out, _ = _fee_and_hits(params, wfs, unique, wfs.shape[1] + 1 - 3, rngseed + 1, normals)
    return (out, wfs, unique) if return_wfs else out


# ---------------------------------------------------------------- probabilistic front end

def _fee_prob(params, wfs, stop_threshold, distributions, reductions):
    lib = _abi.load()
    w = torch.as_tensor(wfs).to(device=_device(), dtype=torch.float32).contiguous()
    if w.dim() != 2:
        raise ValueError(f"wfs must be (n_pixels, n_ticks), got {tuple(w.shape)}")
    if not params.RESET_NOISE_CHARGE > 0:
        raise ValueError("the probabilistic front end needs RESET_NOISE_CHARGE > 0 (its noise width)")
    P, T = w.shape
    H = int(params.MAX_ADC_VALUES)
    lp = _abi.make_params(params)
    ws = torch.empty(lib.lsim_fee_prob_workspace_bytes(lp), dtype=torch.uint8, device=w.device)
    f = dict(dtype=torch.float32, device=w.device)
    log_prob = torch.empty((P, H, T - 1), **f) if distributions else None
    charge = torch.empty((P, H, T - 1), **f) if distributions else None
    red = [torch.empty((P, H), **f) for _ in range(3)] if reductions else [None] * 3
    _abi.check(lib, lib.lsim_fee_prob(lp, _ptr(w), P, T, int(params.fee_paths_scaling), float(stop_threshold),
                                      _ptr(log_prob), _ptr(charge), *(_ptr(r) for r in red), _ptr(ws),
                                      ws.numel(), _stream()))
    return log_prob, charge, red


def _fee_prob_vjp(params, wfs, stop_threshold, g_lp=None, g_ch=None, g_red=None):
    lib = _abi.load()
    w = wfs.detach().to(dtype=torch.float32).contiguous()
    P, T = w.shape
    lp = _abi.make_params(params)
    K = int(params.fee_paths_scaling)
    ws = torch.empty(lib.lsim_fee_prob_vjp_workspace_bytes(lp, P, K), dtype=torch.uint8, device=w.device)
    g = torch.empty_like(w)
    c = lambda t: None if t is None else t.to(torch.float32).contiguous()   # noqa: E731
    red = [None] * 3 if g_red is None else [c(t) for t in g_red]
    g_lp, g_ch = c(g_lp), c(g_ch)
    _abi.check(lib, lib.lsim_fee_prob_vjp(lp, _ptr(w), P, T, K, float(stop_threshold), _ptr(g_lp), _ptr(g_ch),
                                          *(_ptr(r) for r in red), _ptr(g), _ptr(ws), ws.numel(), _stream()))
    return g


class _FeeProbDistFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, wfs, params, stop_threshold):
        log_prob, charge, _ = _fee_prob(params, wfs, stop_threshold, True, False)
        ctx.save_for_backward(wfs)
        ctx.params, ctx.stop = params, stop_threshold
        return log_prob, charge

    @staticmethod
    def backward(ctx, g_lp, g_ch):
        (wfs,) = ctx.saved_tensors
        return _fee_prob_vjp(ctx.params, wfs, ctx.stop, g_lp=g_lp, g_ch=g_ch), None, None


class _FeeProbRedFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, wfs, params, stop_threshold):
        _, _, (e_tick, e_adc, lam) = _fee_prob(params, wfs, stop_threshold, False, True)
        ctx.save_for_backward(wfs)
        ctx.params, ctx.stop = params, stop_threshold
        return e_tick, e_adc, lam

    @staticmethod
    def backward(ctx, g_t, g_a, g_l):
        (wfs,) = ctx.saved_tensors
        zero = lambda g: torch.zeros(wfs.shape[0], int(ctx.params.MAX_ADC_VALUES), device=wfs.device) \
            if g is None else g   # noqa: E731
        return _fee_prob_vjp(ctx.params, wfs, ctx.stop, g_red=(zero(g_t), zero(g_a), zero(g_l))), None, None


def _as_wfs(wfs):
    w = torch.as_tensor(wfs)
    return (w if w.is_cuda else w.to(device=_device())).to(torch.float32)


def get_adc_values_average_noise_vmap(params, wfs, stop_threshold=1e-9):
    """Probabilistic self-trigger front end (fee_jax.py:386-461): a beam
    search over ``fee_paths_scaling`` paths and MAX_ADC_VALUES hits with
    noise width RESET_NOISE_CHARGE.  Returns (log_prob, charge), each
    (P, MAX_ADC_VALUES, T - 1): the log-probability that hit h is read at
    each tick and the expected charge if it is.  Differentiable with
    respect to ``wfs`` (lsim_fee_prob_vjp)."""
    return _FeeProbDistFn.apply(_as_wfs(wfs), params, stop_threshold)


def average_hit_values(params, wfs, stop_threshold=1e-9):
    """get_average_hit_values (fee_jax.py:463-480) of the probabilistic
    front end's output, fused into the beam search so the (P, H, T - 1)
    distributions are never stored: (expected_ticks, expected_adcs,
    lambda), each (P, MAX_ADC_VALUES).  Differentiable with respect to
    ``wfs`` (lsim_fee_prob_vjp)."""
    return _FeeProbRedFn.apply(_as_wfs(wfs), params, stop_threshold)


def get_average_hit_values(ticks_prob, adcs_distrib):
    """fee_jax.py:463-480 on given distributions (probabilities, not logs):
    (expected_ticks, expected_adcs, lambda) per (pixel, hit)."""
    tp = torch.as_tensor(ticks_prob, dtype=torch.float32)
    ad = torch.as_tensor(adcs_distrib, dtype=torch.float32, device=tp.device)
    lam = tp.sum(dim=2)
    ticks = torch.arange(tp.shape[2], dtype=torch.float32, device=tp.device)
    den = torch.clamp(lam, min=1e-10)
    return (ticks * tp).sum(dim=2) / den, (ad * tp).sum(dim=2) / den, lam


def pixel_coordinates(params, unique_pixels):
    """(pixel_x, pixel_y, plane, event) of each pixel id: id2pixel +
    get_pixel_coordinates (detsim_jax.py:264-306)."""
    lib = _abi.load()
    u = torch.as_tensor(unique_pixels).to(device=_device(), dtype=torch.int32).contiguous()
    n = u.shape[0]
    x = torch.empty(n, dtype=torch.float32, device=u.device)
    y = torch.empty(n, dtype=torch.float32, device=u.device)
    plane = torch.empty(n, dtype=torch.int32, device=u.device)
    event = torch.empty(n, dtype=torch.int32, device=u.device)
    _abi.check(lib, lib.lsim_pixel_coords(_abi.make_params(params), _ptr(u), n, _ptr(x), _ptr(y), _ptr(plane),
                                          _ptr(event), _stream()))
    return x, y, plane, event


def simulate_probabilistic(params, wfs, unique_pixels):
    """sim_jax.py:771-813: (adcs_distrib, pixel_x, pixel_y, ticks_prob,
    event); ticks_prob holds the log-probabilities of the beam search and
    adcs_distrib the digitised expected charges, both (P, H, T - 1)."""
    from .fee import digitize
    log_prob, charge = get_adc_values_average_noise_vmap(params, wfs)
    x, y, _, event = pixel_coordinates(params, unique_pixels)
    return digitize(params, charge), x, y, log_prob, event


# ---------------------------------------------------------------- differentiable front end

class _FeeFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, wfs, params, normals):
        lib = _abi.load()
        w = wfs.detach().to(dtype=torch.float32).contiguous()
        P, T = w.shape
        H = int(params.MAX_ADC_VALUES)
        lp = _abi.make_params(params)
        adc = torch.empty((P, H), dtype=torch.float32, device=w.device)
        ticks = torch.empty((P, H), dtype=torch.float32, device=w.device)
        _abi.check(lib, lib.lsim_fee(lp, _ptr(w), P, T, _ptr(normals), _ptr(adc), _ptr(ticks), None, _stream()))
        ctx.save_for_backward(w)
        ctx.lp, ctx.normals = lp, normals
        ctx.mark_non_differentiable(ticks)
        return adc, ticks

    @staticmethod
    def backward(ctx, g_adc, g_ticks):
        (w,) = ctx.saved_tensors
        lib = _abi.load()
        P, T = w.shape
        g = torch.zeros_like(w)
        if g_adc is None:
            return g, None, None
        ga = g_adc.to(torch.float32).contiguous()
        ws = torch.empty(lib.lsim_fee_vjp_workspace_bytes(P), dtype=torch.uint8, device=w.device)
        _abi.check(lib, lib.lsim_fee_vjp(ctx.lp, _ptr(w), P, T, _ptr(ctx.normals), _ptr(ga), _ptr(g), _ptr(ws),
                                         ws.numel(), _stream()))
        return g, None, None


def fee_adc(params, wfs, rngseed=0, normals=None):
    """Self-trigger front end + digitize (fee_jax.py:55-71, :168-279) as a
    differentiable function of the waveforms: (adc, ticks), each (P, H);
    ``adc.backward(g)`` gives dL/dwfs with the reference's gradient
    treatment (lsim_fee_vjp)."""
    w = torch.as_tensor(wfs)
    if not w.is_cuda:
        w = w.to(device=_device())
    w = w.to(torch.float32)
    nrm = _noise_normals(params, w.shape[0], rngseed, normals)
    return _FeeFn.apply(w, params, nrm)


# ---------------------------------------------------------------- differentiable parametrised mode

class _ParamWfsFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, params, tracks, fields, offsets):
        from .grad import GRAD_PARAMS
        vals = theta.detach().cpu().numpy().astype(np.float64)
        p = params.replace(**{k: float(v) for k, v in zip(GRAD_PARAMS, vals)})
        lp = _abi.make_params(p)
        st = run_stage1(p, tracks, fields, lp, param_mode=True, normals=offsets)
        st.raise_status()
        p_unique = st.n_em1 + st.n_valid + st.any_m1
        p_pad = pad_size(p_unique, "unique_pixels")
        lib = _abi.load()
        T = lp.n_ticks - 1
        wfs = torch.empty((p_pad, T), dtype=torch.float32, device=st.tracks.device)
        unique = torch.empty((p_pad,), dtype=torch.int32, device=st.tracks.device)
        _abi.check(lib, lib.lsim_param_stage2(lp, _ptr(st.ws), st.n_rows, st.n_events, p_pad, st.n_em1, st.n_valid,
                                              _ptr(wfs), _ptr(unique), _stream()))
        ctx.st, ctx.lp = st, lp
        ctx.theta_device, ctx.theta_dtype = theta.device, theta.dtype
        ctx.mark_non_differentiable(unique)
        return wfs, unique

    @staticmethod
    def backward(ctx, g_wfs, g_unique):
        if g_wfs is None:
            return (None,) * 5
        lib = _abi.load()
        st = ctx.st
        g = g_wfs.to(dtype=torch.float32).contiguous()
        out = torch.empty(_abi.NPARAM, dtype=torch.float32, device=g.device)
        _abi.check(lib, lib.lsim_param_wfs_vjp(ctx.lp, _ptr(st.ws), st.n_rows, st.n_events, _ptr(g), g.shape[0],
                                               st.n_valid, _ptr(out), _stream()))
        return out.to(device=ctx.theta_device, dtype=ctx.theta_dtype), None, None, None, None


def param_wfs_fn(theta, params, tracks, fields, offsets):
    """Differentiable parametrised-mode waveforms (simulate_parametrized's
    signal stage, sim_jax.py:339-368) as a function of ``theta`` = the 8
    parameter values (order grad.GRAD_PARAMS), with the Monte-Carlo
    diffusion offsets (N, 3) held fixed: returns (wfs, unique_pixels);
    backward runs lsim_param_wfs_vjp.  Compose with fee_adc for the ADCs."""
    if int(params.number_pix_neighbors) != 0:
        raise ValueError("parametrised mode requires number_pix_neighbors == 0")
    if not params.mc_diff or not params.diffusion_in_current_sim:
        raise NotImplementedError("the differentiable parametrised mode covers mc_diff=True with "
                                  "diffusion_in_current_sim=True")
    t = as_tracks(tracks)
    off = torch.as_tensor(offsets).to(device=t.device, dtype=torch.float32).contiguous()
    return _ParamWfsFn.apply(theta, params, t, tuple(fields), off)
