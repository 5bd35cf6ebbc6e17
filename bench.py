#!/usr/bin/env python3
"""Benchmark: batched LUT-mode forward + backward on GB300.

Workload (one "step"): the sum-of-squared-ADC loss and its gradient with
respect to the 8 physics parameters (Ab, kb, eField, lifetime, vdrift,
long_diff, tran_diff, lArDensity) for a batch of 64 events whose segment
counts are log-uniform in [1k, 50k] (straight tracks + short-segment
showers), number_pix_neighbors = 4, signal_length = 150, a seeded
45x45x1950 LUT expanded to 100 long-diffusion templates.  The prediction is
simulated at parameters perturbed by N(0, 5%) from the target's nominal
values.  Metric: forward+backward segments per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  ``value`` times the device-resident step
(inputs in HBM); ``e2e`` times the public API call with the tracks in
pinned host memory, copied in and the loss/gradient copied out inside the
timed region.  ``--impl reference`` times the CPU restatement of the
reference's algorithm (the reference is JAX; no JAX exists on the target
machines) on a bounded sample of the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "larnd-sim-jax_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import numpy as np  # noqa: E402

METRIC = "fwd+bwd segments/s"
UNIT = "segments/s"
N_EVENTS, MIN_SEG, MAX_SEG = 64, 1000, 50000
N_NEIGH, SIG_LEN = 4, 150
PERTURB_SEED = 1234
L2_FLUSH_BYTES = 512 << 20
CPU_CHUNK = 150          # segments per CPU reference sample (one run per process)
KERNELS_PER_STEP = 20   # stage 1: reset, segments, 3 scan, scatter, 2 sort; gradient: 3 template-order kernels,
                        # main records, heavy-pixel list, target index, pixels, main adjoint, 2 record reductions,
                        # target-only, finalize (counted in the launch list of the step)
# DRAM bytes per simulated pixel of one k_lut_pixels<grad> launch, from an
# ncu capture of the 8-event case of this workload (22,066 pixels; traffic
# scales with the pixel count)
PIXEL_KERNEL_DRAM_BYTES_PER_PIXEL = 14072   # 310.5 MB over 22,066 pixels


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--events", type=int, default=N_EVENTS, help="events per batch (profiling runs use fewer)")
    ap.add_argument("--hits", type=int, default=None, help="hits of --path records (profiling runs use fewer)")
    ap.add_argument("--path", choices=["grad", "forward", "param", "param_grad", "chop", "prob", "loss", "records",
                                       "fit"],
                    default="grad",
                    help="grad: the fwd+bwd step (default); chop: on-device chop_tracks of one 500k-segment event; "
                         "prob: the probabilistic front end on the waveforms of 8 events; loss: mse_adc forward + "
                         "gradient on the hits of the 64-event batch; forward / param: the plain forward "
                         "drop-in (LUT mode / parametrised mode) on the 64-event batch; param_grad: the "
                         "parametrised-mode SSE-ADC loss and its gradient (autograd through the waveform, "
                         "front-end and current-model adjoints); records: the driver's hit records (clean "
                         "mask, compaction, charge, per-event runs) of 32M hits; fit: 200 steps of the "
                         "reference's gradient-descent fit (sigmoid normalisation, Adam) on 32 events x 20k "
                         "segments, one CUDA graph per step")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def workload(rank, seed, n_events=N_EVENTS):
    from larndsim_gb300 import workloads
    tracks, fields = workloads.batched_events(seed=seed + 1000 * rank, n_events=n_events,
                                              min_segments=MIN_SEG, max_segments=MAX_SEG)
    return tracks, fields


def nominal_params():
    from larndsim_gb300 import consts
    return consts.Params(number_pix_neighbors=N_NEIGH, signal_length=SIG_LEN, RESET_NOISE_CHARGE=0,
                         UNCORRELATED_NOISE_CHARGE=0)


def perturbed(params):
    from larndsim_gb300.grad import GRAD_PARAMS
    rng = np.random.default_rng(PERTURB_SEED)
    upd = {k: float(getattr(params, k)) * (1.0 + 0.05 * rng.standard_normal()) for k in GRAD_PARAMS}
    return params.replace(**upd)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=5)
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def lut_bytes_touched(seg_tidx, n_templates, lut_nx, lut_ny, L, Nt):
    """Distinct LUT floats read: the three templates around every used
    template index on the 5x5 main sub-positions and all template-0 rows,
    each an L-tick window plus three cumulative-sum entries."""
    used = np.unique(np.concatenate([seg_tidx - 1, seg_tidx, seg_tidx + 1]))
    rows = used.size * 25 + lut_nx * lut_ny
    return rows * (L + 3)


def run_ours(args):
    import torch
    from larndsim_gb300 import _abi, grad, sim, workloads

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    dev = torch.device("cuda", local)

    params = nominal_params()
    resp = workloads.synthetic_response(seed=0)
    tmpl, params = sim.load_lut(resp, params)
    tracks, fields = workload(rank, args.seed, args.events)
    n_seg = tracks.shape[0]
    chain = grad.LUTChain(params, tmpl, tracks, fields)
    target = chain.target(params)
    pp = perturbed(params)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step(ev=None):
        return chain.loss_and_grad_device(pp, target, events=ev)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    st = chain._stage
    n_pix = st.n_valid
    seg_rec = st.ws[256:256 + 96 * n_seg].view(torch.int32).view(n_seg, 24).cpu().numpy()
    ne = seg_rec[:, 0].view(np.float32)
    active = int((ne > 0).sum())
    # ---- launch shapes picked by the autotuner for this device and batch
    from larndsim_gb300 import tune
    tuned, _ = tune.autotune(step, key=("bench", n_seg, N_NEIGH))
    # ---- the pixel kernel alone, CUDA events around its launch (eager steps)
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
    for e in kev:
        flush.fill_(1.0)
        _abi.set_kernel_events(*e)
        step()
    torch.cuda.synchronize()
    _abi.set_kernel_events(None, None)
    kern_ms = [a.elapsed_time(b) for a, b in kev]
    # ---- timed region: device-resident step, the whole step replayed as one CUDA graph
    graph, out = chain.capture(pp, target)
    for _ in range(args.warmup):
        graph.replay()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(torch.cuda.current_device())
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    total = torch.empty_like(out)
    for i in range(args.steps):
        flush.fill_(float(i))              # evict L2 between steps (untimed)
        starts[i].record()
        graph.replay()
        if pg:
            total.copy_(out)
            pg.all_reduce(total)           # the fit step's exchange: [loss, gradient] summed over event shards
        ends[i].record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = float(np.mean(step_ms))
    if pg:
        t = torch.tensor([ms], device=dev)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
        out = total
    clk = clocks.stop()
    value = n_seg * world / (ms * 1e-3)
    # ---- end-to-end through the public API (host tracks, pinned)
    host = torch.from_numpy(tracks).pin_memory()
    n_events = int(tracks[:, fields.index("eventID")].max()) + 1
    for _ in range(2):
        grad.lut_value_and_grad(pp, tmpl, host, fields, target, n_events=n_events)
    torch.cuda.synchronize()
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        loss, g = grad.lut_value_and_grad(pp, tmpl, host, fields, target, n_events=n_events)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    # ---- roofline of the dominant kernel, k_lut_pixels<grad>
    # Algorithmic bytes: the fixed per-unit formula of the path (S active
    # segments, P pixels, T ticks, H hits, F_u consumed track columns, W_LUT
    # distinct LUT floats): A_fwd = 4 F_u S + 4 T P + 8 P + 8 H P + 4 W_LUT,
    # A_fwd+bwd = A_fwd + 4 F_u S + 4 T P + 32 S + 4 W_LUT; the pixel kernel is
    # charged A_fwd+bwd - 8 F_u S (the track columns are read by k_segments_lut).
    T, H, F_u = 2000, int(params.MAX_ADC_VALUES), 7
    lut = chain.lut
    w_lut = lut_bytes_touched(seg_rec[ne > 0, 6], lut.n_templates, lut.shape[1], lut.shape[2], SIG_LEN,
                              lut.shape[3])
    a_fwd = 4 * F_u * active + 4 * T * n_pix + 8 * n_pix + 8 * H * n_pix + 4 * w_lut
    a_fb = a_fwd + 4 * F_u * active + 4 * T * n_pix + 4 * 8 * active + 4 * w_lut
    a_kernel = a_fb - 2 * 4 * F_u * active
    # Bytes this design must move in that launch (it keeps waveforms on chip):
    # segment records, slot lists, LUT windows + cumulative sums, main-bin
    # records in and their cotangents out, targets, per-pixel records.
    counts = st.ws[:64].view(torch.int32).cpu().numpy()   # LsimCounts at the workspace start, after the gradient
    n_rec = int(counts[7])                 # main-bin records of the last accumulation
    n_tgt = int(target.pids.numel())
    halo = max(N_NEIGH, 1)
    design_bytes = (192 * active + 4 * n_seg + 8 * (2 * halo + 1) ** 2 * n_pix
                    + 4 * lut.shape[1] * lut.shape[2] * (160 + lut.shape[3])
                    + (656 + 640) * n_rec + (4 + 4 * H) * n_tgt + 48 * n_pix)
    k_ms = float(np.mean(kern_ms))
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = a_kernel / (k_ms * 1e-3) / 1e9
    traffic = None if PIXEL_KERNEL_DRAM_BYTES_PER_PIXEL is None else int(PIXEL_KERNEL_DRAM_BYTES_PER_PIXEL * n_pix)
    rec = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded tracks and LUT)",
        "config": {"workload": f"batched fwd+bwd LUT mode: {args.events} events, log-uniform 1k-50k segments/event "
                               "(tracks + showers), n_neighbors=4, L=150, 100x45x45x1950 templates, "
                               "SSE-ADC loss vs nominal target, params perturbed N(0,5%)",
                   "segments": n_seg, "active_segments": active, "pixels": n_pix, "events": n_events,
                   "l2": "flushed between timed steps (512 MiB write)", "parallelism": f"replicas x{world}",
                   "step": "stage 1 + forward + adjoint replayed as one captured CUDA graph",
                   "launch_shapes": tuned},
        "e2e": {"value": n_seg * world / e2e_s, "unit": UNIT, "ms_per_step": e2e_s * 1e3,
                "h2d_bytes_per_step": int(tracks.nbytes), "d2h_bytes_per_step": 4 * (1 + 8)},
        "roofline": {"bound": "hbm", "kernel": "k_lut_pixels<grad> (pixel-major forward + front end + loss + adjoint)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "algorithmic_bytes": int(a_kernel), "design_bytes": int(design_bytes), "kernel_ms": k_ms,
                     "main_records": n_rec,
                     "peak_source": "measured" if "hbm_gbs" in peaks else "fallback", "traffic": traffic},
        "gpu_launches": KERNELS_PER_STEP * args.steps,
        "clocks": clk,
        "wall_s_timed": wall,
        "loss": float(out[0].item()), "grad_norm": float(out[1:].norm().item()),
    }
    # ---- the plain forward drop-in on the same batch (after the timed region)
    fwd, (wfs_f, unique_f) = lut_forward_record(args, params, tmpl, tracks, fields, dev, flush)
    rec["forward"] = fwd
    # ---- the one-event plain forward (12 muons, about 900 segments): launch-
    # and sync-bound, reported for the configuration the reference runs on CPU
    rec["forward_one_event"] = one_event_forward_record(params, tmpl, dev)
    cpu_leg = rank == 0 and world == 1 and not args.no_cpu_baseline
    if cpu_leg:
        # the oracle reads the template bank the GPU built (the builder itself is
        # compared with the oracle's load_lut in the tests)
        rec["parity"] = forward_parity(params, tmpl.cpu().numpy(), tracks, fields, wfs_f, unique_f)
    del wfs_f, unique_f
    if world == 1:
        # ---- the one-event 500k-segment shower, recompute and store variants
        rec["large_event"] = large_event_record(params, tmpl, dev)
        # ---- the fit loop with the reference's default flags (200 steps)
        rec["fit_loop"] = fit_loop_record(params, tmpl, dev)
        # ---- and with the fitter's default loss, mse_adc on the hits (10 eager steps)
        rec["fit_loop_mse_adc"] = fit_loop_hits_record(params, tmpl, dev)
    if cpu_leg:
        rec["cpu_baseline"] = cpu_baseline(tracks, fields, params, pp, resp, sample_events=8)
    if rank == 0:
        print(json.dumps(rec), flush=True)
    if pg:
        pg.destroy_process_group()


# ---------------------------------------------------------------- CPU side

def _event_sample(tracks, fields, k, chunk=None):
    """k samples from the smallest events; with ``chunk`` each sample is a
    run of ``chunk`` consecutive segments, taken from the smallest events in
    turn until there are k runs."""
    ev = tracks[:, fields.index("eventID")].astype(int)
    counts = np.bincount(ev)
    order = np.argsort(counts, kind="stable")
    out = []
    if chunk:
        for e in order:
            rows = tracks[ev == e]
            for i in range(len(rows) // chunk):
                out.append(rows[i * chunk:(i + 1) * chunk].copy())
                if len(out) == k:
                    break
            if len(out) == k:
                break
    else:
        out = [tracks[ev == e].copy() for e in order[:k]]
    for r in out:
        r[:, fields.index("eventID")] = 0
    return out


def _cpu_target(args_tuple):
    """Target of one sample: the oracle's ADC grid at nominal parameters
    (made once, outside the timed region, as the GPU step's target is)."""
    tmpl_path, tracks, fields, params = args_tuple
    from oracle import reference_np as R
    tmpl = np.load(tmpl_path, mmap_mode="r")
    w, u = R.simulate_wfs(params, tmpl, tracks, fields, history={})
    o = R.simulate_stochastic(params, w, u)
    v = u >= 0
    return u[v], o["grid_adcs"][v]


def _cpu_step(args_tuple):
    """One fwd+bwd of a sample in the reference's arithmetic type: the
    float32 forward of the oracle (waveforms, front end, digitisation, with
    the discrete decisions recorded), the SSE-ADC loss, and the reverse pass
    in float32 down to the 8 parameters."""
    tmpl_path, tracks, fields, pp, tgt_pids, tgt_adc = args_tuple
    from oracle import grad64, reference_np as R
    tmpl = np.load(tmpl_path, mmap_mode="r")
    t0 = time.perf_counter()
    fr = grad64.Frozen(pp, tmpl, tracks, fields, tgt_pids, tgt_adc)
    adc = R.digitize(pp, fr.adc_f32[fr.valid])
    resid = adc - fr.tgt.astype(np.float32)
    float((resid * resid).sum(dtype=np.float32))
    grad64.adjoint64(fr, grad64.theta_dict(pp), g_adc=(2 * resid).astype(np.float32), dtype=np.float32)
    return time.perf_counter() - t0, tracks.shape[0]


def _cpu_jobs(path, sample, fields, params, pp, pool=None):
    targets = (pool.map if pool else map)(_cpu_target, [(path, s, fields, params) for s in sample])
    return [(path, s, fields, pp, tp, ta) for s, (tp, ta) in zip(sample, list(targets))]


def forward_parity(params, tmpl, tracks, fields, wfs, unique, n_events=2):
    """The oracle's forward on the smallest events of the batch against the
    CUDA rows of the same events (events are independent): largest waveform
    deviation relative to each row's scale, and the fraction of front-end
    hit slots whose crossing tick differs (near-threshold crossings) with
    the largest ADC deviation where the ticks agree."""
    import torch
    from larndsim_gb300 import sim
    from oracle import reference_np as R
    col = fields.index("eventID")
    ev = tracks[:, col].astype(np.int64)
    order = np.argsort(np.bincount(ev), kind="stable")[:n_events]
    u = unique.cpu().numpy()
    px, py, plane, pev = R.id2pixel(params, np.maximum(u, 0))
    w_err = a_err = 0.0
    slots = diff = segs = pixels = 0
    for e in order:
        sel = (u >= 0) & (pev == e)
        rows = wfs.index_select(0, torch.from_numpy(np.nonzero(sel)[0]).to(wfs.device))
        one = tracks[ev == e].copy()
        one[:, col] = 0
        wo, uo = R.simulate_wfs(params, tmpl, one, fields, history={})
        v = uo >= 0
        if not np.array_equal(R.pixel2id(params, px[sel], py[sel], plane[sel], 0), uo[v]):
            return {"events": [int(x) for x in order], "unique_pixels_equal": False}
        r_g = rows.cpu().numpy()
        scale = np.abs(wo[v]).max(axis=1, keepdims=True)
        w_err = max(w_err, float((np.abs(r_g - wo[v]) / np.where(scale > 0, scale, 1.0)).max()))
        integral, ticks = sim.get_adc_values(params, rows)
        adc_g, tick_g = R.digitize(params, integral.cpu().numpy()), ticks.cpu().numpy()
        io, to = R.get_adc_values(params, wo[v])
        adc_o = R.digitize(params, io)
        same = np.cumprod(tick_g == to, axis=1).astype(bool)
        slots += same.size
        diff += int((~same).sum())
        if same.any():
            a_err = max(a_err, float((np.abs(adc_g - adc_o) / np.maximum(np.abs(adc_o), 1e-6))[same].max()))
        segs += int(one.shape[0])
        pixels += int(v.sum())
    return {"events": [int(x) for x in order], "segments": segs, "pixels": pixels, "unique_pixels_equal": True,
            "max_wfs_rel": w_err, "hit_slots": slots, "tick_mismatch_slots": diff,
            "tick_mismatch_frac": diff / max(slots, 1), "max_adc_rel_where_ticks_agree": a_err,
            "tolerance": "waveforms 1e-5 of the row scale; ADC 1e-5 relative where the crossing tick agrees"}


def cpu_baseline(tracks, fields, params, pp, resp, sample_events=2, processes=1):
    """CPU restatement timed on the host cores on the smallest events."""
    from oracle import reference_np as R
    tmpl = R.load_lut_templates(resp, params)
    path = tempfile.mktemp(suffix=".npy")
    np.save(path, tmpl)
    del tmpl
    sample = _event_sample(tracks, fields, sample_events)
    jobs = _cpu_jobs(path, sample, fields, params, pp)
    t0 = time.perf_counter()
    if processes > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(processes) as pool:
            res = pool.map(_cpu_step, jobs)
    else:
        res = [_cpu_step(j) for j in jobs]
    wall = time.perf_counter() - t0
    os.unlink(path)
    segs = sum(r[1] for r in res)
    return {"value": segs / wall, "unit": UNIT, "cores": processes, "kind": "port",
            "sample": f"{len(sample)} smallest events ({segs} segments): numpy float32 forward "
                      f"(waveforms, front end, digitisation) + SSE-ADC loss and its float32 reverse-mode "
                      f"gradient in the 8 parameters, {wall:.1f} s; target made outside the timing"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    from larndsim_gb300 import workloads
    params = nominal_params()
    pp = perturbed(params)
    resp = workloads.synthetic_response(seed=0)
    tracks, fields = workload(0, args.seed)
    procs = max(1, min(os.cpu_count() or 1, 16))
    # one step = one sample of `procs` small events processed in parallel
    from oracle import reference_np as R
    tmpl = R.load_lut_templates(resp, params)
    path = tempfile.mktemp(suffix=".npy")
    np.save(path, tmpl)
    del tmpl
    sample = _event_sample(tracks, fields, procs, chunk=CPU_CHUNK)
    times = []
    with mp.get_context("spawn").Pool(procs) as pool:
        jobs = _cpu_jobs(path, sample, fields, params, pp, pool)
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            res = pool.map(_cpu_step, jobs)
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                times.append(dt)
    os.unlink(path)
    segs = sum(len(s) for s in sample)
    ms = float(np.mean(times)) * 1e3
    value = segs / (ms * 1e-3)
    rec = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded tracks and LUT)", "impl": "reference",
           "config": {"workload": "batched fwd+bwd LUT mode (same generator, n_neighbors=4, L=150, "
                                  "100x45x45x1950 templates), CPU sample: consecutive segment runs of the "
                                  "smallest event",
                      "segments_per_step": segs, "samples_per_step": len(sample)},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                            "sample": f"{len(sample)} runs of {CPU_CHUNK} consecutive segments of the smallest "
                                      f"events, {segs} segments per step, one process per run: numpy "
                                      "restatement, float32 forward (waveforms, front end, digitisation) + "
                                      "SSE-ADC loss + float32 reverse-mode gradient in the 8 parameters "
                                      "(the reference's arithmetic type); targets made outside the timing"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(rec), flush=True)


# ---------------------------------------------------------------- chop_tracks

CHOP_SEGMENTS, CHOP_PRECISION, CHOP_CPU_TRACKS = 500_000, 0.001, 20_000


def run_chop(args):
    """On-device chop_tracks (optimize/dataio.py:63-106) of one 500k-segment
    shower event at the reference's default step of 0.001 cm (about 50M
    output rows, 5.2 GB).  value: output rows/s of lsim_chop_tracks with the
    tracks in HBM and the output allocated (one count-and-fill call);
    e2e: dataio.chop_tracks on pinned host tracks (copy in, count, read the
    count, allocate, fill)."""
    import torch
    from larndsim_gb300 import _abi, dataio, sim, workloads
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _abi.load()
    tracks, fields = workloads.large_shower_event(seed=2, n_segments=CHOP_SEGMENTS, n_subtracks=40)
    t = torch.from_numpy(tracks).to(dev)
    fm = _abi.field_map(fields)
    n = t.shape[0]
    ws = torch.empty(lib.lsim_chop_workspace_bytes(n), dtype=torch.uint8, device=dev)
    cnt = torch.zeros(1, dtype=torch.int64, device=dev)
    s = sim._stream()
    _abi.check(lib, lib.lsim_chop_tracks(fm, t.data_ptr(), n, CHOP_PRECISION, None, 0, cnt.data_ptr(),
                                         ws.data_ptr(), ws.numel(), s))
    rows = int(cnt.item())
    out = torch.empty((rows, len(fields)), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step():
        _abi.check(lib, lib.lsim_chop_tracks(fm, t.data_ptr(), n, CHOP_PRECISION, out.data_ptr(), rows,
                                             cnt.data_ptr(), ws.data_ptr(), ws.numel(), s))

    for _ in range(args.warmup):
        step()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(torch.cuda.current_device())
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.fill_(float(i))
        starts[i].record()
        step()
        ends[i].record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = float(np.mean([a.elapsed_time(b) for a, b in zip(starts, ends)]))
    value = rows / (ms * 1e-3)
    host = torch.from_numpy(tracks).pin_memory()
    for _ in range(2):
        dataio.chop_tracks(host, fields, CHOP_PRECISION)
    torch.cuda.synchronize()
    del out
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        r = dataio.chop_tracks(host, fields, CHOP_PRECISION)
        del r
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    algo = 4 * len(fields) * (n + rows)          # read the tracks, write the steps
    achieved = algo / (ms * 1e-3) / 1e9
    rec = {"metric": "chop_tracks steps/s", "value": value, "unit": "steps/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 (float64 step positions)", "data": "synthetic (seeded tracks)",
           "config": {"workload": f"chop_tracks of one {n}-segment shower event (40 sub-tracks) at "
                                  f"{CHOP_PRECISION} cm", "tracks": n, "steps_out": rows, "columns": len(fields),
                      "l2": "flushed between timed steps (512 MiB write); output 5 GB >> L2"},
           "e2e": {"value": rows / e2e_s, "unit": "steps/s", "ms_per_step": e2e_s * 1e3,
                   "h2d_bytes_per_step": int(tracks.nbytes), "d2h_bytes_per_step": 8},
           "roofline": {"bound": "hbm", "kernel": "lsim_chop_tracks (count, scan, offsets, fill; timed together)",
                        "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "algorithmic_bytes": algo,
                        "peak_source": "measured" if "hbm_gbs" in peaks else "fallback", "traffic": None},
           "gpu_launches": 4 * args.steps, "clocks": clk}
    if not args.no_cpu_baseline:
        from oracle import reference_np as R
        sample = tracks[:CHOP_CPU_TRACKS]
        t0 = time.perf_counter()
        ref = R.chop_tracks(sample, fields, CHOP_PRECISION)
        dt = time.perf_counter() - t0
        rec["cpu_baseline"] = {"value": ref.shape[0] / dt, "unit": "steps/s", "cores": 1, "kind": "port",
                               "sample": f"first {CHOP_CPU_TRACKS} tracks ({ref.shape[0]} steps), vectorised "
                                         f"numpy restatement, {dt:.2f} s"}
    print(json.dumps(rec), flush=True)


# ---------------------------------------------------------------- probabilistic front end

PROB_EVENTS, PROB_CPU_PIXELS = 8, 16


def _prob_workload(seed=0):
    """Waveforms (valid rows) of the first 8 events of the batched
    workload, LUT mode n_neighbors = 4, L = 150, noise width 900 e-."""
    from larndsim_gb300 import sim, workloads
    params = nominal_params().replace(RESET_NOISE_CHARGE=900.0)
    tmpl, params = sim.load_lut(workloads.synthetic_response(seed=0), params)
    tracks, fields = workload(0, seed, n_events=PROB_EVENTS)
    wfs, unique = sim.simulate_wfs(params, tmpl, tracks, fields)
    return params, wfs[unique >= 0].contiguous()


def run_prob(args):
    """The beam search of get_adc_values_average_noise_vmap
    (fee_jax.py:386-461) with the reductions of get_average_hit_values
    fused in (lsim_fee_prob), on every simulated pixel of 8 events.
    value: pixels/s with the waveforms in HBM; e2e: pinned host waveforms
    in, the three (P, H) reductions out."""
    import torch
    from larndsim_gb300 import sim
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    params, wfs = _prob_workload(args.seed)
    P = wfs.shape[0]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=wfs.device)
    for _ in range(args.warmup):
        sim.average_hit_values(params, wfs)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(torch.cuda.current_device())
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.fill_(float(i))
        starts[i].record()
        sim.average_hit_values(params, wfs)
        ends[i].record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = float(np.mean([a.elapsed_time(b) for a, b in zip(starts, ends)]))
    host = wfs.cpu().pin_memory()
    e2e_steps = max(3, min(args.steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        out = [t.cpu() for t in sim.average_hit_values(params, host)]
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    H = int(params.MAX_ADC_VALUES)
    # forward + adjoint with cotangents on the expected values (the collapsed-hit loss case)
    wg = wfs.clone().requires_grad_(True)
    cot = [torch.randn((P, H), device=wfs.device) for _ in range(3)]

    def fwd_bwd():
        wg.grad = None
        et, ea, lam = sim.average_hit_values(params, wg)
        torch.autograd.backward([et, ea, lam], cot)
        return wg.grad

    fwd_bwd()
    torch.cuda.synchronize()
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n_fb = 2
    b0.record()
    for _ in range(n_fb):
        fwd_bwd()
    b1.record()
    torch.cuda.synchronize()
    fb_ms = b0.elapsed_time(b1) / n_fb
    rec = {"metric": "probabilistic FEE pixels/s", "value": P / (ms * 1e-3), "unit": "pixels/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded tracks and LUT)",
           "config": {"workload": f"beam search (fee_paths_scaling={int(params.fee_paths_scaling)}, H={H}, "
                                  f"RESET_NOISE_CHARGE=900) on the {P} simulated pixels of {PROB_EVENTS} events of "
                                  "the batched LUT workload (n_neighbors=4, L=150), expected tick / ADC / hit "
                                  "probability fused", "pixels": P, "ticks": int(wfs.shape[1]),
                      "l2": "flushed between timed steps (512 MiB write)"},
           "e2e": {"value": P / e2e_s, "unit": "pixels/s", "ms_per_step": e2e_s * 1e3,
                   "h2d_bytes_per_step": int(host.numel() * 4), "d2h_bytes_per_step": int(3 * P * H * 4)},
           "roofline": {"bound": "issue", "kernel": "k_fee_prob",
                        "note": "transcendental-function bound (erf/erfc, log, exp, expm1 per path and tick); "
                                "HBM traffic is the waveform read only"},
           "gpu_launches": 2 * args.steps, "clocks": clk,
           "fwd_bwd": {"ms": fb_ms, "pixels_per_s": P / (fb_ms * 1e-3),
                       "note": "forward with the step paths recorded + lsim_fee_prob_vjp (reverse pass per tick class), "
                               "cotangents on the expected tick, ADC and hit probability"}}
    if not args.no_cpu_baseline:
        from oracle import reference_np as R
        sample = wfs[:PROB_CPU_PIXELS].cpu().numpy()
        t0 = time.perf_counter()
        R.get_average_hit_values(*(lambda lp, q: (np.exp(lp), R.digitize(params, q)))(
            *R.get_adc_values_average_noise(params, sample)))
        dt = time.perf_counter() - t0
        rec["cpu_baseline"] = {"value": PROB_CPU_PIXELS / dt, "unit": "pixels/s", "cores": 1, "kind": "port",
                               "sample": f"first {PROB_CPU_PIXELS} pixels, float32 numpy restatement, {dt:.1f} s"}
    print(json.dumps(rec), flush=True)


# ---------------------------------------------------------------- plain forward

def _timed(step, steps, warmup, flush):
    import torch
    for _ in range(warmup):
        step()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    clocks = ClockSampler(torch.cuda.current_device())
    torch.cuda.synchronize()
    for i in range(steps):
        flush.fill_(float(i))
        starts[i].record()
        step()
        ends[i].record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    return float(np.mean([a.elapsed_time(b) for a, b in zip(starts, ends)])), clk


def lut_forward_record(args, params, tmpl, tracks, fields, dev, flush):
    """The plain LUT-mode forward drop-in, simulate_wfs + simulate_stochastic
    (sim_jax.py:689-769), through the public functions with the reference's
    device-to-host synchronisation points: device-resident ms per step,
    e2e from pinned host tracks to host hits, and the roofline of the
    waveform kernel k_lut_pixels<wfs> (CUDA events around its launch)
    against the fixed forward formula.  Returns the record and the last
    step's (wfs, unique)."""
    import torch
    from larndsim_gb300 import _abi, grad, sim
    n_seg = tracks.shape[0]
    t_dev = torch.from_numpy(tracks).to(dev)

    def step(tr=t_dev):
        wfs, unique = sim.simulate_wfs(params, tmpl, tr, fields)
        return sim.simulate_stochastic(params, wfs, unique), wfs, unique

    ms, clk = _timed(step, args.steps, args.warmup, flush)
    rec = {"metric": "forward segments/s", "value": n_seg / (ms * 1e-3), "unit": "segments/s",
           "ms_per_step": ms, "steps": args.steps, "warmup": args.warmup,
           "workload": f"simulate_wfs + simulate_stochastic (n_neighbors=4, L=150, 100x45x45x1950 templates) on "
                       f"the same batch ({n_seg} segments), noise off",
           "step": "public functions, eager, with the reference's device-to-host syncs; L2 flushed between "
                   "timed steps (512 MiB write)",
           "clocks": clk}
    host = torch.from_numpy(tracks).pin_memory()
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d2h = 0
    for _ in range(e2e_steps):
        out = step(host.to(dev, non_blocking=True))[0]
        cpu = [o.cpu() for o in out]
        d2h = sum(c.numel() * 4 for c in cpu)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    rec["e2e"] = {"value": n_seg / e2e_s, "unit": "segments/s", "ms_per_step": e2e_s * 1e3,
                  "h2d_bytes_per_step": int(tracks.nbytes), "d2h_bytes_per_step": int(d2h)}
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
    for e in kev:
        flush.fill_(1.0)
        _abi.set_kernel_events(*e)
        _, wfs, unique = step()
    torch.cuda.synchronize()
    _abi.set_kernel_events(None, None)
    k_ms = float(np.mean([a.elapsed_time(b) for a, b in kev]))
    n_valid = int((unique >= 0).sum())
    T = wfs.shape[1]
    # the waveform kernel's share of the fixed forward formula: the rows it
    # writes (4 T P), their pixel ids (8 P) and the distinct LUT floats
    chain = grad.LUTChain(params, tmpl, tracks, fields)
    st = chain.stage1(params)
    seg_rec = st.ws[256:256 + 96 * n_seg].view(torch.int32).view(n_seg, 24).cpu().numpy()
    ne = seg_rec[:, 0].view(np.float32)
    lut = chain.lut
    w_lut = lut_bytes_touched(seg_rec[ne > 0, 6], lut.n_templates, lut.shape[1], lut.shape[2], SIG_LEN,
                              lut.shape[3])
    algo = 4 * T * n_valid + 8 * n_valid + 4 * w_lut
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = algo / (k_ms * 1e-3) / 1e9
    rec["roofline"] = {"bound": "hbm", "kernel": "k_lut_pixels<wfs> (pixel-major waveform accumulation)",
                       "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                       "algorithmic_bytes": int(algo), "kernel_ms": k_ms, "pixels": n_valid,
                       "peak_source": "measured" if "hbm_gbs" in peaks else "fallback", "traffic": None}
    return rec, (wfs, unique)


def large_event_record(params, tmpl, dev, reps=5):
    """Forward + adjoint of the SSE-ADC loss on one 500k-segment shower
    event (40 sub-tracks): the recomputing adjoint (waveforms never stored)
    against the store-the-waveforms variant, device time per gradient call
    (CUDA events around stage 1 + the gradient call) and peak device memory
    of each: the bytes torch's allocator held for this event at its peak
    (tracks, stage-1 workspace, transient buffers of the call) above what
    was resident before, plus the template bank it reads."""
    import torch
    from larndsim_gb300 import grad, workloads
    tracks, fields = workloads.large_shower_event(seed=0, n_segments=500_000, n_subtracks=40)
    torch.cuda.synchronize()
    resident = torch.cuda.memory_allocated(dev)
    bank = tmpl.numel() * tmpl.element_size()
    chain = grad.LUTChain(params, tmpl, torch.from_numpy(tracks).to(dev), fields)
    target = chain.target(params)
    pp = perturbed(params)
    out = {"workload": f"one shower event, {tracks.shape[0]} segments around 40 sub-tracks, n_neighbors=4, L=150",
           "segments": int(tracks.shape[0])}
    for name, fn in (("recompute", lambda: chain.loss_and_grad_device(pp, target)),
                     ("store", lambda: chain.loss_and_grad_stored(pp, target))):
        fn()
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats(dev)
        before = torch.cuda.memory_allocated(dev)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in ev:
            a.record()
            fn()
            b.record()
        torch.cuda.synchronize()
        ms = float(np.median([a.elapsed_time(b) for a, b in ev]))
        out[name] = {"ms": ms, "segments_per_s": tracks.shape[0] / (ms * 1e-3),
                     "peak_device_bytes": int(torch.cuda.max_memory_allocated(dev) - resident + bank),
                     "call_transient_bytes": int(torch.cuda.max_memory_allocated(dev) - before)}
    out["pixels"] = int(chain._stage.n_valid)
    return out


def one_event_forward_record(params, tmpl, dev, reps=20):
    """simulate_wfs + simulate_stochastic on one event of 12 straight muons
    cut into 0.4 cm segments (about 900 segments), through the public
    functions with the reference's host synchronisation points: median
    device-inclusive wall time per call with the tracks on the device, and
    e2e from pinned host tracks to host hits."""
    import torch
    from larndsim_gb300 import sim, workloads
    tracks, fields = workloads.muon_event(seed=0, n_tracks=12)
    t_dev = torch.from_numpy(tracks).to(dev)
    host = torch.from_numpy(tracks).pin_memory()

    def call(tr):
        wfs, unique = sim.simulate_wfs(params, tmpl, tr, fields)
        return sim.simulate_stochastic(params, wfs, unique)

    for _ in range(3):
        call(t_dev)
    torch.cuda.synchronize()
    dev_s, e2e_s = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        out = call(t_dev)
        torch.cuda.synchronize()
        dev_s.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        out = [o.cpu() for o in call(host.to(dev, non_blocking=True))]
        e2e_s.append(time.perf_counter() - t0)
    ms, e2e_ms = 1e3 * float(np.median(dev_s)), 1e3 * float(np.median(e2e_s))
    n = int(tracks.shape[0])
    return {"workload": f"one event, 12 straight muons, {n} segments, n_neighbors=4, L=150, full template bank",
            "segments": n, "ms": ms, "segments_per_s": n / (ms * 1e-3), "e2e_ms": e2e_ms,
            "e2e_segments_per_s": n / (e2e_ms * 1e-3), "hits": int(out[0].shape[0]),
            "timing": "host wall clock per call (median of 20), the call's own device-to-host syncs included"}


def run_forward(args, param_mode=False):
    """The plain forward drop-in on the 64-event batch: simulate_wfs +
    simulate_stochastic (sim_jax.py:689-769), or simulate_parametrized
    (sim_jax.py:339-372, n_neighbors = 0, Monte-Carlo diffusion offsets
    supplied), through the public functions with the reference's host
    synchronisation points.  LUT mode also reports the roofline of the
    waveform kernel k_lut_pixels<wfs> (CUDA events around its launch)."""
    import torch
    from larndsim_gb300 import sim, workloads
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    tracks, fields = workload(0, args.seed)
    n_seg = tracks.shape[0]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    base = {"metric": "forward segments/s", "unit": "segments/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded tracks and LUT)"}
    if not param_mode:
        params = nominal_params()
        tmpl, params = sim.load_lut(workloads.synthetic_response(seed=0), params)
        fwd, _ = lut_forward_record(args, params, tmpl, tracks, fields, dev, flush)
        rec = dict(base, value=fwd["value"], ms_per_step=fwd["ms_per_step"],
                   config={"workload": fwd["workload"], "segments": n_seg,
                           "l2": "flushed between timed steps (512 MiB write)", "step": fwd["step"]},
                   clocks=fwd["clocks"], e2e=fwd["e2e"], roofline=fwd["roofline"], gpu_launches=None)
        print(json.dumps(rec), flush=True)
        return
    t_dev = torch.from_numpy(tracks).to(dev)
    params = nominal_params().replace(number_pix_neighbors=0, mc_diff=True)
    offsets = sim.draw_offsets(n_seg, 7, dev)

    def step(tr=t_dev, off=offsets):
        return sim.simulate_parametrized(params, tr, fields, offsets=off)

    ms, clk = _timed(step, args.steps, args.warmup, flush)
    rec = dict(base, value=n_seg / (ms * 1e-3), ms_per_step=ms,
               config={"workload": f"simulate_parametrized (n_neighbors=0, mc_diff offsets supplied) on the "
                                   f"64-event batch ({n_seg} segments), noise off",
                       "segments": n_seg, "l2": "flushed between timed steps (512 MiB write)",
                       "step": "public functions, eager, with the reference's device-to-host syncs"},
               clocks=clk)
    host = torch.from_numpy(tracks).pin_memory()
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d2h = 0
    for _ in range(e2e_steps):
        out = step(host.to(dev, non_blocking=True), offsets)
        cpu = [o.cpu() for o in out]
        d2h = sum(c.numel() * 4 for c in cpu)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    rec["e2e"] = {"value": n_seg / e2e_s, "unit": "segments/s", "ms_per_step": e2e_s * 1e3,
                  "h2d_bytes_per_step": int(tracks.nbytes), "d2h_bytes_per_step": int(d2h)}
    rec["gpu_launches"] = None
    print(json.dumps(rec), flush=True)


# ---------------------------------------------------------------- fit loop

FIT_EVENTS, FIT_SEGMENTS, FIT_STEPS, FIT_LR, FIT_SEED = 32, 20_000, 200, 1e-3, 77


def fit_loop_record(params, tmpl, dev, steps=FIT_STEPS):
    """The fit loop of the reference's GradientDescentFitter with its default
    flags (sigmoid normalisation, optax.adam, no clipping; optimize/
    fit_params.py:781-895, example_run.py) on 32 events x 20k segments:
    ``steps`` steps on the 7 parameters the loss depends on (vdrift does not
    enter), target simulated at hidden parameters drawn from N(nominal, 5 %)
    inside the ranges.  Device steps/s of the loop (stage 1, forward +
    adjoint, optimiser update replayed as one CUDA graph per step) and e2e
    (pinned host tracks in, the fit set up, the steps, the final parameters
    read back)."""
    import torch
    from larndsim_gb300 import fit, grad, workloads
    from larndsim_gb300.grad import GRAD_PARAMS
    names = tuple(k for k in GRAD_PARAMS if k != "vdrift")
    tracks, fields = workloads.batched_events(seed=FIT_SEED, n_events=FIT_EVENTS, min_segments=FIT_SEGMENTS,
                                              max_segments=FIT_SEGMENTS + 1)
    rng = np.random.default_rng(FIT_SEED)
    hid = {}
    for k in names:
        r = fit.RANGES[k]
        hid[k] = float(np.clip(float(getattr(params, k)) * (1.0 + 0.05 * rng.standard_normal()), r["down"], r["up"]))
    hidden = params.replace(**hid)
    t_dev = torch.from_numpy(tracks).to(dev)
    target = grad.LUTChain(params, tmpl, t_dev, fields).target(hidden)

    def make(tr):
        return fit.DeviceFit(params, tmpl, tr, fields, target, fit_params=names, lr=FIT_LR,
                             normalization_scheme="sigmoid", max_steps=steps + 8)

    f = make(t_dev)
    f.capture()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(torch.cuda.current_device())
    torch.cuda.synchronize()
    start.record()
    for _ in range(steps):
        f.graph.replay()
    end.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = start.elapsed_time(end) / steps
    loss, th = f.history()
    err = {k: float(th[-1, GRAD_PARAMS.index(k)] / hid[k] - 1.0) for k in names}
    err0 = {k: float(float(getattr(params, k)) / hid[k] - 1.0) for k in names}
    host = torch.from_numpy(tracks).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g = make(host.to(dev, non_blocking=True))
    g.run(steps, graph=True)
    final = g.theta.cpu()
    e2e_s = time.perf_counter() - t0
    return {"workload": f"GradientDescentFitter loop, {FIT_EVENTS} events x {FIT_SEGMENTS} segments "
                        f"({tracks.shape[0]} segments), n_neighbors=4, L=150, 100x45x45x1950 templates, SSE-ADC "
                        f"loss, 7 parameters, sigmoid normalisation, Adam lr {FIT_LR}, {steps} steps",
            "segments": int(tracks.shape[0]), "steps": steps, "ms_per_step": ms, "steps_per_s": 1e3 / ms,
            "step": "stage 1 + forward + adjoint + optimiser update, one CUDA graph replay per step",
            "loss_first": float(loss[0]), "loss_last": float(loss[-1]),
            "start_rel_error": err0, "final_rel_error": err,
            "e2e": {"steps_per_s": steps / e2e_s, "seconds": e2e_s, "h2d_bytes": int(tracks.nbytes)},
            "final_theta": [float(x) for x in final], "clocks": clk}


def fit_loop_hits_record(params, tmpl, dev, steps=10):
    """The reference fitter with its default loss (mse_adc on the simulated
    hits, GenericLossStrategy; sigmoid normalisation, Adam) on the same 32
    events x 20k segments: ``steps`` eager steps (forward to ADCs, hits,
    mse_adc and its gradient, the LUT adjoint, the update; the hit count is
    read on the host every step), host wall clock per step."""
    import torch
    from larndsim_gb300 import fit, losses, strategies, workloads
    from larndsim_gb300.grad import GRAD_PARAMS
    names = tuple(k for k in GRAD_PARAMS if k != "vdrift")
    tracks, fields = workloads.batched_events(seed=FIT_SEED, n_events=FIT_EVENTS, min_segments=FIT_SEGMENTS,
                                              max_segments=FIT_SEGMENTS + 1)
    rng = np.random.default_rng(FIT_SEED)
    hid = {}
    for k in names:
        r = fit.RANGES[k]
        hid[k] = float(np.clip(float(getattr(params, k)) * (1.0 + 0.05 * rng.standard_normal()), r["down"], r["up"]))
    t_dev = torch.from_numpy(tracks).to(dev)
    h = strategies.LUTSimulation(tmpl).predict(params.replace(**hid), t_dev, fields, 0)
    ref = (losses.adc2charge(h["adcs"], params), h["pixel_x"], h["pixel_y"], h["pixel_z"], h["ticks"],
           h["hit_prob"], h["event"])
    f = fit.DeviceFit(params, tmpl, t_dev, fields, fit_params=names, lr=FIT_LR, normalization_scheme="sigmoid",
                      loss_fn=losses.mse_adc, ref_hits=ref, max_steps=steps + 2)
    f.step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    f.run(steps)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / steps
    loss, _ = f.history()
    return {"workload": f"GradientDescentFitter with its default loss (mse_adc on the hits, sigma 1, lambda_Q 1), "
                        f"{FIT_EVENTS} events x {FIT_SEGMENTS} segments, 7 parameters, sigmoid, Adam lr {FIT_LR}",
            "reference_hits": int(ref[0].shape[0]), "steps": steps, "ms_per_step": ms, "steps_per_s": 1e3 / ms,
            "timing": "host wall clock over the eager steps (each reads its hit count on the host)",
            "loss_first": float(loss[0]), "loss_last": float(loss[-1])}


def run_fit(args):
    """``fit_loop_record`` as its own line (metric fit steps/s)."""
    import torch
    from larndsim_gb300 import sim, workloads
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    params = nominal_params()
    tmpl, params = sim.load_lut(workloads.synthetic_response(seed=0), params)
    r = fit_loop_record(params, tmpl, dev)
    rec = {"metric": "fit steps/s", "value": r["steps_per_s"], "unit": "steps/s", "n_gpus": 1, "steps": r["steps"],
           "warmup": 1, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded tracks and LUT)",
           "config": {"workload": r["workload"], "segments": r["segments"], "step": r["step"],
                      "l2": "inputs and work set larger than L2"},
           "fit": {k: r[k] for k in ("loss_first", "loss_last", "start_rel_error", "final_rel_error")},
           "e2e": {"value": r["e2e"]["steps_per_s"], "unit": "steps/s", "seconds": r["e2e"]["seconds"],
                   "h2d_bytes_per_step": r["e2e"]["h2d_bytes"] // r["steps"], "d2h_bytes_per_step": 0},
           "gpu_launches": (KERNELS_PER_STEP + 1) * r["steps"], "clocks": r["clocks"],
           "final_theta": r["final_theta"]}
    print(json.dumps(rec), flush=True)


def run_param_grad(args):
    """Parametrised mode fwd+bwd on the 64-event batch: waveforms at the
    perturbed parameters (offsets fixed), front end, SSE against the ADCs
    at the nominal parameters, and dL/dtheta through lsim_fee_vjp and
    lsim_param_wfs_vjp (torch autograd composes them)."""
    import torch
    from larndsim_gb300 import grad, sim
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    tracks, fields = workload(0, args.seed)
    n_seg = tracks.shape[0]
    t_dev = torch.from_numpy(tracks).to(dev)
    params = nominal_params().replace(number_pix_neighbors=0, mc_diff=True)
    offsets = sim.draw_offsets(n_seg, 7, dev)
    with torch.no_grad():
        w0, u0 = sim.param_wfs_fn(grad.theta_of(params, device=dev), params, t_dev, fields, offsets)
        a0, _ = sim.fee_adc(params, w0[u0 >= 0])
    pp = params.replace(lifetime=float(params.lifetime) * 1.05, Ab=float(params.Ab) * 0.97)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step(tr=t_dev):
        theta = grad.theta_of(pp, device=dev).requires_grad_(True)
        wfs, unique = sim.param_wfs_fn(theta, pp, tr, fields, offsets)
        adc, _ = sim.fee_adc(pp, wfs[unique >= 0])
        loss = ((adc - a0) ** 2).sum()
        loss.backward()
        return loss.detach(), theta.grad

    ms, clk = _timed(step, args.steps, args.warmup, flush)
    host = torch.from_numpy(tracks).pin_memory()
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        loss, g = step(host.to(dev, non_blocking=True))
        vals = (float(loss), g.cpu())
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    rec = {"metric": "parametrised fwd+bwd segments/s", "value": n_seg / (ms * 1e-3), "unit": "segments/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded tracks)",
           "config": {"workload": f"parametrised mode (n_neighbors=0, mc_diff offsets fixed) on the 64-event batch "
                                  f"({n_seg} segments): waveforms, front end, SSE-ADC loss against the nominal "
                                  "parameters' ADCs, gradient in the 8 parameters (eager, waveforms stored)",
                      "segments": n_seg, "l2": "flushed between timed steps (512 MiB write)"},
           "e2e": {"value": n_seg / e2e_s, "unit": "segments/s", "ms_per_step": e2e_s * 1e3,
                   "h2d_bytes_per_step": int(tracks.nbytes), "d2h_bytes_per_step": 4 * (1 + 8)},
           "clocks": clk, "gpu_launches": None}
    print(json.dumps(rec), flush=True)


# ---------------------------------------------------------------- hit-level fit loss

def run_loss(args):
    """mse_adc (losses_jax.py:60-79) forward + gradient with respect to the
    hit charges and z, on the hits of the 64-event batch simulated at the
    perturbed parameters against those at the nominal ones."""
    import torch
    from larndsim_gb300 import grad, losses, sim, workloads
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    params = nominal_params()
    tmpl, params = sim.load_lut(workloads.synthetic_response(seed=0), params)
    tracks, fields = workload(0, args.seed)
    chain = grad.LUTChain(params, tmpl, tracks, fields)
    with torch.no_grad():
        ref = [t.detach() for t in grad.predicted_hits(grad.theta_of(params, device="cuda"), chain, params)]
        pred = [t.detach() for t in grad.predicted_hits(grad.theta_of(perturbed(params), device="cuda"), chain,
                                                        perturbed(params))]
    Q, x, y, z, t, hp, ev = pred
    n, m = Q.shape[0], ref[0].shape[0]

    def step():
        q = Q.clone().requires_grad_(True)
        zz = z.clone().requires_grad_(True)
        loss, _ = losses.mse_adc(params, q, x, y, zz, t, hp, ev, *ref)
        loss.backward()
        return loss

    for _ in range(args.warmup):
        step()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(torch.cuda.current_device())
    torch.cuda.synchronize()
    for i in range(args.steps):
        starts[i].record()
        step()
        ends[i].record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = float(np.mean([a.elapsed_time(b) for a, b in zip(starts, ends)]))
    counts = torch.bincount(ev.long()).cpu().numpy().astype(np.float64)
    rcounts = torch.bincount(ref[6].long()).cpu().numpy().astype(np.float64)
    k = min(len(counts), len(rcounts))
    pairs = float((counts ** 2).sum() + (rcounts ** 2).sum() + (counts[:k] * rcounts[:k]).sum())
    host = [a.cpu().pin_memory() for a in pred + ref]
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        hq = host[0].cuda(non_blocking=True).requires_grad_(True)
        hz = host[3].cuda(non_blocking=True).requires_grad_(True)
        rest = [a.cuda(non_blocking=True) for a in host]
        loss, _ = losses.mse_adc(params, hq, rest[1], rest[2], hz, rest[4], rest[5], rest[6], *rest[7:])
        loss.backward()
        out = (float(loss.detach()), hq.grad.cpu(), hz.grad.cpu())
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    rec = {"metric": "mse_adc fwd+bwd hits/s", "value": n / (ms * 1e-3), "unit": "hits/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded tracks and LUT)",
           "config": {"workload": f"mse_adc (sigma=1, lambda_Q=1) of the {n} predicted vs {m} reference hits of the "
                                  "64-event batch, loss + dL/dQ + dL/dz", "hits": n, "ref_hits": m,
                      "same_event_pair_terms": pairs, "l2": "working set < L2 (hits only)"},
           "e2e": {"value": n / e2e_s, "unit": "hits/s", "ms_per_step": e2e_s * 1e3,
                   "h2d_bytes_per_step": int(sum(a.numel() * 4 for a in host)), "d2h_bytes_per_step": 4 + 8 * n},
           "roofline": {"bound": "issue", "kernel": "k_rbf_rows",
                        "note": "pairwise exp per same-event pair; inputs are a few MB"},
           "gpu_launches": 7 * args.steps, "clocks": clk}
    if not args.no_cpu_baseline:
        from oracle import losses_np as L
        e0 = (ev == 0).cpu().numpy()
        r0 = (ref[6] == 0).cpu().numpy()
        a = [v.cpu().numpy() for v in pred]
        b = [v.cpu().numpy() for v in ref]
        t0 = time.perf_counter()
        L.mse_adc(a[0][e0], a[1][e0], a[2][e0], a[3][e0], a[5][e0], a[6][e0], b[0][r0], b[1][r0], b[2][r0],
                  b[3][r0], b[5][r0], b[6][r0])
        L.mse_adc_grad(a[0][e0], a[1][e0], a[2][e0], a[3][e0], a[6][e0], b[0][r0], b[1][r0], b[2][r0], b[3][r0],
                       b[6][r0])
        dt = time.perf_counter() - t0
        rec["cpu_baseline"] = {"value": float(e0.sum()) / dt, "unit": "hits/s", "cores": 1, "kind": "port",
                               "sample": f"event 0 ({int(e0.sum())} hits vs {int(r0.sum())}), float64 numpy "
                                         f"restatement, loss + gradients, {dt:.2f} s"}
    print(json.dumps(rec), flush=True)


def run_chop_reference(args):
    """CPU arm of --path chop: the numpy restatement of chop_tracks, one
    bounded sample (the first 20k tracks of the same event) per step."""
    if dist_env()[0] != 0:
        return
    from larndsim_gb300 import workloads
    from oracle import reference_np as R
    tracks, fields = workloads.large_shower_event(seed=2, n_segments=CHOP_SEGMENTS, n_subtracks=40)
    sample = tracks[:CHOP_CPU_TRACKS]
    times, rows = [], 0
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        rows = R.chop_tracks(sample, fields, CHOP_PRECISION).shape[0]
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    ms = float(np.mean(times)) * 1e3
    value = rows / (ms * 1e-3)
    print(json.dumps({"metric": "chop_tracks steps/s", "value": value, "unit": "steps/s", "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
                      "data": "synthetic (seeded tracks)",
                      "config": {"workload": f"chop_tracks at {CHOP_PRECISION} cm, first {CHOP_CPU_TRACKS} "
                                             "tracks of the 500k-segment shower event", "steps_out": rows},
                      "cpu_baseline": {"value": value, "unit": "steps/s", "cores": 1, "kind": "port",
                                       "sample": f"{CHOP_CPU_TRACKS} tracks, {rows} steps per step"},
                      "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


# ---------------------------------------------------------------- output side

RECORDS_HITS, RECORDS_EVENTS, RECORDS_CPU_HITS = 32_000_000, 1000, 4_000_000
# DRAM bytes per input hit of one lsim_hit_records call (three kernels), from
# an ncu capture of an 8M-hit case (575.3 MB; traffic scales with the hits)
RECORDS_DRAM_BYTES_PER_HIT = 575_320_064 / 8_000_000


def _records_workload(n, seed=0):
    """Hit columns of the shape simulate_stochastic returns: events sorted
    (hits come out pixel-major, pixel ids packing the event), ADCs on the
    digitisation range with 1% at the lowest ADC (dropped), 0.5% event -1."""
    from larndsim_gb300 import consts, output
    rng = np.random.default_rng(seed)
    params = consts.Params()
    ev = np.sort(rng.integers(0, RECORDS_EVENTS, n)).astype(np.int32)
    ev[rng.random(n) < 0.005] = -1
    adc = rng.uniform(75.8, 256, n).astype(np.float32)
    adc[rng.random(n) < 0.01] = np.float32(output.adc_lowest(params))
    cols = [adc, rng.uniform(-30, 30, n).astype(np.float32), rng.uniform(-60, 60, n).astype(np.float32),
            rng.uniform(-30, 30, n).astype(np.float32), rng.integers(0, 1997, n).astype(np.float32),
            np.ones(n, np.float32), ev, rng.integers(0, 1 << 30, n).astype(np.int32)]
    return params, cols


def run_records(args):
    """Hit records of the simulate driver (optimize/simulate.py:129-176) on
    32M synthetic hits of 1000 events.  value: input hits/s of
    lsim_hit_records with the columns in HBM (3 launches: tile summaries,
    scan, write); e2e: output.hit_records on pinned host columns plus the
    copy of the records back to host memory."""
    import torch
    from larndsim_gb300 import _abi, output, sim
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _abi.load()
    n = args.hits or RECORDS_HITS
    params, cols = _records_workload(n)
    din = [torch.from_numpy(c).to(dev) for c in cols]
    names = ("adc", "pix_x", "pix_y", "pix_z", "ticks", "hit_prob", "event", "pixels")
    dout = [torch.empty_like(c) for c in din]
    clean, q = torch.empty(n, dtype=torch.float32, device=dev), torch.empty(n, dtype=torch.float32, device=dev)
    run_event = torch.empty(n, dtype=torch.int32, device=dev)
    run_start = torch.empty(n + 1, dtype=torch.int64, device=dev)
    counts = torch.zeros(2, dtype=torch.int64, device=dev)
    ws = torch.empty(lib.lsim_hit_records_workspace_bytes(n), dtype=torch.uint8, device=dev)
    lp = _abi.make_params(params)
    lo = output.adc_lowest(params)
    cin = _abi.LsimHitColumns(*[c.data_ptr() for c in din])
    cout = _abi.LsimHitColumns(*[c.data_ptr() for c in dout])
    s = sim._stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step():
        _abi.check(lib, lib.lsim_hit_records(lp, lo, cin, n, cout, clean.data_ptr(), q.data_ptr(),
                                             run_event.data_ptr(), run_start.data_ptr(), counts.data_ptr(),
                                             ws.data_ptr(), ws.numel(), s))

    for _ in range(args.warmup):
        step()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(torch.cuda.current_device())
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.fill_(float(i))
        starts[i].record()
        step()
        ends[i].record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    kept, runs = (int(v) for v in counts.cpu().tolist())
    ms = float(np.mean([a.elapsed_time(b) for a, b in zip(starts, ends)]))
    host = [torch.from_numpy(c).pin_memory() for c in cols]
    del din, dout, clean, q, run_event, run_start, ws

    def e2e_step():
        rec = output.hit_records(params, host)
        return {k: v.cpu() for k, v in rec.items()}

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        back = e2e_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    d2h = int(sum(v.numel() * v.element_size() for v in back.values()))
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    algo = 32 * n + 40 * kept + 12 * runs + 8    # read 8 columns, write 10 kept columns and the runs
    achieved = algo / (ms * 1e-3) / 1e9
    rec = {"metric": "hit records hits/s", "value": n / (ms * 1e-3), "unit": "hits/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32/int32", "data": "synthetic (seeded hit columns)",
           "config": {"workload": f"hit records (clean mask, compaction, charge, event runs) of {n} hits of "
                                  f"{RECORDS_EVENTS} events", "hits": n, "kept": kept, "runs": runs,
                      "l2": f"flushed between timed steps (512 MiB write); columns {32 * n / 1e9:.2f} GB in, "
                            f"{40 * kept / 1e9:.2f} GB out"},
           "e2e": {"value": n / e2e_s, "unit": "hits/s", "ms_per_step": e2e_s * 1e3,
                   "h2d_bytes_per_step": int(sum(c.nbytes for c in cols)), "d2h_bytes_per_step": d2h},
           "roofline": {"bound": "hbm", "kernel": "lsim_hit_records (3 launches timed together)",
                        "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "algorithmic_bytes": algo,
                        "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                        "traffic": int(RECORDS_DRAM_BYTES_PER_HIT * n)},
           "gpu_launches": 3 * args.steps, "clocks": clk}
    if not args.no_cpu_baseline:
        from oracle import reference_np as R
        m = min(RECORDS_CPU_HITS, n)
        t0 = time.perf_counter()
        r = R.hit_records(params, *[c[:m] for c in cols])
        R.hit_records_by_event(r)
        dt = time.perf_counter() - t0
        rec["cpu_baseline"] = {"value": m / dt, "unit": "hits/s", "cores": 1, "kind": "port",
                               "sample": f"first {m} hits: numpy restatement (mask, compaction, charge, "
                                         f"per-event split), {dt:.2f} s"}
    print(json.dumps(rec), flush=True)


def run_records_reference(args):
    """CPU arm of --path records: the numpy restatement (mask, compaction,
    charge and the per-event split of simulate.py:129-156) on the first 4M
    hits of the same columns per step."""
    if dist_env()[0] != 0:
        return
    from oracle import reference_np as R
    params, cols = _records_workload(RECORDS_HITS)
    m = RECORDS_CPU_HITS
    sample = [c[:m] for c in cols]
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        R.hit_records_by_event(R.hit_records(params, *sample))
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    ms = float(np.mean(times)) * 1e3
    value = m / (ms * 1e-3)
    print(json.dumps({"metric": "hit records hits/s", "value": value, "unit": "hits/s", "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f32/int32", "impl": "reference",
                      "data": "synthetic (seeded hit columns)",
                      "config": {"workload": f"hit records of the first {m} of {RECORDS_HITS} hits"},
                      "cpu_baseline": {"value": value, "unit": "hits/s", "cores": 1, "kind": "port",
                                       "sample": f"{m} hits per step"},
                      "e2e": {"value": value, "unit": "hits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


def main():
    args = parse()
    if args.path == "records":
        (run_records_reference if args.impl == "reference" else run_records)(args)
        return
    if args.path == "fit":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "fit path: its CPU arm is the default path's "
                                                                  "fwd+bwd restatement"}))
        else:
            run_fit(args)
        return
    if args.path == "param_grad":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "param_grad path: no CPU arm"}))
        else:
            run_param_grad(args)
        return
    if args.path in ("forward", "param"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "forward paths: the reference arm of the "
                                                                  "default path times the CPU restatement"}))
        else:
            run_forward(args, param_mode=args.path == "param")
        return
    if args.path == "loss":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "loss path: its CPU arm is the cpu_baseline of "
                                                                  "--path loss (the numpy restatement)"}))
        else:
            run_loss(args)
        return
    if args.path == "prob":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "prob path: its CPU arm is the cpu_baseline of "
                                                                  "--path prob (the numpy restatement)"}))
        else:
            run_prob(args)
        return
    if args.path == "chop":
        if args.impl == "reference":
            run_chop_reference(args)
        else:
            run_chop(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
