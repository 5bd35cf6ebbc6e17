"""Autotuner for the launch shapes of the LUT kernels.

The shapes that matter on a given GPU and workload are the number of
persistent pixel-kernel blocks per SM and the grid and block size of the
segment-major main-bin kernels.  ``autotune`` times a step function under
each candidate shape (CUDA events, median of a few repetitions), keeps the
fastest and applies it through ``lsim_set_tuning``; results are cached per
device and workload key.  Every shape computes bit-identical results (the
per-pixel and per-segment records do not depend on which warp computes
them), so tuning never changes numbers.
"""

from __future__ import annotations

import ctypes as C
import itertools

import numpy as np
import torch

from . import _abi


class LsimTuning(C.Structure):
    _fields_ = [("pixel_blocks_per_sm", C.c_int32), ("main_blocks", C.c_int32), ("main_block_warps", C.c_int32),
                ("reserved", C.c_int32 * 5)]


FIELDS = ("pixel_blocks_per_sm", "main_blocks", "main_block_warps")
DEFAULT_CANDIDATES = tuple(
    dict(zip(FIELDS, v)) for v in itertools.product((0, 4, 3), (512, 1024, 2048), (8, 4)))
_cache: dict = {}


def set_tuning(cfg=None):
    """Apply a launch shape (dict with FIELDS; None or zeros: defaults) to
    this thread's later LUT calls."""
    lib = _abi.load()
    if cfg is None:
        lib.lsim_set_tuning(None)
        return
    t = LsimTuning(*(int(cfg.get(k, 0)) for k in FIELDS))
    lib.lsim_set_tuning(C.byref(t))


def autotune(step, key=None, candidates=DEFAULT_CANDIDATES, reps=3, warmup=1):
    """Time ``step()`` under each candidate shape; apply and return the
    fastest as (cfg, {shape: ms})."""
    dev = torch.cuda.get_device_name()
    ck = (dev, key)
    if key is not None and ck in _cache:
        set_tuning(_cache[ck][0])
        return _cache[ck]
    times = {}
    for cfg in candidates:
        set_tuning(cfg)
        for _ in range(warmup):
            step()
        ms = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            step()
            b.record()
            b.synchronize()
            ms.append(a.elapsed_time(b))
        times[tuple(cfg[k] for k in FIELDS)] = float(np.median(ms))
    best = min(times, key=times.get)
    cfg = dict(zip(FIELDS, best))
    set_tuning(cfg)
    result = (cfg, times)
    if key is not None:
        _cache[ck] = result
    return result
