"""Input side of the simulate path (reference: optimize/dataio.py).

``chop_tracks`` cuts tracks into fixed-length steps on the GPU
(``lsim_chop_tracks``), with the reference's name, arguments and result
rows; the result is a float32 CUDA tensor, ready for ``simulate_wfs`` or
``simulate_parametrized``.  There is no CPU fallback.
"""

from __future__ import annotations

import torch

from . import _abi, sim


def chop_tracks(tracks, fields, precision=0.001):
    """Cut every track into max(ceil(length / precision), 1) steps
    (optimize/dataio.py:63-106).

    ``tracks`` is an (N, F) float32 array or tensor with the columns named
    in ``fields``; the rows of track i come before those of track i + 1.
    Raises ValueError, as the reference does, when a track length is not
    finite.
    """
    lib = _abi.load()
    fields = tuple(fields)
    t = sim.as_tracks(tracks)
    if t.dim() != 2 or t.shape[1] != len(fields):
        raise ValueError(f"tracks of shape {tuple(t.shape)} do not match {len(fields)} fields")
    precision = float(precision)
    if not precision > 0:
        raise ValueError(f"precision must be positive, got {precision}")
    fm = _abi.field_map(fields)
    n = t.shape[0]
    ws = torch.empty(max(lib.lsim_chop_workspace_bytes(n), 1), dtype=torch.uint8, device=t.device)
    count = torch.zeros(1, dtype=torch.int64, device=t.device)
    s = sim._stream()
    _abi.check(lib, lib.lsim_chop_tracks(fm, sim._ptr(t), n, precision, None, 0, sim._ptr(count), sim._ptr(ws),
                                         ws.numel(), s))
    total = int(count.item())
    if total < 0:
        raise ValueError("chop_tracks: a track length is not finite")
    out = torch.empty((total, len(fields)), dtype=torch.float32, device=t.device)
    if total:
        _abi.check(lib, lib.lsim_chop_tracks(fm, sim._ptr(t), n, precision, sim._ptr(out), total, sim._ptr(count),
                                             sim._ptr(ws), ws.numel(), s))
    return out
