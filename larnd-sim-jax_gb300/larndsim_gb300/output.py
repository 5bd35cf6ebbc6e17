"""Output side of the simulate driver (reference: optimize/simulate.py:129-176).

``hit_records`` turns the 8 outputs of ``simulate_stochastic`` /
``simulate_parametrized`` into the records the reference's driver writes:
the hits whose ADC differs from ``digitize(DISCRIMINATION_THRESHOLD)`` and
whose event is not -1, with the cleaned ADC and the charge in ke-, plus the
runs of equal event that split them per event -- all on the GPU
(``lsim_hit_records``); there is no CPU fallback.  The writers produce the
driver's two formats: the flat ``--out_np`` archive (``write_hits_npz``) and
the per-batch, per-event groups (``write_hits_h5`` with h5py, or the same
layout in an ``.npz`` with ``write_hits_groups_npz``).
"""

from __future__ import annotations

import numpy as np
import torch

from . import _abi, sim

GROUP_FIELDS = ("adc_clean", "adc", "Q", "pixels", "ticks", "eventID", "pix_x", "pix_y", "pix_z")
_COLUMNS = ("adc", "pix_x", "pix_y", "pix_z", "ticks", "hit_prob", "event", "pixels")


def adc_lowest(params) -> float:
    """digitize(params, DISCRIMINATION_THRESHOLD) in float32 (simulate.py:129)."""
    f = np.float32
    x = (f(params.DISCRIMINATION_THRESHOLD) * f(params.GAIN) + f(params.V_PEDESTAL)) - f(params.V_CM)
    y = (np.maximum(x, f(0)) * f(params.ADC_COUNTS)) / f(params.V_REF - params.V_CM)
    return float(np.minimum(y, f(params.ADC_COUNTS)))


class HitRecords(dict):
    """Kept hit columns (CUDA tensors: adc, adc_clean, Q, pix_x, pix_y, pix_z,
    ticks, hit_prob, event, pixels) and the event runs (``run_event``,
    ``run_start`` with the kept count appended)."""

    def by_event(self, global_event_ids=None):
        """One group per local event id >= 0, keyed by its global id, with the
        reference's dataset names (simulate.py:139-156).  Host arrays."""
        if "run_start" not in self:
            raise ValueError("these records were made with runs=False: no event runs to split by")
        starts = self["run_start"].cpu().numpy()
        events = self["run_event"].cpu().numpy()
        host = {k: self[k].cpu().numpy() for k in ("adc_clean", "adc", "Q", "pixels", "ticks", "pix_x", "pix_y",
                                                   "pix_z")}
        l2g = {i: int(g) for i, g in enumerate(global_event_ids)} if global_event_ids is not None else {}
        groups = {}
        for local in np.unique(events).astype(int):
            if local < 0:
                continue
            runs = np.flatnonzero(events == local)
            g = l2g.get(local, local)
            if runs.size == 1:
                sl = slice(starts[runs[0]], starts[runs[0] + 1])
                grp = {k: v[sl] for k, v in host.items()}
            else:
                idx = np.concatenate([np.arange(starts[r], starts[r + 1]) for r in runs])
                grp = {k: v[idx] for k, v in host.items()}
            grp["eventID"] = np.full(grp["adc"].shape[0], g, dtype=np.int64)
            groups[g] = {k: grp[k] for k in GROUP_FIELDS}
        return groups

    def flat(self):
        """The ``--out_np`` columns of this batch (simulate.py:168-176)."""
        return {"adcs": self["adc"], "Q": self["Q"], "x": self["pix_x"], "y": self["pix_y"], "z": self["pix_z"],
                "ticks": self["ticks"], "hit_prob": self["hit_prob"], "event_id": self["event"]}


def hit_records(params, outputs, adc_lowest_value=None, runs=True) -> HitRecords:
    """Records of one batch from ``(adcs, pixel_x, pixel_y, pixel_z, ticks,
    hit_prob, event, hit_pixels)`` (simulate.py:129-133)."""
    if len(outputs) != 8:
        raise ValueError(f"expected the 8 simulate outputs, got {len(outputs)}")
    lib = _abi.load()
    dev = sim._device()
    cols = []
    for i, t in enumerate(outputs):
        dt = torch.int32 if i >= 6 else torch.float32
        cols.append(torch.as_tensor(t).to(device=dev, dtype=dt).reshape(-1).contiguous())
    n = cols[0].numel()
    if any(c.numel() != n for c in cols):
        raise ValueError("the hit columns differ in length")
    lowest = adc_lowest(params) if adc_lowest_value is None else float(adc_lowest_value)
    out = {k: torch.empty(n, dtype=c.dtype, device=dev) for k, c in zip(_COLUMNS, cols)}
    clean = torch.empty(n, dtype=torch.float32, device=dev)
    q = torch.empty(n, dtype=torch.float32, device=dev)
    run_event = torch.empty(n, dtype=torch.int32, device=dev) if runs else None
    run_start = torch.empty(n + 1, dtype=torch.int64, device=dev) if runs else None
    counts = torch.zeros(2, dtype=torch.int64, device=dev)
    ws = torch.empty(max(lib.lsim_hit_records_workspace_bytes(n), 1), dtype=torch.uint8, device=dev)
    p = sim._ptr
    cin = _abi.LsimHitColumns(*[p(c) for c in cols])
    cout = _abi.LsimHitColumns(*[p(out[k]) for k in _COLUMNS])
    _abi.check(lib, lib.lsim_hit_records(_abi.make_params(params), lowest, cin, n, cout, p(clean), p(q),
                                         p(run_event), p(run_start), p(counts), p(ws), ws.numel(), sim._stream()))
    n_kept, n_runs = (int(v) for v in counts.cpu().tolist())
    rec = HitRecords({k: v[:n_kept] for k, v in out.items()})
    rec["adc_clean"] = clean[:n_kept]
    rec["Q"] = q[:n_kept]
    if runs:
        rec["run_event"] = run_event[:n_runs]
        rec["run_start"] = run_start[:n_runs + 1]
    return rec


def write_hits_npz(path, batches):
    """The ``--out_np`` archive: the batches' kept columns concatenated
    (simulate.py:168-179; keys adcs, Q, x, y, z, ticks, hit_prob, event_id)."""
    flats = [b.flat() for b in batches]
    keys = ("adcs", "Q", "x", "y", "z", "ticks", "hit_prob", "event_id")
    arrays = {k: np.concatenate([f[k].cpu().numpy() for f in flats]) if flats else np.zeros(0, np.float32)
              for k in keys}
    np.savez(path, **arrays)


def _groups(batches, global_event_ids):
    for ib, rec in enumerate(batches):
        gids = None if global_event_ids is None else global_event_ids[ib]
        yield ib, rec.by_event(gids)


def write_hits_h5(path, batches, global_event_ids=None):
    """Groups ``batch_{i}/event_{global id}`` with the reference's datasets
    (simulate.py:135-156).  Needs h5py."""
    try:
        import h5py
    except ImportError as e:
        raise ImportError("write_hits_h5 needs h5py; write_hits_groups_npz writes the same layout to an .npz") from e
    with h5py.File(path, "a") as f:
        for ib, groups in _groups(batches, global_event_ids):
            bg = f.create_group(f"batch_{ib}")
            for g, grp in groups.items():
                eg = bg.create_group(f"event_{g}")
                for name in GROUP_FIELDS:
                    eg.create_dataset(name, data=grp[name])


def write_hits_groups_npz(path, batches, global_event_ids=None):
    """The per-event layout of ``write_hits_h5`` as ``.npz`` keys
    ``batch_{i}/event_{global id}/{dataset}``."""
    arrays = {}
    for ib, groups in _groups(batches, global_event_ids):
        for g, grp in groups.items():
            for name in GROUP_FIELDS:
                arrays[f"batch_{ib}/event_{g}/{name}"] = grp[name]
    np.savez(path, **arrays)
