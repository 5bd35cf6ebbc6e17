"""Input side of the simulate path (reference: optimize/dataio.py).

``chop_tracks`` cuts tracks into fixed-length steps on the GPU
(``lsim_chop_tracks``), with the reference's name, arguments and result
rows; the result is a float32 CUDA tensor, ready for ``simulate_wfs`` or
``simulate_parametrized``.  ``TracksDataset`` gives the reference's batches
of whole events, assembled on the GPU from a track table kept in device
memory.  There is no CPU fallback.
"""

from __future__ import annotations

import numpy as np
import torch
from numpy.lib import recfunctions as rfn

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


# ---------------------------------------------------------------- tracks dataset

_RENAME = {"event_id": "eventID", "traj_id": "trackID"}
_ZERO_PAD_FIELDS = ("n_electrons", "dE", "dEdx", "dx", "long_diff", "tran_diff")
_NEG_ONE_PAD_FIELDS = ("trackID", "pixel_plane")


def read_segments(source):
    """The ``segments`` table: a structured array given directly, or read
    from an HDF5 file (needs h5py)."""
    if isinstance(source, np.ndarray) and source.dtype.names:
        return source.copy()
    try:
        import h5py
    except ImportError as e:
        raise ImportError("reading an HDF5 segments file needs h5py; pass the structured segments array instead") from e
    with h5py.File(source, "r") as f:
        return f["segments"][:]


def np_from_structured(tracks):
    """Structured rows as an (N, F) float32 array (optimize/dataio.py:42-45)."""
    return np.asarray(rfn.structured_to_unstructured(tracks, copy=True, dtype=np.float32), dtype=np.float32)


def remap_event_ids_to_local(batch_arr, source_event_ids, batch_event_ids, fields):
    """Replace the eventID column by the position of each row's event in the
    sorted ``batch_event_ids`` (optimize/dataio.py:47-61); raises ValueError
    when an event is missing."""
    col = tuple(fields).index("eventID")
    src = np.asarray(source_event_ids, dtype=np.int64)
    if src.size == 0:
        return batch_arr
    local = _local_event_ids(src, np.asarray(batch_event_ids, dtype=np.int64))
    batch_arr[:, col] = local.astype(np.float32)
    return batch_arr


def _local_event_ids(src, batch_events):
    local = np.searchsorted(batch_events, src)
    if np.any(local >= batch_events.size) or not np.array_equal(batch_events[local], src):
        missing = np.setdiff1d(np.unique(src), batch_events)
        raise ValueError(f"Failed to remap eventID to local indices. Missing global eventID values: "
                         f"{missing[:16].tolist()}")
    return local


def _swap_xz(tracks):
    for a, b in (("x_start", "z_start"), ("x_end", "z_end"), ("x", "z")):
        xa = np.copy(tracks[a])
        tracks[a] = np.copy(tracks[b])
        tracks[b] = xa


class _DeviceBatches:
    """Device assembly shared by the two datasets: the table in HBM as
    float32, the batch rows gathered with their local event ids, chopped and
    padded with the reference's invalidated rows."""

    def _init_device(self, fields):
        self._evt_col = fields.index("eventID")
        self._roles = np.zeros(len(fields), dtype=np.int8)
        for name in _ZERO_PAD_FIELDS:
            if name in fields:
                self._roles[fields.index(name)] = 1
        for name in _NEG_ONE_PAD_FIELDS:
            if name in fields:
                self._roles[fields.index(name)] = 2
        self._table = None
        self._batch_dev = {}

    def _device_table(self):
        if self._table is None:
            self._table = torch.from_numpy(np_from_structured(self.tracks_struct)).to(sim._device())
        return self._table

    def _batch_index(self, idx):
        if idx not in self._batch_dev:
            rows = np.asarray(self.batch_row_indices[idx], dtype=np.int64)
            local = _local_event_ids(self.tracks_struct[rows]["eventID"].astype(np.int64),
                                     self.batch_event_global_ids[idx])
            dev = sim._device()
            self._batch_dev[idx] = (torch.from_numpy(rows).to(dev),
                                    torch.from_numpy(local.astype(np.float32)).to(dev))
        return self._batch_dev[idx]

    def _assemble(self, idx, fields):
        lib = _abi.load()
        table = self._device_table()
        rows, local = self._batch_index(idx)
        n, nf = rows.numel(), len(fields)
        out = torch.empty((n, nf), dtype=torch.float32, device=table.device)
        status = torch.zeros(1, dtype=torch.int32, device=table.device)
        _abi.check(lib, lib.lsim_gather_tracks(sim._ptr(table), table.shape[0], nf, sim._ptr(rows), n,
                                               self._evt_col, sim._ptr(local), sim._ptr(out), sim._ptr(status),
                                               sim._stream()))
        if self.chopped and n > 0:
            out = chop_tracks(out, fields, precision=self.electron_sampling_resolution)
        if int(status.item()) != 0:
            raise ValueError("batch row index outside the track table")
        if self.pad and self.max_batch_nsteps > 0 and out.shape[0] < self.max_batch_nsteps:
            out = self.pad_batch(out, self.max_batch_nsteps, idx)
        return out

    def pad_batch(self, batch_arr, target_len, idx=None):
        """Pad to ``target_len`` rows with invalidated rows and invalidate rows
        whose event is not a local event of batch ``idx`` (dataio.py:357-373,
        :525-542).  Returns a new float32 CUDA tensor."""
        lib = _abi.load()
        b = torch.as_tensor(batch_arr).to(device=sim._device(), dtype=torch.float32)
        cur = b.shape[0]
        out = torch.empty((max(cur, int(target_len)), b.shape[1]), dtype=torch.float32, device=b.device)
        out[:cur].copy_(b)
        n_local = len(self.batch_event_global_ids[idx]) if idx is not None else -1
        roles = self._roles.ctypes.data_as(_abi.C.c_void_p)
        _abi.check(lib, lib.lsim_pad_tracks(sim._ptr(out), cur, int(target_len), b.shape[1], self._evt_col, roles,
                                            n_local, sim._stream()))
        return out

    def get_batch_global_event_ids(self, idx=None):
        return self.batch_event_global_ids if idx is None else self.batch_event_global_ids[idx]


class TracksDataset(_DeviceBatches):
    """Batches of whole events from a segments table
    (TracksDataset, optimize/dataio.py:108-424).

    The batch layout (which trajectories and events form each batch, the
    local event ids, the padded step count) is host bookkeeping with the
    reference's rules and gives the same batches.  The rows themselves are
    assembled on the GPU: the table is kept in device memory as float32,
    ``ds[i]`` gathers the batch's rows with their local event ids
    (``lsim_gather_tracks``), chops them (``lsim_chop_tracks``) and pads
    them (``lsim_pad_tracks``), and returns a float32 CUDA tensor.
    ``filename`` may be the structured segments array itself (HDF5 reading
    needs h5py).
    """

    def __init__(self, filename, nevents, max_nbatch=None, swap_xz=True, random_nevents=False, data_seed=42,
                 track_len_sel=2., max_abs_costheta_sel=0.966, min_abs_segz_sel=15., track_z_bound=28.,
                 max_batch_len=50, print_input=False, chopped=True, pad=True, electron_sampling_resolution=0.1,
                 live_selection=False):
        tracks = read_segments(filename)
        if swap_xz:
            _swap_xz(tracks)
        if "t0" not in tracks.dtype.names:
            tracks = rfn.append_fields(tracks, "t0", np.zeros(tracks.shape[0]), usemask=False)
        self.track_fields = tuple(_RENAME.get(f, f) for f in tracks.dtype.names)
        tracks.dtype.names = self.track_fields
        if max_batch_len is not None and max_nbatch is not None and max_nbatch > 0:
            tracks = self._trim_to_budget(tracks, max_batch_len * (max_nbatch + 2))
        traj_rows = self._trajectory_rows(tracks, live_selection, track_len_sel, max_abs_costheta_sel,
                                          min_abs_segz_sel, track_z_bound)
        self.tracks_struct = tracks
        traj_event = np.array([tracks[r[0]]["eventID"] for r in traj_rows])
        traj_rows = self._select_events(traj_rows, traj_event, nevents, random_nevents, data_seed)
        self.trajectory_row_indices = traj_rows
        if max_batch_len is not None:
            self.batch_traj_indices, tot = self._pack_events(traj_rows, max_batch_len, max_nbatch)
        else:
            self.batch_traj_indices = [[i] for i in range(len(traj_rows))]
            tot = np.sum([tracks[r]["dx"].sum() for r in traj_rows])
        if min(len(b) for b in self.batch_traj_indices) == 0:
            raise ValueError("There exist some empty batch in the simulation input!")
        self.batch_nsteps, self.batch_row_keys, self.batch_event_global_ids, self.batch_row_indices = [], [], [], []
        for b in self.batch_traj_indices:
            rows = np.concatenate([traj_rows[t] for t in b])
            dx = tracks[rows]["dx"]
            self.batch_nsteps.append(int(np.sum(np.maximum(np.ceil(dx / electron_sampling_resolution), 1)
                                                .astype(int))))
            keys = np.ascontiguousarray(np.unique(tracks[rows][["eventID", "trackID"]]))
            self.batch_row_keys.append(keys)
            self.batch_event_global_ids.append(np.asarray(np.unique(keys["eventID"]), dtype=np.int64))
            self.batch_row_indices.append(np.asarray(rows, dtype=np.int64))
        self.max_batch_nsteps = int(max(self.batch_nsteps)) if self.batch_nsteps else 0
        self.chopped, self.pad, self.print_input = chopped, pad, print_input
        self.electron_sampling_resolution = electron_sampling_resolution
        self.tot_data_length = tot
        self._init_device(self.track_fields)

    # -- layout (host)

    @staticmethod
    def _trim_to_budget(tracks, budget):
        """Keep whole events up to a cumulative track length (dataio.py:148-160)."""
        cum = np.cumsum(tracks["dx"])
        cut = int(np.searchsorted(cum, budget, side="left"))
        if cut < len(tracks):
            other = tracks["eventID"][:cut + 1] != tracks["eventID"][cut]
            if other.any():
                tracks = tracks[:int(np.flatnonzero(other)[-1]) + 1]
        return tracks

    @staticmethod
    def _trajectory_rows(tracks, live_selection, track_len_sel, max_abs_costheta_sel, min_abs_segz_sel,
                         track_z_bound):
        """Row lists of the (eventID, trackID) trajectories (dataio.py:165-218).
        With live_selection the keys come from the selected rows and, as in
        the reference, their positions index the full table."""
        if live_selection:
            sel = tracks[abs(tracks["z"]) < min_abs_segz_sel]
            _, first = np.unique(sel[["eventID", "trackID"]], return_index=True)
            first = np.sort(first)
            last = np.r_[first[1:] - 1, len(sel) - 1]
            a, b = sel[first], sel[last]
            d = np.column_stack((a["x_start"] - b["x_end"], a["y_start"] - b["y_end"], a["z_start"] - b["z_end"]))
            cos = np.abs(np.dot(d, np.array([0, 0, 1]))) / (np.linalg.norm(d, axis=1) + 1e-10)
            ok = (np.sqrt(d[:, 0] ** 2 + d[:, 1] ** 2 + d[:, 2] ** 2) > track_len_sel) & (cos < max_abs_costheta_sel)
            ok &= np.maximum(abs(a["z"]), abs(b["z"])) < track_z_bound
            keys = np.ascontiguousarray(sel[np.repeat(ok, last - first + 1)][["eventID", "trackID"]])
        else:
            keys = np.ascontiguousarray(tracks[["eventID", "trackID"]])
        uniq, inv = np.unique(keys, return_inverse=True)
        order = np.argsort(inv)
        vals = inv[order]
        present, starts = np.unique(vals, return_index=True)
        ends = np.append(starts[1:], len(vals))
        rows = [np.empty(0, dtype=int) for _ in range(len(uniq))]
        for v, s, e in zip(present, starts, ends):
            rows[int(v)] = order[s:e]
        return rows

    @staticmethod
    def _select_events(traj_rows, traj_event, nevents, random_nevents, data_seed):
        """The first (or seeded random) nevents events (dataio.py:227-246)."""
        if nevents is None or nevents <= 0:
            return traj_rows
        events, first = np.unique(traj_event, return_index=True)
        ordered = events[np.argsort(first)]
        if random_nevents:
            rng = np.random.default_rng(seed=data_seed)
            chosen = rng.choice(ordered, size=nevents, replace=False) if nevents < len(ordered) else ordered
        else:
            chosen = ordered[:nevents]
        return [traj_rows[i] for i in np.flatnonzero(np.isin(traj_event, chosen))]

    def _pack_events(self, traj_rows, max_batch_len, max_nbatch):
        """Whole events packed into batches by the floor of their cumulative
        length over max_batch_len (dataio.py:251-296)."""
        tracks = self.tracks_struct
        length = np.array([tracks[r]["dx"].sum() for r in traj_rows])
        valid = np.flatnonzero(length <= max_batch_len)
        lengths = length.copy()[length <= max_batch_len]
        if lengths.size == 0:
            raise ValueError("All tracks are longer than the batch size! Please check.")
        ev = np.array([tracks[traj_rows[v][0]]["eventID"] for v in valid])
        uniq, inv = np.unique(ev, return_inverse=True)
        groups = [[] for _ in range(len(uniq))]
        ev_len = np.zeros(len(uniq))
        for pos, (k, ln) in enumerate(zip(inv, lengths)):
            groups[k].append(valid[pos])
            ev_len[k] += ln
        cum = np.cumsum(ev_len)
        splits = np.flatnonzero(np.diff(np.floor_divide(cum, max_batch_len)) > 0) + 1
        splits = np.insert(np.append(splits, len(cum)), 0, 0)
        if max_nbatch and max_nbatch > 0:
            splits = splits[:max_nbatch + 1]
        batches = [[t for k in range(splits[i], splits[i + 1]) for t in groups[k]] for i in range(len(splits) - 1)]
        return batches, cum[splits[-1] - 1]

    def __len__(self):
        return len(self.batch_traj_indices)

    def __getitem__(self, idx):
        """Batch ``idx`` as an (n, F) float32 CUDA tensor (dataio.py:378-406)."""
        if idx < 0 or idx >= len(self):
            raise IndexError("Batch index out of range")
        return self._assemble(idx, self.track_fields)

    def get_track_fields(self):
        return self.track_fields

    def get_batch_row_keys(self):
        return self.batch_row_keys

    def get_batch_row_indices(self, idx=None):
        return self.batch_row_indices if idx is None else self.batch_row_indices[idx]


def _pack_keys(event_ids, track_ids):
    """(eventID, trackID) pairs as uint64 keys, event in the high 32 bits."""
    e = np.asarray(event_ids, dtype=np.int64).astype(np.uint64)
    t = np.asarray(track_ids, dtype=np.int64).astype(np.uint64)
    return (e << np.uint64(32)) | (t & np.uint64(0xFFFFFFFF))


class TgtTracksDataset(_DeviceBatches):
    """Target batches matched to a simulation dataset's batches
    (TgtTracksDataset, optimize/dataio.py:426-640): batch i holds every
    target row whose (eventID, trackID) key is one of the keys of the
    simulation dataset's batch i, in table order, with the simulation
    batch's local event ids; chopped and padded like TracksDataset, on the
    GPU.  ``filename`` may be the structured target segments array."""

    def __init__(self, filename, dataset_sim, swap_xz=True, chopped=True, pad=True, electron_sampling_resolution=0.1,
                 print_input=False):
        self.chopped, self.pad, self.print_input = chopped, pad, print_input
        self.electron_sampling_resolution = electron_sampling_resolution
        self.swap_xz = swap_xz
        self.sim_track_fields = dataset_sim.get_track_fields()
        tracks = read_segments(filename)
        if "t0" not in tracks.dtype.names:
            tracks = rfn.append_fields(tracks, "t0", np.zeros(tracks.shape[0]), usemask=False)
        self.tgt_track_fields = tuple(_RENAME.get(f, f) for f in tracks.dtype.names)
        tracks.dtype.names = self.tgt_track_fields
        if swap_xz:
            _swap_xz(tracks)
        self.tracks_struct = tracks
        keys = _pack_keys(tracks["eventID"], tracks["trackID"])
        order = np.argsort(keys)
        self._key_order = order
        self._keys, self._key_starts = np.unique(keys[order], return_index=True)
        self._key_ends = np.append(self._key_starts[1:], len(order))
        self.batch_keys = dataset_sim.get_batch_row_keys()
        self.batch_event_global_ids = dataset_sim.get_batch_global_event_ids()
        self.batch_row_indices, self.batch_nsteps = [], []
        self.tot_data_length = 0
        for keys_b in self.batch_keys:
            if keys_b.size == 0:
                self.batch_row_indices.append(np.empty((0,), dtype=int))
                self.batch_nsteps.append(0)
                continue
            rows = self._rows_for_key_ids(np.unique(_pack_keys(keys_b["eventID"], keys_b["trackID"])))
            self.batch_row_indices.append(rows)
            if rows.size == 0:
                self.batch_nsteps.append(0)
            else:
                dx = tracks[rows]["dx"]
                self.batch_nsteps.append(int(np.sum(np.maximum(np.ceil(dx / electron_sampling_resolution), 1)
                                                    .astype(int))))
                self.tot_data_length += np.sum(dx)
        self.max_batch_nsteps = int(max(self.batch_nsteps)) if self.batch_nsteps else 0
        self.n_batches = len(self.batch_keys)
        self._init_device(self.tgt_track_fields)

    def _rows_for_key_ids(self, key_ids):
        """Sorted target rows of the given keys; every key must be present
        (dataio.py:577-599)."""
        left = np.searchsorted(self._keys, key_ids, side="left")
        right = np.searchsorted(self._keys, key_ids, side="right")
        missing = left == right
        if missing.any():
            miss = key_ids[missing][:16]
            pairs = list(zip((miss >> np.uint64(32)).astype(np.int64).tolist(),
                             (miss & np.uint64(0xFFFFFFFF)).astype(np.int64).tolist()))
            raise ValueError(f"{int(missing.sum())} of {len(key_ids)} sim key(s) are absent from the target file. "
                             f"Missing (eventID, trackID) sample: {pairs}")
        chunks = [self._key_order[self._key_starts[u]:self._key_ends[u]] for lo, hi in zip(left, right)
                  for u in range(lo, hi)]
        return np.sort(np.concatenate(chunks)) if chunks else np.empty((0,), dtype=int)

    def __len__(self):
        return self.n_batches

    def __getitem__(self, idx):
        """Target batch ``idx`` as an (n, F) float32 CUDA tensor (dataio.py:604-626)."""
        if idx < 0 or idx >= self.n_batches:
            raise IndexError("TgtTracksDataset index out of range")
        if self.batch_row_indices[idx].size == 0:
            return torch.empty((0, len(self.tgt_track_fields)), dtype=torch.float32, device=sim._device())
        return self._assemble(idx, self.tgt_track_fields)

    def get_track_fields(self):
        return self.tgt_track_fields


class DataLoader:
    """Groups of ``batch_size`` dataset items (optimize/dataio.py:9-40); the
    items are CUDA tensors, stacked on the device."""

    def __init__(self, dataset, batch_size):
        self.dataset, self.batch_size = dataset, batch_size
        self.index = 0
        self.indices = np.arange(len(dataset))

    def __iter__(self):
        self.index = 0
        return self

    def __getitem__(self, idx):
        return self.dataset[idx]

    def __next__(self):
        if self.index >= len(self.dataset):
            raise StopIteration
        items = [self.dataset[int(i)] for i in self.indices[self.index:self.index + self.batch_size]]
        self.index += self.batch_size
        return torch.stack(items)

    def __len__(self):
        return (len(self.dataset) + self.batch_size - 1) // self.batch_size
