"""Golden batches of the reference's TracksDataset (optimize/dataio.py:108-424).

Imports optimize/dataio.py of larnd-sim-jax with a stand-in ``h5py`` module
whose ``File(name)["segments"]`` returns a seeded synthetic structured
array (the reference reads that dataset and nothing else), builds the
dataset under several option sets and stores, per case, every batch
``ds[i]``, the per-batch global event ids and source rows, the padded
step count, the total track length and one ``pad_batch`` call, in
dataset_ref.npz; and the target batches of TgtTracksDataset (:426-640) for
a second seeded table (other energy deposits, shuffled rows, one extra
event) matched to two of those cases.  Both structured arrays are stored
too, so the tests feed the same rows to the GB300 implementation.
Generated with NumPy 2.

Usage: python tests/golden/make_dataset_golden.py /path/to/larnd-sim-jax   (or LARNDSIM_JAX_SRC=/path/to/larnd-sim-jax)
"""

import importlib.util
import os
import sys
import types
from pathlib import Path

import numpy as np

# the larnd-sim-jax source tree: the first argument, or LARNDSIM_JAX_SRC
REF = Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LARNDSIM_JAX_SRC", ""))
if not (REF / "src" / "larndsim").is_dir():
    raise SystemExit(f"{Path(__file__).name}: give the larnd-sim-jax source tree as the first argument "
                     "or in LARNDSIM_JAX_SRC")
OUT = Path(__file__).resolve().parent / "dataset_ref.npz"

# HDF5 field names of the reference's segments dataset (event_id / traj_id
# are renamed to eventID / trackID by the loader; t0 is appended when absent)
NAMES = ("event_id", "traj_id", "x_start", "y_start", "z_start", "x_end", "y_end", "z_end", "x", "y", "z",
         "t", "t_start", "t_end", "t0_start", "t0_end", "dx", "dE", "dEdx", "n_electrons", "n_photons",
         "long_diff", "tran_diff", "pixel_plane", "pdgId")
INT_NAMES = {"event_id", "traj_id", "pixel_plane", "pdgId"}


def make_segments(seed=0, n_events=9):
    """Events with a few trajectories each; every trajectory a straight line
    cut into 0.3-0.6 cm segments.  Global event ids are not contiguous."""
    rng = np.random.default_rng(seed)
    dtype = np.dtype([(n, "i4" if n in INT_NAMES else "f4") for n in NAMES])
    rows = []
    event_ids = np.sort(rng.choice(np.arange(100, 200), n_events, replace=False))
    for ev in event_ids:
        for traj in range(int(rng.integers(1, 5))):
            start = rng.uniform(-25, 25, 3)
            u = rng.standard_normal(3)
            u /= np.linalg.norm(u)
            length = rng.uniform(0.5, 14.0)
            seg = rng.uniform(0.3, 0.6)
            n = max(int(length / seg), 1)
            edges = start + np.outer(np.linspace(0, length, n + 1), u)
            for k in range(n):
                s, e = edges[k], edges[k + 1]
                r = {name: 0 for name in NAMES}
                r.update(event_id=ev, traj_id=traj + 10 * int(rng.integers(0, 3)), pixel_plane=0, pdgId=13)
                r.update(x_start=s[0], y_start=s[1], z_start=s[2], x_end=e[0], y_end=e[1], z_end=e[2])
                r.update(x=0.5 * (s[0] + e[0]), y=0.5 * (s[1] + e[1]), z=0.5 * (s[2] + e[2]))
                r.update(dx=np.linalg.norm(e - s), dE=rng.uniform(0.1, 1.5), t=rng.uniform(0, 5))
                r["dEdx"] = r["dE"] / r["dx"]
                r.update(t_start=r["t"], t_end=r["t"] + 0.01, n_electrons=r["dE"] * 4e4, long_diff=0.0,
                         tran_diff=0.0, n_photons=1.0)
                rows.append(tuple(r[nm] for nm in NAMES))
    return np.array(rows, dtype=dtype)


CASES = {
    "batched": dict(nevents=6, max_batch_len=25.0, chopped=True, pad=True, electron_sampling_resolution=0.1),
    "one_traj_per_batch": dict(nevents=None, max_batch_len=None, chopped=False, pad=False, max_nbatch=None),
    "random_live": dict(nevents=5, random_nevents=True, data_seed=7, live_selection=True, track_len_sel=2.0,
                        max_abs_costheta_sel=0.95, min_abs_segz_sel=20.0, track_z_bound=24.0, max_batch_len=30.0,
                        chopped=True, pad=True, electron_sampling_resolution=0.2, max_nbatch=2),
    "no_swap_unpadded": dict(nevents=4, swap_xz=False, max_batch_len=18.0, chopped=True, pad=False,
                             electron_sampling_resolution=0.25),
}


def make_target(seg, seed=1):
    """Target segments for TgtTracksDataset: the same trajectories with other
    energy deposits, rows in another order, plus one extra event."""
    rng = np.random.default_rng(seed)
    tgt = seg.copy()
    tgt["dE"] = (tgt["dE"] * rng.uniform(0.8, 1.2, tgt.shape[0])).astype(np.float32)
    extra = seg[seg["event_id"] == seg["event_id"][0]].copy()
    extra["event_id"] = 999
    tgt = np.concatenate([tgt, extra])
    return tgt[rng.permutation(tgt.shape[0])]


def load_reference(segments, target=None):
    fake = types.ModuleType("h5py")

    class File:
        def __init__(self, name, mode="r"):
            self.table = target if str(name).startswith("target") else segments

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

        def __getitem__(self, key):
            assert key == "segments"
            return self.table.copy()

    fake.File = File
    sys.modules["h5py"] = fake
    spec = importlib.util.spec_from_file_location("ref_dataio", REF / "optimize" / "dataio.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


TARGET_CASES = {
    "tgt_batched": ("batched", dict(chopped=True, pad=True, electron_sampling_resolution=0.1)),
    "tgt_unchopped": ("no_swap_unpadded", dict(swap_xz=False, chopped=False, pad=True)),
}


def main():
    seg = make_segments()
    tgt = make_target(seg)
    mod = load_reference(seg, tgt)
    arrays = {"segments": seg, "target_segments": tgt}
    for name, (sim_case, kw) in TARGET_CASES.items():
        skw = dict(CASES[sim_case])
        nevents = skw.pop("nevents")
        sim = mod.TracksDataset("segments.h5", nevents, **skw)
        ds = mod.TgtTracksDataset("target.h5", sim, **kw)
        arrays[f"{name}/n_batches"] = np.array(len(ds))
        arrays[f"{name}/fields"] = np.array(ds.get_track_fields())
        arrays[f"{name}/max_batch_nsteps"] = np.array(ds.max_batch_nsteps)
        arrays[f"{name}/tot_data_length"] = np.array(ds.tot_data_length, dtype=np.float64)
        for i in range(len(ds)):
            arrays[f"{name}/batch_{i}"] = ds[i]
            arrays[f"{name}/rows_{i}"] = np.asarray(ds.batch_row_indices[i])
    for name, kw in CASES.items():
        kw = dict(kw)
        nevents = kw.pop("nevents")
        ds = mod.TracksDataset("segments.h5", nevents, **kw)
        arrays[f"{name}/n_batches"] = np.array(len(ds))
        arrays[f"{name}/fields"] = np.array(ds.get_track_fields())
        arrays[f"{name}/max_batch_nsteps"] = np.array(ds.max_batch_nsteps)
        arrays[f"{name}/tot_data_length"] = np.array(ds.tot_data_length, dtype=np.float64)
        for i in range(len(ds)):
            arrays[f"{name}/batch_{i}"] = ds[i]
            arrays[f"{name}/events_{i}"] = np.asarray(ds.get_batch_global_event_ids(i))
            arrays[f"{name}/rows_{i}"] = np.asarray(ds.get_batch_row_indices(i))
        b0 = ds[0]
        arrays[f"{name}/pad_batch_0"] = ds.pad_batch(b0, b0.shape[0] + 37, 0)
    np.savez_compressed(OUT, **arrays)
    print(OUT, len(arrays), "arrays,", seg.shape[0], "segments")


if __name__ == "__main__":
    main()
