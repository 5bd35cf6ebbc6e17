"""Golden vectors of the reference's track chopping (chop_tracks).

Imports optimize/dataio.py of larnd-sim-jax (the module imports h5py at
the top but chop_tracks does not use it, so an empty stand-in module is
registered under that name), runs chop_tracks on seeded synthetic tracks
and stores inputs and outputs in chop_ref.npz.  The cases cover the
step sizes the reference uses (0.001 cm, the electron_sampling_resolution
default of consts_jax.py:275; 0.1 cm, the TracksDataset default of
dataio.py:111; and 0.04 cm), zero-length tracks, tracks shorter than one
step, tracks of an exact multiple of the step, axis-aligned tracks and
negative coordinates.  Generated with NumPy 2.

Usage: python tests/golden/make_chop_golden.py /path/to/larnd-sim-jax   (or LARNDSIM_JAX_SRC=/path/to/larnd-sim-jax)
"""

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
OUT = Path(__file__).resolve().parent / "chop_ref.npz"

FIELDS = ("eventID", "trackID", "x_start", "y_start", "z_start", "x_end", "y_end", "z_end", "x", "y", "z",
          "t", "t_start", "t_end", "t0", "t0_start", "t0_end", "dx", "dE", "dEdx", "n_electrons", "n_photons",
          "long_diff", "tran_diff", "pixel_plane", "pdgId")


def make_tracks(seed, n, mean_len, precision):
    rng = np.random.default_rng(seed)
    col = {f: i for i, f in enumerate(FIELDS)}
    t = rng.uniform(-5, 5, (n, len(FIELDS))).astype(np.float32)
    start = rng.uniform(-30, 30, (n, 3))
    u = rng.standard_normal((n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    length = rng.exponential(mean_len, n)
    # special lengths: zero, below one step, exact multiples, tiny, axis-aligned
    length[0] = 0.0
    length[1] = 0.3 * precision
    length[2] = 7 * precision
    length[3] = precision
    length[4] = 1e-7
    u[5] = (0.0, 0.0, 1.0)
    u[6] = (-1.0, 0.0, 0.0)
    length[5:7] = 12.5 * precision
    end = start + u * length[:, None]
    for a, (cs, ce) in enumerate((("x_start", "x_end"), ("y_start", "y_end"), ("z_start", "z_end"))):
        t[:, col[cs]] = start[:, a]
        t[:, col[ce]] = end[:, a]
    t[:, col["x"]] = 0.5 * (t[:, col["x_start"]] + t[:, col["x_end"]])
    t[:, col["y"]] = 0.5 * (t[:, col["y_start"]] + t[:, col["y_end"]])
    t[:, col["z"]] = 0.5 * (t[:, col["z_start"]] + t[:, col["z_end"]])
    seg = t[:, [col["x_end"], col["y_end"], col["z_end"]]] - t[:, [col["x_start"], col["y_start"], col["z_start"]]]
    t[:, col["dx"]] = np.sqrt((seg.astype(np.float64) ** 2).sum(1)).astype(np.float32)
    t[:, col["dE"]] = rng.uniform(0.0, 3.0, n).astype(np.float32)
    t[:, col["eventID"]] = np.sort(rng.integers(0, 4, n)).astype(np.float32)
    t[:, col["trackID"]] = np.arange(n, dtype=np.float32)
    return t


def main():
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))
    sys.path.insert(0, str(REF))
    from optimize.dataio import chop_tracks

    cases = {"p0p04": (1, 120, 0.3, 0.04), "p0p001": (2, 30, 0.01, 0.001), "p0p1": (3, 40, 0.8, 0.1)}
    arrays = {"fields": np.array(FIELDS)}
    for name, (seed, n, mean_len, precision) in cases.items():
        tracks = make_tracks(seed, n, mean_len, precision)
        out = chop_tracks(tracks.copy(), FIELDS, precision=precision)
        assert out.dtype == np.float32
        arrays[f"{name}_in"] = tracks
        arrays[f"{name}_out"] = out
        arrays[f"{name}_precision"] = np.array(precision, np.float64)
    np.savez_compressed(OUT, **arrays)
    print(OUT, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
