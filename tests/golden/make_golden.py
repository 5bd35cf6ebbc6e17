"""Extract golden vectors from the reference's committed outputs.

Reads output/jax_ref/output_{lut,parametrized}_1.npz of larnd-sim-jax (made
by optimize/simulate.py --out_np) and keeps, per file, the distinct
(adc, Q, x, y, z, ticks, event) rows.  These pin, bit for bit, the pixel
centres (get_pixel_coordinates), hit z (get_hit_z with get_vdrift), the
digitisation of zero charge and the ADC->charge inverse (adc2charge) of
the reference as XLA compiled them.

Usage: python tests/golden/make_golden.py /path/to/larnd-sim-jax   (or LARNDSIM_JAX_SRC=/path/to/larnd-sim-jax)
"""

import os
import sys
from pathlib import Path

import numpy as np

# the larnd-sim-jax source tree: the first argument, or LARNDSIM_JAX_SRC
REF = Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LARNDSIM_JAX_SRC", ""))
if not (REF / "src" / "larndsim").is_dir():
    raise SystemExit(f"{Path(__file__).name}: give the larnd-sim-jax source tree as the first argument "
                     "or in LARNDSIM_JAX_SRC")
OUT = Path(__file__).resolve().parent / "jax_ref_hits.npz"


def main():
    arrays = {}
    for tag in ("lut", "parametrized"):
        d = np.load(REF / "output" / "jax_ref" / f"output_{tag}_1.npz")
        rec = np.stack([d["adcs"].view(np.uint32), d["Q"].view(np.uint32), d["x"].view(np.uint32),
                        d["y"].view(np.uint32), d["z"].view(np.uint32), d["ticks"].view(np.uint32),
                        d["event_id"].astype(np.int32).view(np.uint32)], axis=1)
        uniq = np.unique(rec, axis=0)
        arrays[f"{tag}_rows"] = uniq
    np.savez_compressed(OUT, **arrays)
    print(OUT, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
