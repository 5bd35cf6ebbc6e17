"""Golden vectors of the reference's LUT simulate path, from its own source.

Runs larnd-sim-jax's ``load_detector_properties`` and ``load_lut``
(consts_jax.py:220-449), ``simulate_wfs`` (sim_jax.py:689-736, through
simulate_drift_new, quench, drift and simulate_signals), ``get_adc_values``
and ``digitize`` (fee_jax.py:55-71, :168-279) and ``simulate_stochastic``
(sim_jax.py:738-769, through parse_output) on seeded synthetic events, in a
process without JAX: the reference's modules are imported from its source
tree with the numpy stand-in of jax_numpy_standin.py registered as jax /
flax, the package's YAML subset reader as yaml, and an empty h5py.  Noise
amplitudes are zero (optimize/simulate.py:77-78 without --noise), so the
stand-in's random draws do not enter the outputs.

Each case stores its inputs (the track array, the options, the seed and
size of the synthetic response with a checksum), samples of the template
bank, the waveforms (non-zero entries as row, tick, value), the pixel ids,
the front end's integral and tick grids, the digitised grid and the 8
compacted outputs of simulate_stochastic, in lut_ref.npz.

Usage: python tests/golden/make_lut_golden.py /path/to/larnd-sim-jax   (or LARNDSIM_JAX_SRC=/path/to/larnd-sim-jax)
"""

import json
import os
import sys
import tempfile
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
# the larnd-sim-jax source tree: the first argument, or LARNDSIM_JAX_SRC
REF = Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LARNDSIM_JAX_SRC", ""))
if not (REF / "src" / "larndsim").is_dir():
    raise SystemExit(f"{Path(__file__).name}: give the larnd-sim-jax source tree as the first argument "
                     "or in LARNDSIM_JAX_SRC")
OUT = HERE / "lut_ref.npz"

sys.path[:0] = [str(HERE), str(REPO / "larnd-sim-jax_gb300")]

from larndsim_gb300 import workloads, yaml_lite  # noqa: E402

import jax_numpy_standin  # noqa: E402

# Each case: the event (workload generator and its arguments), the
# simulation options, and the response LUT size (10n+5 sub-positions cover
# the neighbour LUT index 10n+4).
CASES = {
    "muons_n1": dict(event=("muon", dict(seed=31, n_tracks=4)), n=1, L=150, mode="BIRKS", n_templates=10, lut=15),
    "muons_n4_L100": dict(event=("muon", dict(seed=32, n_tracks=3)), n=4, L=100, mode="BIRKS", n_templates=10,
                          lut=45),
    "two_events_box_n2": dict(event=("two_events", dict(seed=33)), n=2, L=150, mode="BOX", n_templates=12, lut=25),
    "tpc1_ellipsoid_n0": dict(event=("muon", dict(seed=34, n_tracks=3, box_lo=(0.5, 0.5, -30.3),
                                                  box_hi=(30.5, 30.5, -0.3))),
                              n=0, L=150, mode="ELLIPSOID", n_templates=10, lut=15),
}
RESPONSE_SEED = 0


def make_event(kind, kw):
    """The case's track array (float32, reference field order) and fields."""
    if kind == "muon":
        return workloads.muon_event(**kw)
    if kind == "two_events":
        # a muon event, a short-segment shower as event 1, and padding rows
        # (eventID -1, zero charge) as the reference's dataset appends them
        a, fields = workloads.muon_event(seed=kw["seed"], n_tracks=2)
        b, _ = workloads.shower_event(seed=kw["seed"] + 100, n_segments=120, event_id=1, n_subtracks=3)
        pad = np.zeros((7, a.shape[1]), np.float32)
        f = list(fields)
        pad[:, f.index("eventID")] = -1
        pad[:, f.index("trackID")] = -1
        pad[:, f.index("pixel_plane")] = -1
        return np.concatenate([a, b, pad]).astype(np.float32), fields
    raise ValueError(kind)


def response_checksum(resp):
    return int(zlib.crc32(np.ascontiguousarray(resp, np.float32).tobytes()))


def load_reference(ref=REF, x64=False):
    """The reference's consts_jax, fee_jax and sim_jax modules imported
    with the numpy stand-in (``x64``: with 64-bit types enabled), and its
    module0 parameters (no gradient fields) from its own YAML files."""
    jax_numpy_standin.install(yaml_lite.loads, x64=x64)
    sys.path[:0] = [str(ref / "src"), str(ref)]
    from larndsim import consts_jax as C
    from larndsim import fee_jax as F
    from larndsim import sim_jax as S

    Params = C.build_params_class([])
    base = C.load_detector_properties(Params, str(ref / "src/larndsim/detector_properties/module0.yaml"),
                                      str(ref / "src/larndsim/pixel_layouts/multi_tile_layout-2.4.16_v4.yaml"))
    return C, F, S, base


def main():
    C, F, S, base = load_reference()
    import jax.numpy as jnp

    out = {}
    tmp = Path(tempfile.mkdtemp())
    for name, case in CASES.items():
        S.size_history_dict.clear()
        p = base.replace(long_diff_template=jnp.linspace(0.001, 10, case["n_templates"]),
                         number_pix_neighbors=case["n"], signal_length=case["L"], time_window=case["L"],
                         RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0,
                         recombination_mode=getattr(C.RecombinationMode, case["mode"]))
        resp = workloads.synthetic_response(seed=RESPONSE_SEED, nx=case["lut"], ny=case["lut"])
        np.save(tmp / f"{name}.npy", resp)
        tmpl, p = C.load_lut(str(tmp / f"{name}.npy"), p)
        tracks, fields = make_event(*case["event"])
        wfs, unique = S.simulate_wfs(p, tmpl, jnp.asarray(tracks), tuple(fields))
        integral, ticks = F.get_adc_values(p, wfs, jax_numpy_standin.prng_key(0))
        grid_adcs = F.digitize(p, integral)
        hits = S.simulate_stochastic(p, wfs, unique, 0)
        wfs = np.asarray(wfs)
        for a in (tmpl, wfs, integral, grid_adcs) + tuple(hits[:6]):
            assert not np.isnan(np.asarray(a)).any(), f"{name}: NaN in the reference outputs"
        rng = np.random.default_rng(zlib.crc32(name.encode()))
        t = np.asarray(tmpl)
        flat = rng.choice(t.size, 4096, replace=False)
        rows, cols = np.nonzero(wfs)
        cfg = dict(case, event=[case["event"][0], case["event"][1]], response_seed=RESPONSE_SEED,
                   response_crc32=response_checksum(resp), fields=list(fields))
        out[f"{name}/config"] = np.array(json.dumps(cfg))
        out[f"{name}/tracks"] = tracks
        out[f"{name}/tmpl_index"] = flat.astype(np.int64)
        out[f"{name}/tmpl_value"] = t.ravel()[flat]
        out[f"{name}/tmpl_sum"] = t.astype(np.float64).reshape(t.shape[0], -1).sum(axis=1)
        out[f"{name}/unique_pixels"] = np.asarray(unique)
        out[f"{name}/wfs_shape"] = np.array(wfs.shape, np.int64)
        out[f"{name}/wfs_row"] = rows.astype(np.int32)
        out[f"{name}/wfs_tick"] = cols.astype(np.int16)
        out[f"{name}/wfs_value"] = wfs[rows, cols]
        out[f"{name}/integral"] = np.asarray(integral)
        out[f"{name}/ticks"] = np.asarray(ticks)
        out[f"{name}/grid_adcs"] = np.asarray(grid_adcs)
        for key, a in zip(("adcs", "pixel_x", "pixel_y", "pixel_z", "ticks", "hit_prob", "event", "pixels"), hits):
            out[f"{name}/hits_{key}"] = np.asarray(a)
        print(f"{name}: {tracks.shape[0]} segments, {int((np.asarray(unique) >= 0).sum())} pixels, "
              f"{rows.size} non-zero samples, {hits[0].shape[0]} hits")
    np.savez_compressed(OUT, **out)
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
