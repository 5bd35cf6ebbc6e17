"""Golden vectors of the reference's parametrised-current path, from its own source.

Runs larnd-sim-jax's ``simulate_parametrized`` (sim_jax.py:339-372:
simulate_drift with generate_electrons, get_pixels, current_mc with
current_model_diff, accumulate_signals_parametrized, get_adc_values,
digitize, parse_output) on seeded synthetic events, with the reference's
modules imported through the numpy stand-in of jax_numpy_standin.py
(make_lut_golden.load_reference).  Nothing is re-implemented here: the
stand-in's ``jax.random.normal`` records the diffusion draws it hands to
generate_electrons (detsim_jax.py:393), and thin wrappers record the pixel
list passed to simulate_signals_parametrized and the waveforms passed to
get_adc_values, then call the reference's functions unchanged.  Noise
amplitudes are zero.  mc_diff is on, as the reference's deterministic
branch (apply_tran_diff) cannot run: it reads a ``pixels`` name it never
defines (detsim_jax.py:358-365).

Each case stores the track array, the options, the recorded draws (N, 3),
the pixel ids, the waveforms (non-zero entries), the front end's integral
and tick grids, and the 8 outputs of simulate_parametrized, in
param_ref.npz.

Usage: python tests/golden/make_param_golden.py /path/to/larnd-sim-jax   (or LARNDSIM_JAX_SRC=/path/to/larnd-sim-jax)
"""

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from make_lut_golden import load_reference, make_event  # noqa: E402

OUT = HERE / "param_ref.npz"

CASES = {
    "param_muons": dict(event=("muon", dict(seed=41, n_tracks=4)), mode="BIRKS", rngseed=3),
    "param_two_events_box": dict(event=("two_events", dict(seed=42)), mode="BOX", rngseed=5),
    "param_tpc1_ellipsoid": dict(event=("muon", dict(seed=43, n_tracks=3, box_lo=(0.5, 0.5, -30.3),
                                                     box_hi=(30.5, 30.5, -0.3))), mode="ELLIPSOID", rngseed=7),
}
HIT_KEYS = ("adcs", "pixel_x", "pixel_y", "pixel_z", "ticks", "hit_prob", "event", "pixels")


def main():
    C, F, S, base = load_reference()
    import jax
    import jax.numpy as jnp

    rec = {}
    draw = jax.random.normal

    def recording_normal(key, shape=(), dtype=np.float32):
        out = draw(key, shape, dtype)
        if len(tuple(shape)) == 2 and tuple(shape)[1] == 3:
            rec["draws"] = np.asarray(out)
        return out
    jax.random.normal = recording_normal

    signals = S.simulate_signals_parametrized
    fee = S.get_adc_values

    def recording_signals(params, electrons, pIDs, unique_pixels, rngkey, fields):
        rec["unique"] = np.asarray(unique_pixels)
        return signals(params, electrons, pIDs, unique_pixels, rngkey, fields)

    def recording_fee(params, pixels_signals, key):
        integral, ticks = fee(params, pixels_signals, key)
        rec.update(wfs=np.asarray(pixels_signals), integral=np.asarray(integral), ticks=np.asarray(ticks))
        return integral, ticks
    S.simulate_signals_parametrized = recording_signals
    S.get_adc_values = recording_fee

    out = {}
    for name, case in CASES.items():
        S.size_history_dict.clear()
        rec.clear()
        p = base.replace(number_pix_neighbors=0, mc_diff=True, diffusion_in_current_sim=True,
                         RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0,
                         recombination_mode=getattr(C.RecombinationMode, case["mode"]))
        tracks, fields = make_event(*case["event"])
        hits = S.simulate_parametrized(p, jnp.asarray(tracks), tuple(fields), rngseed=case["rngseed"])
        assert rec["draws"].shape == (tracks.shape[0], 3)
        for a in (rec["wfs"], rec["integral"]) + tuple(hits[:6]):
            assert not np.isnan(np.asarray(a)).any(), f"{name}: NaN in the reference outputs"
        rows, cols = np.nonzero(rec["wfs"])
        cfg = dict(case, event=[case["event"][0], case["event"][1]], fields=list(fields))
        out[f"{name}/config"] = np.array(json.dumps(cfg))
        out[f"{name}/tracks"] = tracks
        out[f"{name}/draws"] = rec["draws"].astype(np.float32)
        out[f"{name}/unique_pixels"] = rec["unique"]
        out[f"{name}/wfs_shape"] = np.array(rec["wfs"].shape, np.int64)
        out[f"{name}/wfs_row"] = rows.astype(np.int32)
        out[f"{name}/wfs_tick"] = cols.astype(np.int16)
        out[f"{name}/wfs_value"] = rec["wfs"][rows, cols]
        out[f"{name}/integral"] = rec["integral"]
        out[f"{name}/ticks"] = rec["ticks"]
        for key, a in zip(HIT_KEYS, hits):
            out[f"{name}/hits_{key}"] = np.asarray(a)
        print(f"{name}: {tracks.shape[0]} segments, {int((rec['unique'] >= 0).sum())} pixels, "
              f"{rows.size} non-zero samples, {hits[0].shape[0]} hits")
    np.savez_compressed(OUT, **out)
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
