"""Golden values of the reference's fit losses, from its own source.

Runs larnd-sim-jax's ``mse_adc`` (losses_jax.py:13-79), ``chamfer_3d``
(:181-229) and ``nll_loss`` (:329-359) through the numpy stand-in for jax
(make_lut_golden.load_reference) on two hit sets: the predicted hits are
the reference's own simulate_stochastic outputs of a two-event case of
tests/golden/lut_ref.npz, the reference hits a seeded perturbation of them
(charges scaled, z shifted, a tenth dropped, three added).

Values are taken twice: in a 32-bit run (what JAX evaluates by default;
the losses stack x + event * 1e5 or 1e9 in float32, which rounds x) and in
a run with 64-bit types on x values pre-rounded so that the stacked
coordinate equals the 32-bit one exactly, which isolates the formulas from
float32 rounding.  The 64-bit run also gives central differences with
respect to Q and z of the first 12 predicted hits (and hit_prob for
nll_loss), step 1e-6 max(|v|, 1).

Usage: python tests/golden/make_loss_golden.py /path/to/larnd-sim-jax   (or LARNDSIM_JAX_SRC=/path/to/larnd-sim-jax)
"""

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from make_lut_golden import load_reference  # noqa: E402

import jax_numpy_standin  # noqa: E402

OUT = HERE / "loss_ref.npz"
LUT_GOLD = HERE / "lut_ref.npz"
CASE = "two_events_box_n2"
N_FD = 12
OFFSETS = {"mse_adc": 1e5, "chamfer_3d": 1e9, "nll_loss": 1e9}
COLS = ("Q", "x", "y", "z", "ticks", "hit_prob", "event")


def hit_sets(seed=0):
    """(predicted, reference) hit columns, float32 (event int32)."""
    g = np.load(LUT_GOLD)
    pred = {"Q": g[f"{CASE}/hits_adcs"], "x": g[f"{CASE}/hits_pixel_x"], "y": g[f"{CASE}/hits_pixel_y"],
            "z": g[f"{CASE}/hits_pixel_z"], "ticks": g[f"{CASE}/hits_ticks"],
            "hit_prob": g[f"{CASE}/hits_hit_prob"], "event": g[f"{CASE}/hits_event"]}
    rng = np.random.default_rng(seed)
    n = pred["Q"].shape[0]
    keep = np.sort(rng.choice(n, n - n // 10, replace=False))
    ref = {k: v[keep].copy() for k, v in pred.items()}
    ref["Q"] = (ref["Q"] * rng.uniform(0.9, 1.1, keep.size)).astype(np.float32)
    ref["z"] = (ref["z"] + rng.normal(0, 0.3, keep.size)).astype(np.float32)
    extra = {k: v[:3].copy() for k, v in ref.items()}
    extra["x"] = (extra["x"] + 2.0).astype(np.float32)
    ref = {k: np.concatenate([ref[k], extra[k]]) for k in COLS}
    # hit probabilities in (0, 1] for the prediction, so nll_loss sees them
    pred["hit_prob"] = rng.uniform(0.3, 1.0, n).astype(np.float32)
    return pred, ref


def prerounded_x(x, event, offset):
    """x such that x + event * offset in float64 equals the float32 sum."""
    s32 = (np.float32(x) + (event.astype(np.float32) * np.float32(offset)).astype(np.float32)).astype(np.float32)
    return s32.astype(np.float64) - event.astype(np.float64) * offset


def main():
    C, F, S, base = load_reference()
    from larndsim import losses_jax as Lj
    import jax.numpy as jnp

    pred, ref = hit_sets()
    out = {f"pred_{k}": v for k, v in pred.items()}
    out.update({f"ref_{k}": v for k, v in ref.items()})

    def call(name, pr, rf):
        S.size_history_dict.clear()
        args = [jnp.asarray(pr[k]) for k in COLS] + [jnp.asarray(rf[k]) for k in COLS]
        return float(np.asarray(getattr(Lj, name)(base, *args)[0]))

    for name, off in OFFSETS.items():
        jax_numpy_standin._X64[0] = False
        v32 = call(name, pred, ref)
        jax_numpy_standin._X64[0] = True
        p64 = {k: v.astype(np.float64) if k != "event" else v.astype(np.int64) for k, v in pred.items()}
        r64 = {k: v.astype(np.float64) if k != "event" else v.astype(np.int64) for k, v in ref.items()}
        p64["x"] = prerounded_x(pred["x"], pred["event"], off)
        r64["x"] = prerounded_x(ref["x"], ref["event"], off)
        v64 = call(name, p64, r64)
        wrt = ("Q", "z", "hit_prob") if name == "nll_loss" else ("Q", "z")
        for col in wrt:
            g = np.zeros(N_FD)
            for i in range(N_FD):
                h = 1e-6 * max(abs(p64[col][i]), 1.0)
                pp, pm = dict(p64), dict(p64)
                pp[col], pm[col] = p64[col].copy(), p64[col].copy()
                pp[col][i] += h
                pm[col][i] -= h
                g[i] = (call(name, pp, r64) - call(name, pm, r64)) / (2 * h)
            out[f"{name}/fd_{col}"] = g
        S.size_history_dict.clear()
        out[f"{name}/loss32"] = np.array(v32)
        out[f"{name}/loss64"] = np.array(v64)
        print(f"{name}: 32-bit {v32:.9g}, 64-bit {v64:.12g}")
    out["config"] = np.array(json.dumps(dict(case=CASE, n_fd=N_FD, offsets=OFFSETS, seed=0)))
    np.savez_compressed(OUT, **out)
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
