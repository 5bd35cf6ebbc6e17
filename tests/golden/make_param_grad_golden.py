"""Central differences of the reference's parametrised-mode waveforms, in float64.

Runs larnd-sim-jax's ``simulate_parametrized`` (sim_jax.py:339-372)
through the numpy stand-in with 64-bit types (make_lut_golden.load_reference)
on the tracks of the ``param_muons`` case of param_ref.npz, with the
stand-in's ``jax.random.normal`` returning that case's recorded diffusion
draws (the offsets stay fixed, as this package's parametrised-mode
gradient holds them).  A wrapper records the waveforms handed to
get_adc_values, one the t0 ticks current_mc returns and one the pixel list
passed to simulate_signals_parametrized.  For the
functional sum(c * W) over the simulated rows, c a seeded standard-normal
array (numpy default_rng(seed), shape (simulated pixels, ticks)), it takes
central differences with respect to Ab, kb, eField, lifetime, vdrift,
long_diff, tran_diff and lArDensity at parameters perturbed by N(0, 5 %),
step 1e-6 |theta|, halved until the pixel list and every t0 tick are the
same on both sides.  The simulated pixel ids at the perturbed parameters
are stored with the derivatives.  Stored in param_grad_ref.npz.

Usage: python tests/golden/make_param_grad_golden.py /path/to/larnd-sim-jax   (or LARNDSIM_JAX_SRC=/path/to/larnd-sim-jax)
"""

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from make_lut_golden import load_reference  # noqa: E402

OUT = HERE / "param_grad_ref.npz"
PARAM_GOLD = HERE / "param_ref.npz"
CASE = "param_muons"
GRAD_PARAMS = ("Ab", "kb", "eField", "lifetime", "vdrift", "long_diff", "tran_diff", "lArDensity")
COT_SEED, THETA_SEED = 7, 3


def main():
    C, F, S, base = load_reference(x64=True)
    import jax
    import jax.numpy as jnp

    g = np.load(PARAM_GOLD)
    cfg = json.loads(str(g[f"{CASE}/config"]))
    tracks, fields, draws = g[f"{CASE}/tracks"], tuple(cfg["fields"]), g[f"{CASE}/draws"].astype(np.float64)
    rec = {}
    jax.random.normal = lambda key, shape=(), dtype=None: (
        jnp.asarray(draws) if tuple(shape) == draws.shape else jnp.zeros(shape))
    fee, cmc, sig = S.get_adc_values, S.current_mc, S.simulate_signals_parametrized

    def recording_signals(params, electrons, pIDs, unique_pixels, rngkey, fields_):
        rec["unique"] = np.asarray(unique_pixels)
        return sig(params, electrons, pIDs, unique_pixels, rngkey, fields_)
    S.simulate_signals_parametrized = recording_signals

    def recording_fee(params, pixels_signals, key):
        rec["wfs"] = np.asarray(pixels_signals, np.float64)
        return fee(params, pixels_signals, key)

    def recording_current(params, electrons, pixels_coord, fields_):
        t0_tick, signals = cmc(params, electrons, pixels_coord, fields_)
        rec["t0_tick"] = np.asarray(t0_tick)
        return t0_tick, signals
    S.get_adc_values, S.current_mc = recording_fee, recording_current

    borders32 = np.asarray(base.tpc_borders, np.float32).astype(np.float64)
    p0 = base.replace(tpc_borders=jnp.asarray(borders32), number_pix_neighbors=0, mc_diff=True,
                      diffusion_in_current_sim=True, RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0,
                      recombination_mode=getattr(C.RecombinationMode, cfg["mode"]))
    tr64 = jnp.asarray(tracks.astype(np.float64))

    def run(p):
        S.size_history_dict.clear()
        S.simulate_parametrized(p, tr64, fields, rngseed=cfg["rngseed"])
        return dict(rec)

    rng = np.random.default_rng(THETA_SEED)
    theta = {k: float(getattr(p0, k)) * (1 + 0.05 * rng.standard_normal()) for k in GRAD_PARAMS}
    p = p0.replace(**theta)
    r0 = run(p)
    unique = r0["unique"]
    valid = unique >= 0
    cot = np.random.default_rng(COT_SEED).standard_normal((int(valid.sum()), r0["wfs"].shape[1]))

    def functional(r):
        return float((cot * r["wfs"][valid]).sum())

    vjp, steps = [], []
    for k in GRAD_PARAMS:
        h = 1e-6 * abs(theta[k])
        for _ in range(25):
            rp, rm = run(p.replace(**{k: theta[k] + h})), run(p.replace(**{k: theta[k] - h}))
            if all(np.array_equal(r["t0_tick"], r0["t0_tick"]) and np.array_equal(r["unique"], unique)
                   for r in (rp, rm)):
                break
            h *= 0.5
        else:
            raise RuntimeError(f"{k}: a t0 tick changes within every step tried")
        vjp.append((functional(rp) - functional(rm)) / (2 * h))
        steps.append(h)
        print(f"d/d{k} = {vjp[-1]:.10g} (step {h:.3g})")
    np.savez_compressed(OUT, theta=np.array([theta[k] for k in GRAD_PARAMS]), fd_vjp=np.array(vjp),
                        fd_step=np.array(steps), t0_tick=r0["t0_tick"], pixels=unique[valid],
                        config=np.array(json.dumps(dict(case=CASE, cot_seed=COT_SEED, theta_seed=THETA_SEED,
                                                        grad_params=list(GRAD_PARAMS)))))
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
