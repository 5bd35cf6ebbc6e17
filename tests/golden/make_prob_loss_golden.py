"""Golden values of the reference's likelihood losses on probabilistic
distributions, from its own source.

Runs larnd-sim-jax's ``ProbabilisticLossStrategy.compute`` and
``compute_occurrence_indices`` (optimize/strategies.py:14-40, :338-567) and
``llhd_loss`` (src/larndsim/losses_jax.py:414-441) through the numpy
stand-in for jax (make_lut_golden.load_reference) on seeded inputs that
``prob_loss_inputs`` / ``llhd_inputs`` rebuild from their seeds (numpy's
PCG64 streams are the same on every platform), so only the outputs are
stored.

The strategy case: 160 simulated pixels sorted with 16 pad rows (-1) in
front as LUTProbabilisticSimulation pads them, distributions of 10 hits x
120 ticks (log-probabilities uniform in [-40, 0], so some fall below
log(1e-10) and are clamped; ADC counts uniform in [0, 255]), and 230
target hits sorted by pixel id: runs of 1-4 hits on simulated pixels,
hits on pixels that were not simulated, and 12 pad hits (-1) at the end.
Values are taken in a 32-bit run (JAX's default types) and a 64-bit run;
the 64-bit run also gives central differences of the loss with respect to
the log-probability and the ADC entries the first 16 valid hits read.

The CollapsedProbabilisticLossStrategy cases (with mse_adc): 48 pixels x
10 hits x 120 ticks of peaked tick probabilities, collapsed to one
pseudo-hit per (pixel, hit), and a sparse variant expanded to one
pseudo-hit per entry above the hit threshold; loss values from a 32-bit
run.

The llhd_loss case: 64 rows x 120 ticks, probabilities uniform in
[1e-6, 1], ticks with about a fifth at or beyond T - 3 (the no-hit
branch), central differences with respect to the gathered probability and
charge, no_hit_prob and charge_mc of the first 16 rows.

Usage: python tests/golden/make_prob_loss_golden.py /path/to/larnd-sim-jax   (or LARNDSIM_JAX_SRC=/path/to/larnd-sim-jax)
"""

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

OUT = HERE / "prob_loss_ref.npz"
N_FD = 16
PROB_SEED, LLHD_SEED, COLLAPSED_SEED = 7, 8, 9


def prob_loss_inputs(seed=PROB_SEED, n_pix=160, n_pad=16, H=10, T=120):
    """(sim_pixels [P], log_prob [P, H, T], adcs [P, H, T], tgt_pixels,
    tgt_ticks, tgt_adcs) of the strategy case."""
    rng = np.random.default_rng(seed)
    ids = np.sort(rng.choice(50_000, n_pix, replace=False)).astype(np.int32)
    sim = np.concatenate([np.full(n_pad, -1, np.int32), ids])
    P = sim.shape[0]
    log_prob = rng.uniform(-40.0, 0.0, (P, H, T)).astype(np.float32)
    adcs = rng.uniform(0.0, 255.0, (P, H, T)).astype(np.float32)
    hit_pix = rng.choice(ids, 60, replace=False)
    runs = rng.integers(1, 5, hit_pix.shape[0])
    absent = np.setdiff1d(rng.choice(50_000, 40, replace=False), ids)[:20].astype(np.int32)
    tp = np.concatenate([np.repeat(hit_pix, runs), absent])
    tp = np.sort(tp).astype(np.int32)
    tp = np.concatenate([tp, np.full(12, -1, np.int32)])
    n = tp.shape[0]
    ticks = rng.integers(0, T, n).astype(np.float32)
    tadc = rng.uniform(0.0, 255.0, n).astype(np.float32)
    return sim, log_prob, adcs, tp, ticks, tadc


def llhd_inputs(seed=LLHD_SEED, N=64, T=120):
    rng = np.random.default_rng(seed)
    tpd = rng.uniform(1e-6, 1.0, (N, T)).astype(np.float32)
    cd = rng.uniform(0.0, 200.0, (N, T)).astype(np.float32)
    ticks = rng.integers(0, T - 20, N)
    ticks[rng.random(N) < 0.2] = T - 3 + rng.integers(0, 3)
    nohit = rng.uniform(1e-4, 1.0, N).astype(np.float32)
    cmc = rng.uniform(0.0, 200.0, N).astype(np.float32)
    return tpd, ticks.astype(np.int32), nohit, cd, cmc


def collapsed_inputs(seed=COLLAPSED_SEED, n_pix=48, H=10, T=120, n_ref=150, sparse=False):
    """Prediction and target dictionaries of the CollapsedProbabilisticLossStrategy
    cases: per (pixel, hit) a peaked tick distribution of total probability
    below 1 (``sparse``: only three ticks non-zero, so that the entries
    above the hit threshold stay few), ADC distributions, pixel centres on
    a 0.4 cm grid in two planes and two events; the target hits nearby."""
    rng = np.random.default_rng(seed)
    t = np.arange(T)
    mu = rng.uniform(10, T - 10, (n_pix, H, 1))
    w = rng.uniform(2.0, 6.0, (n_pix, H, 1))
    prob = np.exp(-0.5 * ((t - mu) / w) ** 2)
    prob = prob / prob.sum(axis=2, keepdims=True) * rng.uniform(0.05, 0.95, (n_pix, H, 1))
    if sparse:
        keep = np.zeros_like(prob, bool)
        for k in range(3):
            idx = np.clip(np.round(mu[..., 0]).astype(int) + k - 1, 0, T - 1)
            np.put_along_axis(keep, idx[..., None], True, axis=2)
        prob = np.where(keep, prob, 0.0)
    pred = {"hit_prob": prob.astype(np.float32),
            "adcs_distrib": rng.uniform(20.0, 200.0, (n_pix, H, T)).astype(np.float32),
            "pixel_x": (0.4 * rng.integers(0, 60, n_pix)).astype(np.float32),
            "pixel_y": (0.4 * rng.integers(0, 60, n_pix)).astype(np.float32),
            "pixel_plane": rng.integers(0, 2, n_pix).astype(np.int32),
            "event": rng.integers(0, 2, n_pix).astype(np.int32)}
    tgt = {"adcs": rng.uniform(20.0, 200.0, n_ref).astype(np.float32),
           "pixel_x": (0.4 * rng.integers(0, 60, n_ref)).astype(np.float32),
           "pixel_y": (0.4 * rng.integers(0, 60, n_ref)).astype(np.float32),
           "pixel_z": rng.uniform(-30.0, 30.0, n_ref).astype(np.float32),
           "ticks": rng.uniform(0, T, n_ref).astype(np.float32),
           "hit_prob": np.ones(n_ref, np.float32),
           "event": rng.integers(0, 2, n_ref).astype(np.int32)}
    return pred, tgt


def main():
    from make_lut_golden import REF, load_reference
    import jax_numpy_standin
    C, F, S, base = load_reference()
    sys.path.insert(0, str(REF / "optimize"))
    import strategies as St
    from larndsim import losses_jax as Lj
    import jax.numpy as jnp

    out = {}
    sim, lp, ad, tp, tt, ta = prob_loss_inputs()
    strat = St.ProbabilisticLossStrategy()
    out["occurrence"] = np.asarray(St.compute_occurrence_indices(jnp.asarray(tp)))

    def call(lp_, ad_, x64):
        jax_numpy_standin._X64[0] = x64
        ft = np.float64 if x64 else np.float32
        pred = {"unique_pixels": jnp.asarray(sim), "hit_prob": jnp.asarray(lp_.astype(ft)),
                "adcs_distrib": jnp.asarray(ad_.astype(ft))}
        tgt = {"pixel_id": jnp.asarray(tp), "ticks": jnp.asarray(tt.astype(ft)), "adcs": jnp.asarray(ta.astype(ft))}
        v, aux = strat.compute(base, pred, tgt)
        return float(np.asarray(v)), {k: float(np.asarray(x)) for k, x in aux.items()}

    v32, aux32 = call(lp, ad, False)
    v64, aux64 = call(lp, ad, True)
    out["prob/loss32"], out["prob/loss64"] = np.array(v32), np.array(v64)
    for k in aux32:
        out[f"prob/aux32/{k}"], out[f"prob/aux64/{k}"] = np.array(aux32[k]), np.array(aux64[k])
    # entries read by the first N_FD valid hits (searchsorted match, run index, tick)
    idx = np.clip(np.searchsorted(sim, tp), 0, sim.shape[0] - 1)
    valid = np.nonzero((sim[idx] == tp) & (tp >= 0))[0][:N_FD]
    occ = out["occurrence"]
    pos = np.stack([idx[valid], np.minimum(occ[valid], lp.shape[1] - 1), tt[valid].astype(np.int64)], axis=1)
    out["prob/fd_pos"] = pos
    lp64, ad64 = lp.astype(np.float64), ad.astype(np.float64)
    for name, arr in (("log_prob", lp64), ("adcs", ad64)):
        g = np.zeros(N_FD)
        for i, (a, b, c) in enumerate(pos):
            h = 1e-6 * max(abs(arr[a, b, c]), 1.0)
            plus, minus = arr.copy(), arr.copy()
            plus[a, b, c] += h
            minus[a, b, c] -= h
            args_p = (plus, ad64) if name == "log_prob" else (lp64, plus)
            args_m = (minus, ad64) if name == "log_prob" else (lp64, minus)
            g[i] = (call(*args_p, True)[0] - call(*args_m, True)[0]) / (2 * h)
        out[f"prob/fd_{name}"] = g
    print(f"ProbabilisticLossStrategy: 32-bit {v32:.9g}, 64-bit {v64:.12g}, aux {aux32}")

    tpd, tk, nh, cd, cm = llhd_inputs()

    def lcall(tpd_, nh_, cd_, cm_, x64):
        jax_numpy_standin._X64[0] = x64
        ft = np.float64 if x64 else np.float32
        v, _ = Lj.llhd_loss(jnp.asarray(tpd_.astype(ft)), jnp.asarray(tk), jnp.asarray(nh_.astype(ft)),
                            jnp.asarray(cd_.astype(ft)), jnp.asarray(cm_.astype(ft)))
        return float(np.asarray(v))

    l32 = lcall(tpd, nh, cd, cm, False)
    l64 = lcall(tpd, nh, cd, cm, True)
    out["llhd/loss32"], out["llhd/loss64"] = np.array(l32), np.array(l64)
    a64 = [x.astype(np.float64) for x in (tpd, nh, cd, cm)]
    rows = np.arange(N_FD)
    T = tpd.shape[1]
    for j, name in enumerate(("ticks_prob", "no_hit_prob", "charge", "charge_mc")):
        g = np.zeros(N_FD)
        for i in rows:
            loc = (i, min(int(tk[i]), T - 1)) if name in ("ticks_prob", "charge") else (i,)
            base_arr = a64[j]
            h = 1e-6 * max(abs(base_arr[loc]), 1e-3)
            plus, minus = [x.copy() for x in a64], [x.copy() for x in a64]
            plus[j][loc] += h
            minus[j][loc] -= h
            g[i] = (lcall(*plus, True) - lcall(*minus, True)) / (2 * h)
        out[f"llhd/fd_{name}"] = g
    print(f"llhd_loss: 32-bit {l32:.9g}, 64-bit {l64:.12g}")
    # CollapsedProbabilisticLossStrategy with the fitter's default mse_adc,
    # collapsed (one pseudo-hit per pixel and hit) and per distribution entry
    jax_numpy_standin._X64[0] = False
    for name, sparse, collapsed in (("collapsed", False, True), ("entries", True, False)):
        pred, tgt = collapsed_inputs(sparse=sparse)
        st = St.CollapsedProbabilisticLossStrategy(Lj.mse_adc, collapsed=collapsed)
        S.size_history_dict.clear()
        v, _ = st.compute(base, {k: jnp.asarray(a) for k, a in pred.items()},
                          {k: jnp.asarray(a) for k, a in tgt.items()})
        out[f"{name}/loss32"] = np.array(float(np.asarray(v)))
        print(f"CollapsedProbabilisticLossStrategy ({name}): {float(np.asarray(v)):.9g}")
    out["config"] = np.array(json.dumps(dict(n_fd=N_FD, prob_seed=PROB_SEED, llhd_seed=LLHD_SEED,
                                             collapsed_seed=COLLAPSED_SEED)))
    np.savez_compressed(OUT, **out)
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
