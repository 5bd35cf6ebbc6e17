"""Central differences of the reference's own LUT chain, in float64.

jax.value_and_grad of the reference (optimize/fit_params.py:704-731)
differentiates simulate_wfs + get_adc_values + digitize with every integer
or comparison-derived quantity held fixed.  Where none of those quantities
changes inside a step, central differences of the same code evaluated in
float64 give that derivative to about 1e-9 relative.  This script runs the
reference's modules through the numpy stand-in with 64-bit types enabled
(jax_enable_x64 semantics; make_lut_golden.load_reference), on float64
copies of float32 inputs (tracks, TPC borders, template nodes: the values a
32-bit run sees), at perturbed parameters where its pixel ids, crossing
ticks and transverse bins match the 32-bit run's (the decisions jax.grad
holds), and
evaluates the sum-of-squared-ADC loss between a
prediction at parameters perturbed by N(0, 5 %) and a target simulated at
the nominal parameters (the grid of simulated rows, aligned by pixel id;
rows the target lacks compare with digitize(0), target rows the prediction
lacks add a constant).  For each of Ab, kb, eField, lifetime, vdrift,
long_diff, tran_diff and lArDensity it takes a central difference with
step 1e-6 |theta| and records that the pixel ids, every crossing tick,
every cathode tick floor(t0/t_sampling) and every template index stay the
same across the step (halving the step up to 24 times until they do: the
waveforms are continuous across a cathode tick, but their slope is not).  Besides the loss it differentiates the linear functional
sum(c * ADC) with c = 2 (ADC - target) from the 32-bit run: the
vector-Jacobian product jax.grad forms for the loss, free of the float32
rounding in the forward values that moves the residuals (the reference's
float32 cumulative sum of the template bank differs from its float64 one
by up to about 1e-4 of a waveform row's scale).

Each case stores the tracks, the options, the perturbed parameters (and
which seeded draw they are), the 32-bit run's simulated pixel ids and tick
and ADC grids there, the
target's pixel ids and float64 ADC grid, the loss at the perturbed
parameters, the steps and the central-difference gradient, in
grad_ref.npz.

Usage: python tests/golden/make_grad_golden.py /path/to/larnd-sim-jax   (or LARNDSIM_JAX_SRC=/path/to/larnd-sim-jax)
"""

import json
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from make_lut_golden import RESPONSE_SEED, load_reference, make_event, response_checksum  # noqa: E402

import jax_numpy_standin  # noqa: E402

from larndsim_gb300 import consts, workloads  # noqa: E402

OUT = HERE / "grad_ref.npz"
GRAD_PARAMS = ("Ab", "kb", "eField", "lifetime", "vdrift", "long_diff", "tran_diff", "lArDensity")

CASES = {
    "grad_muons_birks_n1": dict(event=("muon", dict(seed=61, n_tracks=4)), n=1, L=150, mode="BIRKS",
                                n_templates=10, lut=15, theta_seed=1),
    "grad_two_events_box_n2": dict(event=("two_events", dict(seed=62)), n=2, L=150, mode="BOX", n_templates=12,
                                   lut=25, theta_seed=2),
    "grad_muons_birks_n4": dict(event=("muon", dict(seed=64, n_tracks=2)), n=4, L=150, mode="BIRKS",
                                n_templates=10, lut=45, theta_seed=4),
}


def main():
    C, F, S, base = load_reference(x64=True)
    import jax.numpy as jnp

    # GRAD_GOLDEN_CASES (comma-separated) regenerates only those cases and
    # keeps the others of an existing file
    only = [c for c in os.environ.get("GRAD_GOLDEN_CASES", "").split(",") if c]
    out = {}
    if only and OUT.exists():
        with np.load(OUT) as old:
            out = {k: old[k] for k in old.files if k.split("/")[0] not in only}
    tmp = Path(tempfile.mkdtemp())
    borders32 = np.asarray(base.tpc_borders, np.float32).astype(np.float64)
    for name, case in CASES.items():
        if only and name not in only:
            continue
        nodes = consts.jax_linspace_f32(0.001, 10, case["n_templates"]).astype(np.float64)
        p0 = base.replace(long_diff_template=jnp.asarray(nodes), tpc_borders=jnp.asarray(borders32),
                          number_pix_neighbors=case["n"], signal_length=case["L"], time_window=case["L"],
                          RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0,
                          recombination_mode=getattr(C.RecombinationMode, case["mode"]))
        resp = workloads.synthetic_response(seed=RESPONSE_SEED, nx=case["lut"], ny=case["lut"])
        np.save(tmp / f"{name}.npy", resp)
        jax_numpy_standin._X64[0] = False
        tmpl32, _ = C.load_lut(str(tmp / f"{name}.npy"), p0)
        jax_numpy_standin._X64[0] = True
        tmpl, p0 = C.load_lut(str(tmp / f"{name}.npy"), p0)
        tracks, fields = make_event(*case["event"])
        tr64 = jnp.asarray(tracks.astype(np.float64))
        fields = tuple(fields)

        def run(p, x64=True):
            """(pixel ids, ADC grid, tick grid) of the reference at p; with
            x64=False the 32-bit run JAX makes by default."""
            jax_numpy_standin._X64[0] = x64
            try:
                S.size_history_dict.clear()
                wfs, unique = S.simulate_wfs(p, tmpl if x64 else tmpl32, tr64 if x64 else jnp.asarray(tracks), fields)
                integral, ticks = F.get_adc_values(p, wfs, np.array([0, 0], np.uint32))
                drift = S.simulate_drift_new(p, tr64 if x64 else jnp.asarray(tracks), fields)
                run.bins = [np.asarray(drift[i]) for i in (0, 1, 5, 6, 7)]   # pixel ids and LUT indices
                # cathode ticks and template indices (sim_jax.py:158, :163)
                t0, ld = np.asarray(drift[3], np.float64), np.asarray(drift[4], np.float64)
                run.times = [np.floor(t0 / p.t_sampling), np.searchsorted(nodes, ld)]
                return np.asarray(unique), np.asarray(F.digitize(p, integral), np.float64), np.asarray(ticks)
            finally:
                jax_numpy_standin._X64[0] = True

        t_pids, t_adc, _ = run(p0)
        adc0 = float(np.asarray(F.digitize(p0, np.float64(0.0))))
        tv = t_pids >= 0
        tp, ta = t_pids[tv], t_adc[tv]

        def aligned_target(u):
            """The target ADC of each simulated row (digitize(0) where the
            target lacks the pixel) and the constant of target rows the
            prediction lacks."""
            vp = u[u >= 0]
            pos = np.searchsorted(tp, vp)
            ok = (pos < tp.size) & (tp[np.minimum(pos, tp.size - 1)] == vp)
            tgt = np.full((vp.size, t_adc.shape[1]), adc0)
            tgt[ok] = ta[pos[ok]]
            return tgt, float(((adc0 - ta[~np.isin(tp, vp)]) ** 2).sum())

        def loss(p):
            """Sum-of-squared-ADC loss and the cotangent functional
            sum(c * ADC) (c fixed below) at p, with the decisions."""
            u, adc, ticks = run(p)
            tgt, const = aligned_target(u)
            a = adc[u >= 0]
            lin = float((cot * a).sum()) if cot is not None else 0.0
            return float(((a - tgt) ** 2).sum()) + const, lin, u, ticks

        # the perturbed parameters: the first draw at which the float64 run
        # makes the 32-bit run's discrete decisions (pixel ids, every
        # crossing tick, every transverse bin's pixel and sub-pixel LUT index
        # as simulate_drift_new returns them), so that its derivative is the
        # one jax.grad takes at the 32-bit decisions
        rng = np.random.default_rng(case["theta_seed"])
        cot = None
        for draw in range(20):
            theta = {k: float(getattr(p0, k)) * (1 + 0.05 * rng.standard_normal()) for k in GRAD_PARAMS}
            p = p0.replace(**theta)
            L, _, u_c, ticks_c = loss(p)
            bins64, times_c = run.bins, run.times
            u32, adc32, ticks32 = run(p, x64=False)
            same_bins = all(np.array_equal(a, b) for a, b in zip(run.bins, bins64))
            print(f"  draw {draw}: pixel ids {np.array_equal(u32, u_c)}, ticks {np.array_equal(ticks32, ticks_c)}, "
                  f"bins {same_bins}")
            if np.array_equal(u32, u_c) and np.array_equal(ticks32, ticks_c) and same_bins:
                break
        else:
            raise RuntimeError(f"{name}: no draw with the same decisions in 32 and 64 bits")
        # the cotangent jax.grad of the loss pulls back at the 32-bit run:
        # 2 (ADC - target) on the simulated rows
        tgt32, _ = aligned_target(u32)
        cot = 2 * (adc32[u32 >= 0] - tgt32)
        grad, vjp, steps, halvings = [], [], [], []
        for k in GRAD_PARAMS:
            h = 1e-6 * abs(theta[k])
            for n_half in range(25):
                lp, cp, up, tkp = loss(p.replace(**{k: theta[k] + h}))
                times_p = run.times
                lm, cm, um, tkm = loss(p.replace(**{k: theta[k] - h}))
                times_m = run.times
                same = all(np.array_equal(a, b) for a, b in ((up, u_c), (um, u_c), (tkp, ticks_c), (tkm, ticks_c),
                                                             *zip(times_p, times_c), *zip(times_m, times_c)))
                if same:
                    break
                h *= 0.5
            assert same, f"{name}/{k}: a discrete decision changes within every step tried"
            grad.append((lp - lm) / (2 * h))
            vjp.append((cp - cm) / (2 * h))
            steps.append(h)
            halvings.append(n_half)
        cfg = dict(case, event=[case["event"][0], case["event"][1]], response_seed=RESPONSE_SEED,
                   response_crc32=response_checksum(resp), fields=list(fields), grad_params=list(GRAD_PARAMS))
        out[f"{name}/config"] = np.array(json.dumps(cfg))
        out[f"{name}/tracks"] = tracks
        out[f"{name}/theta"] = np.array([theta[k] for k in GRAD_PARAMS])
        out[f"{name}/target_pixels"] = tp
        out[f"{name}/target_adc"] = ta
        out[f"{name}/theta_draw"] = np.array(draw)
        out[f"{name}/pixels32"] = u32[u32 >= 0]
        out[f"{name}/ticks32"] = ticks32[u32 >= 0]
        out[f"{name}/adc32"] = adc32[u32 >= 0].astype(np.float32)
        out[f"{name}/loss"] = np.array(L)
        out[f"{name}/fd_step"] = np.array(steps)
        out[f"{name}/fd_halvings"] = np.array(halvings)
        out[f"{name}/fd_gradient"] = np.array(grad)
        out[f"{name}/cotangent"] = cot
        out[f"{name}/fd_vjp"] = np.array(vjp)
        print(f"{name}: {tracks.shape[0]} segments, {int((u_c >= 0).sum())} pixels, loss {L:.6g}, draw {draw}")
        for k, g, gv, h, nh in zip(GRAD_PARAMS, grad, vjp, steps, halvings):
            print(f"  d/d{k}: loss {g:.9g}, c.ADC {gv:.9g} (step {h:.3g}, halvings {nh})")
    np.savez_compressed(OUT, **out)
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
