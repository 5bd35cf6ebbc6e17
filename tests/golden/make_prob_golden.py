"""Golden vectors of the reference's probabilistic front end, from its own source.

Runs larnd-sim-jax's ``simulate_wfs`` (sim_jax.py:689-736) on a seeded muon
event, takes rows of those waveforms (the most charged ones, a random
sample of the others and an all-zero row), and runs on them the
reference's ``get_adc_values_average_noise_vmap`` (fee_jax.py:386-461, the
beam search of ``_find_one_hit_step`` :334-384 with ``log_diff_ndtr`` and
the soft clamps :13-53), ``simulate_probabilistic`` (sim_jax.py:771-813)
and ``get_average_hit_values`` (fee_jax.py:463-480, on the probabilities
exp(log p)), with the reference's modules imported through the numpy
stand-in of jax_numpy_standin.py (make_lut_golden.load_reference).  The
stand-in's ``jax.scipy.special.log_ndtr`` is scipy's, evaluated in float64
and rounded to float32, where JAX evaluates its float32 piecewise form.

Each case stores the waveform rows (non-zero entries) and their pixel ids,
the options, the entries of the log-probability and charge distributions
whose log-probability exceeds -60, the digitised distribution's entries
there, and per (pixel, hit) the expected tick, the expected ADC and the
total probability, in prob_ref.npz.

Usage: python tests/golden/make_prob_golden.py /path/to/larnd-sim-jax   (or LARNDSIM_JAX_SRC=/path/to/larnd-sim-jax)
"""

import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from make_lut_golden import RESPONSE_SEED, load_reference, make_event, response_checksum  # noqa: E402

from larndsim_gb300 import workloads  # noqa: E402

OUT = HERE / "prob_ref.npz"
KEEP_LOGP = -60.0

CASES = {
    "prob_muons": dict(event=("muon", dict(seed=51, n_tracks=3)), n=1, L=150, n_templates=10, lut=15,
                       rows=dict(top=32, random=15, seed=0), fee_paths_scaling=20, reset_noise=900.0),
    "prob_muons_k8": dict(event=("muon", dict(seed=52, n_tracks=2)), n=1, L=150, n_templates=10, lut=15,
                          rows=dict(top=16, random=7, seed=1), fee_paths_scaling=8, reset_noise=600.0),
}


def main():
    C, F, S, base = load_reference()
    import jax.numpy as jnp

    out = {}
    tmp = Path(tempfile.mkdtemp())
    for name, case in CASES.items():
        S.size_history_dict.clear()
        p = base.replace(long_diff_template=jnp.linspace(0.001, 10, case["n_templates"]),
                         number_pix_neighbors=case["n"], signal_length=case["L"], time_window=case["L"],
                         RESET_NOISE_CHARGE=0, UNCORRELATED_NOISE_CHARGE=0)
        resp = workloads.synthetic_response(seed=RESPONSE_SEED, nx=case["lut"], ny=case["lut"])
        np.save(tmp / f"{name}.npy", resp)
        tmpl, p = C.load_lut(str(tmp / f"{name}.npy"), p)
        tracks, fields = make_event(*case["event"])
        wfs, unique = S.simulate_wfs(p, tmpl, jnp.asarray(tracks), tuple(fields))
        wfs, unique = np.asarray(wfs), np.asarray(unique)

        valid = np.flatnonzero(unique >= 0)
        charge = np.abs(wfs[valid]).sum(axis=1)
        top = valid[np.argsort(-charge, kind="stable")[:case["rows"]["top"]]]
        rest = np.setdiff1d(valid, top)
        rng = np.random.default_rng(case["rows"]["seed"])
        pick = rng.choice(rest, min(case["rows"]["random"], rest.size), replace=False)
        sel = np.sort(np.concatenate([top, pick]))
        rows = np.concatenate([wfs[sel], np.zeros((1, wfs.shape[1]), np.float32)])
        row_pixels = np.concatenate([unique[sel], np.array([-1], unique.dtype)])

        pp = p.replace(RESET_NOISE_CHARGE=case["reset_noise"], fee_paths_scaling=case["fee_paths_scaling"])
        log_prob, charge_d = F.get_adc_values_average_noise_vmap(pp, jnp.asarray(rows))
        adcs_d, px, py, ticks_prob, event = S.simulate_probabilistic(pp, jnp.asarray(rows), jnp.asarray(row_pixels))
        e_tick, e_adc, lam = F.get_average_hit_values(np.exp(np.asarray(ticks_prob)), adcs_d)
        log_prob, charge_d, adcs_d = np.asarray(log_prob), np.asarray(charge_d), np.asarray(adcs_d)
        assert np.array_equal(log_prob, np.asarray(ticks_prob))
        for a in (log_prob, charge_d, e_tick, e_adc, lam):
            assert not np.isnan(np.asarray(a)).any(), f"{name}: NaN in the reference outputs"
        keep = np.nonzero(log_prob > KEEP_LOGP)
        r_nz, c_nz = np.nonzero(rows)
        cfg = dict(case, event=[case["event"][0], case["event"][1]], response_seed=RESPONSE_SEED,
                   response_crc32=response_checksum(resp), fields=list(fields), keep_logp=KEEP_LOGP)
        out[f"{name}/config"] = np.array(json.dumps(cfg))
        out[f"{name}/rows_shape"] = np.array(rows.shape, np.int64)
        out[f"{name}/rows_row"] = r_nz.astype(np.int32)
        out[f"{name}/rows_tick"] = c_nz.astype(np.int16)
        out[f"{name}/rows_value"] = rows[r_nz, c_nz]
        out[f"{name}/row_pixels"] = row_pixels
        out[f"{name}/dist_shape"] = np.array(log_prob.shape, np.int64)
        out[f"{name}/keep_pixel"] = keep[0].astype(np.int32)
        out[f"{name}/keep_hit"] = keep[1].astype(np.int8)
        out[f"{name}/keep_tick"] = keep[2].astype(np.int16)
        out[f"{name}/log_prob"] = log_prob[keep]
        out[f"{name}/charge"] = charge_d[keep]
        out[f"{name}/adcs"] = adcs_d[keep]
        out[f"{name}/pixel_x"] = np.asarray(px)
        out[f"{name}/pixel_y"] = np.asarray(py)
        out[f"{name}/event"] = np.asarray(event)
        out[f"{name}/expected_ticks"] = np.asarray(e_tick)
        out[f"{name}/expected_adcs"] = np.asarray(e_adc)
        out[f"{name}/lambda"] = np.asarray(lam)
        print(f"{name}: {rows.shape[0]} rows, {keep[0].size} kept entries, "
              f"sum lambda {float(np.asarray(lam).sum()):.3f}")
    np.savez_compressed(OUT, **out)
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
