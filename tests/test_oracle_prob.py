"""The probabilistic front end's special functions in the oracle
(float32 restatements of jax.scipy.special.ndtr / log_ndtr, jax.nn.softplus,
jax.scipy.special.logsumexp, lax.top_k and the reference's log_diff_ndtr,
fee_jax.py:13-53) against float64 / arbitrary-precision values: the
accuracy the probabilistic parity tests rest on."""

import numpy as np
import pytest
from scipy import special

from oracle import reference_np as R

F = np.float32


def _rel(got, want):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    return np.abs(got - want) / np.maximum(np.abs(want), 1e-300)


def test_ndtr_float32_accuracy():
    """Within float32 rounding, widened in the lower tail by the roundings of
    the argument w = x * sqrt(0.5) (the float32 constant and the product),
    which the float32 formula shares: the relative condition number of
    erfc(w) is about 2 w^2."""
    x = np.linspace(-12, 8, 4001).astype(F)
    want = special.ndtr(x.astype(np.float64))
    keep = want > 1e-35
    w2 = 0.5 * x.astype(np.float64) ** 2
    tol = 2e-6 + 2 * w2 * 1.2e-7
    assert np.all(_rel(R.ndtr32(x)[keep], want[keep]) < tol[keep])


def test_log_ndtr_float32_accuracy_across_the_three_pieces():
    # below -10 the asymptotic series, up to 5 the log of the CDF, above it -ndtr(-x)
    x = np.concatenate([np.linspace(-60, -10.01, 500), np.linspace(-10, 5, 1501), np.linspace(5.01, 12, 200)])
    x = x.astype(F)
    want = special.log_ndtr(x.astype(np.float64))
    got = R.log_ndtr32(x).astype(np.float64)
    err = np.abs(got - want) / np.maximum(np.abs(want), 1.0)
    assert err.max() < 2e-6
    tiny = x > 5                                   # -ndtr(-x): relative accuracy of a tiny number
    assert _rel(got[tiny], want[tiny]).max() < 2e-5


def test_softplus_and_sigmoid():
    y = np.linspace(-120, 120, 2401).astype(F)
    assert _rel(R.softplus32(y)[y > -80], np.logaddexp(y.astype(np.float64), 0)[y > -80]).max() < 2e-6
    assert np.all(R.softplus32(y) >= 0) and R.softplus32(F(-200)) == 0
    assert np.abs(R.sigmoid32(y) - special.expit(y.astype(np.float64))).max() < 1e-7


def test_logsumexp():
    rng = np.random.default_rng(0)
    x = rng.normal(0, 30, (50, 20)).astype(F)
    x[3] = -np.inf
    want = special.logsumexp(x.astype(np.float64), axis=1)
    got = R.logsumexp32(x, axis=1)
    fin = np.isfinite(want)
    assert np.all(got[~fin] == -np.inf)
    assert (np.abs(got[fin] - want[fin]) / np.maximum(np.abs(want[fin]), 1)).max() < 2e-6


def test_top_k_order_matches_lax_top_k():
    x = np.array([[1.0, 3.0, 3.0, 2.0, -np.inf, 3.0]])
    np.testing.assert_array_equal(R.top_k_indices(x, 4), [[1, 2, 5, 3]])


@pytest.mark.parametrize("a,b", [(0.3, -0.4), (2.0, 1.0), (-3.0, -3.6), (-9.0, -11.0), (6.0, -1.0), (1.5, 1.0)])
def test_log_diff_ndtr_where_the_clamps_are_inactive(a, b):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 50
    exact = float(mpmath.log(mpmath.ncdf(a) - mpmath.ncdf(b)))
    got = float(R.log_diff_ndtr32(F(a), F(b)))
    # float32 arguments: the exact value at the rounded arguments
    exact32 = float(mpmath.log(mpmath.ncdf(float(F(a))) - mpmath.ncdf(float(F(b)))))
    assert abs(got - exact32) <= 2e-5 * max(1.0, abs(exact32)), (got, exact32, exact)


def test_log_diff_ndtr_clamps():
    # b >= a: the smooth where gives the -1000 floor
    assert float(R.log_diff_ndtr32(F(-1.0), F(-0.9))) == pytest.approx(-1000.0, abs=1e-3)
    # both arguments far in the upper tail: 1 - exp(lb - la) underflows to ~0 and
    # the soft floor _soft_max(., 1e-30, 1e10) returns 1e-30 + softplus(~0) / 1e10,
    # so the result is log(1e-30 + log(2) * 1e-10) (the reference's own clamp)
    v = float(R.log_diff_ndtr32(F(12.0), F(11.5)))
    assert v == pytest.approx(np.log(1e-30 + np.log(2) * 1e-10), abs=1e-4)


def _waveforms(seed, P=6, T=401):
    rng = np.random.default_rng(seed)
    w = np.full((P, T), 2.0, np.float32)             # small pedestal: no flat stretches
    for p in range(P):
        for _ in range(int(rng.integers(1, 4))):
            t0 = int(rng.integers(20, T - 80))
            w[p, t0:t0 + 30] += rng.uniform(300, 3000)
    return w


@pytest.mark.parametrize("seed", [0, 1])
def test_float32_beam_search_agrees_with_float64(seed):
    """The float32 restatement (the probabilistic parity reference) against
    the float64 one with the same top-K choices: the two share no code."""
    from larndsim_gb300 import consts
    p = consts.Params(RESET_NOISE_CHARGE=900.0, MAX_ADC_VALUES=4)
    w = _waveforms(seed)
    lp32, q32, top, n_exec = R.get_adc_values_average_noise(p, w, return_choices=True)
    lp64, q64 = R.beam_search64(p, w, top, n_exec)
    assert n_exec >= 1
    pr32, pr64 = np.exp(lp32.astype(np.float64)), np.exp(lp64)
    assert np.abs(pr32 - pr64).max() < 5e-5
    hi = lp64 > -5
    assert np.abs(lp32[hi] - lp64[hi]).max() < 5e-4
    scale = np.abs(q64).max(axis=-1, keepdims=True) + 1.0
    assert (np.abs(q32 - q64) / scale).max() < 1e-5
