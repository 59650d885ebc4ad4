"""Photon-count draws against the Poisson law, on the GPU through the C-ABI.

dvs_noise_poisson draws counts exactly as the circuit kernels do.  Generator
0 is the reference's stream (curand_init(seed, i, 0) then poisson_electrons,
include/dvs/photon_noise.cuh:4-9); it gets the reference's own check of
tests/test_sensor.cu:58-64 -- 65,536 draws with seed 42 at means 0.1, 10 and
1000, the mean within 6 standard errors and the variance within 7 %.
Generator 1 is the precision mode's Philox sampler (CDF inversion below a
mean of 10, Hormann's PTRS from 10 to 1e6, the rounded normal above); it gets
the same moments on 2^20 draws at means on both sides of every switch, plus a
chi-square goodness-of-fit test against the Poisson pmf at p = 1e-6.
"""
import ctypes as C
import math

import numpy as np
import pytest

from dvsrender4deepspace_gb300 import _capi

pytestmark = pytest.mark.gpu


def draws(generator, lam, n, seed=42):
    lib = _capi.load()
    out = np.empty(n, dtype=np.float64)
    r = lib.dvs_noise_poisson(generator, lam, seed, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    assert r == _capi.DVS_OK, lib.dvs_last_error()
    return out


def poisson_pmf(k, lam):
    return np.exp(k * math.log(lam) - lam - np.array([math.lgamma(float(x) + 1) for x in k]))


def chi_square_p(values, lam):
    """Upper-tail p-value of the chi-square statistic over bins of expected count >= 20."""
    from scipy import stats
    n = len(values)
    lo, hi = int(max(0, math.floor(lam - 8 * math.sqrt(lam) - 5))), int(math.ceil(lam + 8 * math.sqrt(lam) + 10))
    ks = np.arange(lo, hi + 1)
    expected = n * poisson_pmf(ks, lam)
    inside = values[(values >= lo) & (values <= hi)].astype(np.int64) - lo
    observed = np.bincount(inside, minlength=len(ks)).astype(np.float64)
    # merge bins from both tails inward until every bin expects >= 20
    obs_b, exp_b, acc_o, acc_e = [], [], 0.0, 0.0
    for o, e in zip(observed, expected):
        acc_o += o
        acc_e += e
        if acc_e >= 20:
            obs_b.append(acc_o)
            exp_b.append(acc_e)
            acc_o = acc_e = 0.0
    obs_b[-1] += acc_o + (values > hi).sum() + (values < lo).sum()
    exp_b[-1] += acc_e + n - expected.sum()
    obs_b, exp_b = np.array(obs_b), np.array(exp_b)
    chi2 = float(((obs_b - exp_b) ** 2 / exp_b).sum())
    return stats.chi2.sf(chi2, len(obs_b) - 1), chi2, len(obs_b) - 1


@pytest.mark.parametrize("lam", [0.1, 10.0, 1000.0])
def test_reference_stream_mean_and_variance(lam):
    # tests/test_sensor.cu:58-64, same sample size, seed and bounds
    v = draws(0, lam, 65536, seed=42)
    mean, var = v.mean(), v.var()
    assert abs(mean - lam) < 6 * math.sqrt(lam / len(v)), (mean, lam)
    assert abs(var - lam) < 0.07 * lam, (var, lam)
    assert np.all(v == np.floor(v)) and v.min() >= 0


@pytest.mark.parametrize("lam", [0.1, 1.0, 5.0, 9.99, 10.0, 10.5, 30.0, 60.0, 64.0, 70.0, 200.0, 1000.0, 1e5])
def test_philox_sampler_is_poisson(lam):
    pytest.importorskip("scipy")
    n = 1 << 20
    v = draws(1, lam, n, seed=7)
    assert np.all(v == np.floor(v)) and v.min() >= 0
    mean, var = v.mean(), v.var()
    assert abs(mean - lam) < 6 * math.sqrt(lam / n), (mean, lam)
    # standard error of the sample variance of a Poisson(lam) sample: sqrt((lam + 2 lam^2) / n)
    assert abs(var - lam) < 6 * math.sqrt((lam + 2 * lam * lam) / n), (var, lam)
    p, chi2, dof = chi_square_p(v, lam)
    assert p > 1e-6, (lam, chi2, dof, p)


def test_philox_above_the_normal_switch():
    # above 1e6 both generators use the reference's rounded normal approximation
    lam, n = 4e6, 1 << 18
    v = draws(1, lam, n, seed=3)
    assert abs(v.mean() - lam) < 6 * math.sqrt(lam / n)
    assert abs(v.var() - lam) < 0.05 * lam


def test_draws_are_seeded_and_independent_of_the_generator_call():
    a, b = draws(1, 12.0, 4096, seed=11), draws(1, 12.0, 4096, seed=11)
    assert np.array_equal(a, b)
    c = draws(1, 12.0, 4096, seed=12)
    assert not np.array_equal(a, c)
    x, y = draws(0, 3.0, 4096, seed=5), draws(0, 3.0, 4096, seed=5)
    assert np.array_equal(x, y)
