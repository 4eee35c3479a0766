"""The device deviate streams of the thermostats (mdt_rng_deviates reads out exactly what
the Langevin, PILE, Andersen and refill code draws).

- The uniforms are the Philox4x32-10 stream of the numpy restatement bit for bit (that
  restatement is pinned on the generator's published known-answer vectors), on several
  (seed, trajectory, step, stream) keys.
- The normals equal the restatement's FP32 Box-Muller within 4e-6 (FP32 log and cos).
- 2^22 normals have the moments of N(0, 1) (mean, variance, skewness, excess kurtosis
  within 5 standard errors), pass a Kolmogorov-Smirnov test against the normal CDF, have
  the normal tail frequencies beyond 3 and 4 sigma (within 5 binomial standard deviations)
  and no |z| beyond the 24-bit Box-Muller bound sqrt(2 ln 2^24) = 5.77, and neither
  neighbouring slots nor two streams on the same slots are correlated.  The reference
  draws in FP64 (src/useful_things.f90:121-173); these are the properties its noise has
  that the thermostats rely on."""
import ctypes as ct
import math

import numpy as np
import pytest

from md_tian2_gb300._lib import load
from oracle import philox

pytestmark = pytest.mark.gpu
KEYS = [(2024, 0, 0, 1), (2024, 17, 123456, 2), (0xDEADBEEF12345678, 4095, 9, 3), (5, 1, 2**31 - 1, 5)]


def _draw(kind, seed, traj, step, stream, n):
    lib = load()
    out = np.empty(n)
    rc = lib.mdt_rng_deviates(kind, ct.c_uint64(seed), traj, step, stream, n,
                              out.ctypes.data_as(ct.POINTER(ct.c_double)))
    assert rc == 0, rc
    return out


@pytest.mark.parametrize("key", KEYS)
def test_uniforms_are_the_philox_stream(built_lib, key):
    n = 1 << 16
    u = _draw(1, *key, n)
    assert np.array_equal(u, philox.uniforms(*key, n))


@pytest.mark.parametrize("key", KEYS)
def test_normals_are_fp32_box_muller_of_the_stream(built_lib, key):
    n = 1 << 16
    z = _draw(0, *key, n)
    assert np.abs(z - philox.normals(*key, n)).max() < 4e-6


def test_normal_moments_tails_and_independence(built_lib):
    from scipy import stats
    n = 1 << 22
    z = _draw(0, 2024, 3, 77, 1, n)
    se = 1.0 / math.sqrt(n)
    assert abs(z.mean()) < 5 * se
    assert abs(z.var() - 1.0) < 5 * math.sqrt(2.0) * se
    assert abs(stats.skew(z)) < 5 * math.sqrt(6.0) * se
    assert abs(stats.kurtosis(z)) < 5 * math.sqrt(24.0) * se
    assert stats.kstest(z, "norm").pvalue > 1e-4
    for k in (3.0, 4.0):
        p = 2.0 * stats.norm.sf(k)
        cnt = int(np.sum(np.abs(z) > k))
        assert abs(cnt - n * p) < 5 * math.sqrt(n * p * (1 - p)), (k, cnt, n * p)
    assert np.abs(z).max() <= math.sqrt(2.0 * math.log(2.0 ** 24)) + 1e-5
    assert abs(np.corrcoef(z[:-1], z[1:])[0, 1]) < 5 * se
    z2 = _draw(0, 2024, 3, 77, 2, n)
    assert abs(np.corrcoef(z, z2)[0, 1]) < 5 * se


def test_uniform_distribution(built_lib):
    from scipy import stats
    u = _draw(1, 99, 1, 1, 4, 1 << 20)
    assert u.min() >= 0.0 and u.max() < 1.0
    assert stats.kstest(u, "uniform").pvalue > 1e-4


def test_bad_arguments_are_rejected(built_lib):
    lib = load()
    out = np.empty(4)
    p = out.ctypes.data_as(ct.POINTER(ct.c_double))
    assert lib.mdt_rng_deviates(2, ct.c_uint64(1), 0, 0, 1, 4, p) < 0  # kind
    assert lib.mdt_rng_deviates(0, ct.c_uint64(1), 0, 0, 6, 4, p) < 0  # stream
    assert lib.mdt_rng_deviates(0, ct.c_uint64(1), -1, 0, 1, 4, p) < 0  # trajectory
    assert lib.mdt_rng_deviates(0, ct.c_uint64(1), 0, 0, 1, 4, None) < 0
