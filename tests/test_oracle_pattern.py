"""Pins the CPU oracle of the stochastic pattern generator
(src/patterngenerator.f90 and the w3lib Mersenne twister,
src/w3lib/mersenne_twister.f) before it is used to check the GPU.

- MT19937 known answer: the C++ standard fixes the 10000th output of a
  default-seeded std::mt19937 at 4123659995; the oracle's twist and tempering,
  seeded the standard way, must give it (and agree with the C++ library).
- An independent numpy restatement of the w3lib stream (its 69069 seeding,
  the single-precision uniforms, the polar method) must reproduce the
  oracle's uniforms bit for bit and its Gaussians to the last ulp of log.
- random_gauss's pair caching makes the Gaussian stream independent of how
  it is split into calls.
- gaussian_spect's normalization gives the template pattern unit variance;
  AR(1) patterns have variance stdev^2 and lag-one correlation phi.
"""
import numpy as np
import pytest


def np_w3_uniform(seed, n):
    """w3lib random_setseed + random_number, restated with numpy uint32."""
    N, M = 624, 397
    mt = np.zeros(N, np.uint64)
    mt[0] = np.uint64(seed & 0xFFFFFFFF)
    for i in range(1, N):
        mt[i] = (69069 * int(mt[i - 1])) & 0xFFFFFFFF
    mt = [int(v) for v in mt]
    mti = N
    out = np.zeros(n, np.float32)
    for j in range(n):
        if mti >= N:
            for kk in range(N):
                y = (mt[kk] & 0x80000000) | (mt[(kk + 1) % N] & 0x7FFFFFFF)
                mt[kk] = mt[(kk + M) % N] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            mti = 0
        y = mt[mti]
        mti += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        y &= 0xFFFFFFFF
        s = y - (1 << 32) if y >= (1 << 31) else y
        two32 = np.float32(4294967296.0)
        f = np.float32(s)
        out[j] = (f + two32) / two32 if s < 0 else f / two32
    return out


def np_polar(u):
    """Numerical Recipes polar method on consecutive uniform pairs (float32)."""
    g, acc = [], []
    for k in range(0, len(u) - 1, 2):
        v1 = np.float32(2) * u[k] - np.float32(1)
        v2 = np.float32(2) * u[k + 1] - np.float32(1)
        r = v1 * v1 + v2 * v2
        acc.append(bool(r < 1))
        if r < 1:
            fac = np.sqrt(np.float32(-2) * np.log(r) / r)
            g += [v1 * fac, v2 * fac]
    return np.array(g, np.float32), np.array(acc)


def test_mt19937_known_answer(oracle_mod):
    mine, std = oracle_mod.mt_kat()
    assert std == 4123659995
    assert mine == 4123659995


@pytest.mark.parametrize("seed", [1, 12345, -7, 2**31 - 1])
def test_uniform_stream_matches_independent_restatement(oracle_mod, seed):
    n = 1500  # crosses two twists
    np.testing.assert_array_equal(oracle_mod.mt_uniform(seed, n), np_w3_uniform(seed, n))


def test_seed_zero_is_the_default_seed(oracle_mod):
    np.testing.assert_array_equal(oracle_mod.mt_uniform(0, 50), oracle_mod.mt_uniform(4357, 50))


def test_gaussian_stream_matches_independent_restatement(oracle_mod):
    seed, n = 2024, 800
    g = oracle_mod.mt_gauss(seed, [n])
    u = np_w3_uniform(seed, 4 * n)
    gn, acc = np_polar(u)
    assert 0.7 < acc.mean() < 0.86  # pi / 4 of the pairs land inside the unit disc
    np.testing.assert_allclose(g, gn[:n], rtol=4e-7, atol=1e-7)


def test_gaussian_stream_is_independent_of_call_split(oracle_mod):
    whole = oracle_mod.mt_gauss(99, [40])
    np.testing.assert_array_equal(oracle_mod.mt_gauss(99, [3, 5, 4, 7, 1, 20]), whole)
    np.testing.assert_array_equal(oracle_mod.mt_gauss(99, [1] * 40), whole)


def test_gaussian_moments(oracle_mod):
    g = oracle_mod.mt_gauss(31337, [200000]).astype(np.float64)
    assert abs(g.mean()) < 0.01
    assert abs(g.var() - 1.0) < 0.01


def _template_variance(vs, jcap, nf, normfact):
    """computevarspec of gaussian_spect's template pattern, in float64."""
    deg = np.concatenate([np.arange(m, jcap + 1) for m in range(jcap + 1)])
    order = np.concatenate([np.full(jcap + 1 - m, m) for m in range(jcap + 1)])
    s = np.sqrt(2 * deg + 1.0)
    re = np.where(order != 0, 1 / s, np.sqrt(2) / s)
    im = np.where(order != 0, 1 / s, 0.0)
    re[0] = im[0] = 0
    p2 = (vs * nf) ** 2 * (re ** 2 + im ** 2)
    return (np.where(order != 0, 1.0, 0.5) * p2).sum() / normfact


def test_variance_spectrum_normalization(oracle_mod):
    jcap = 62
    normfact = 2 * float(np.float32(np.pi))
    p = oracle_mod.PatternOracle(500e3, 900.0, 21600.0, 0.8, 7, jcap, normfact)
    vs, v1, phi = p.spectra()
    np.testing.assert_allclose(phi, np.exp(-900.0 / 21600.0), rtol=1e-7)
    nf = np.sqrt(normfact / jcap)
    np.testing.assert_allclose(_template_variance(vs, jcap, nf, normfact), 1.0, rtol=2e-6)
    # the spectrum decays with total wavenumber (Gaussian covariance)
    assert np.all(np.diff(v1) < 0)


def test_ar1_statistics(oracle_mod):
    jcap, stdev, tau, dt = 30, 0.6, 6 * 3600.0, 1800.0
    p = oracle_mod.PatternOracle(1000e3, dt, tau, stdev, 11, jcap)
    p.start()
    phi = p.spectra()[2]
    xs, var = [], []
    for _ in range(2000):
        p.advance(1)
        x = p.get()[0]
        xs.append(x)
        var.append(p.varspec())
    xs = np.array(xs)
    assert abs(np.mean(var) / stdev ** 2 - 1) < 0.1
    a, b = xs[:-1].ravel(), xs[1:].ravel()
    lag1 = np.real(np.vdot(a, b)) / np.real(np.vdot(a, a))
    assert abs(lag1 - phi) < 0.01
