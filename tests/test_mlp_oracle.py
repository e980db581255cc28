"""The learned closure's network oracle (oracle/mlp_oracle.py) against
finite differences and its BF16 rounding against exact cases; the network's
C-ABI entry points reject bad arguments without a GPU."""
import numpy as np
import pytest

import mlp_oracle as mo


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 3.0e-3], np.float32)
    r = mo.bf16(x)
    # ties to even: 1 + 2^-8 -> 1, 1 + 3 2^-8 -> 1 + 2^-6; exact values stay
    np.testing.assert_array_equal(r[:4], np.array([1.0, 1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -6], np.float32))
    assert r[4] == -2.5
    assert abs(r[5] - 3.0e-3) <= 3.0e-3 * 2 ** -8
    assert np.all(r.view(np.uint32) & 0xFFFF == 0)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    shp = mo.shapes(7, 11, 2, 5)
    n = sum(fo * fi + fo for fo, fi in shp)
    p = rng.standard_normal(n) * 0.4
    x = rng.standard_normal((13, 7))
    t = rng.standard_normal((13, 5))
    loss, g = mo.loss_grad(p, shp, x, t, round_weights=False)
    h = 1e-6
    for i in rng.choice(n, 40, replace=False):
        q = p.copy()
        q[i] += h
        lp, _ = mo.loss_grad(q, shp, x, t, round_weights=False)
        q[i] -= 2 * h
        lm, _ = mo.loss_grad(q, shp, x, t, round_weights=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), i


def test_gelu_derivative():
    z = np.linspace(-6, 6, 101)
    h = 1e-6
    fd = (mo.gelu(z + h) - mo.gelu(z - h)) / (2 * h)
    np.testing.assert_allclose(mo.gelu_d(z), fd, atol=1e-8)


def test_mlp_abi_rejects_bad_arguments():
    from gdpy import core

    with pytest.raises(core.GdError):
        core.Mlp(0, 8, 1, 4)
    with pytest.raises(core.GdError):
        core.Mlp(4, 8, 0, 4)
