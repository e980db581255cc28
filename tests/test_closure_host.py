"""Host logic of the learned-closure driver (gdpy/closure.py): spectral
truncation between m-major triangular layouts and the zonal-mean error
measure.  No GPU."""
import numpy as np

from gdpy import closure, inputs


def test_truncate_keeps_the_low_degrees_in_order():
    T_hi, T_lo = 12, 5
    deg_hi, ord_hi = inputs.degree_order(T_hi)
    deg_lo, ord_lo = inputs.degree_order(T_lo)
    spec = deg_hi * 100 + ord_hi + 1j * ord_hi  # a value that names (n, m)
    out = closure.truncate(spec, T_hi, T_lo)
    np.testing.assert_array_equal(out, deg_lo * 100 + ord_lo + 1j * ord_lo)
    # leading axes are carried along
    stack = np.stack([spec, 2 * spec])
    np.testing.assert_array_equal(closure.truncate(stack, T_hi, T_lo)[1], 2 * out)
    assert closure.truncate(spec, T_hi, T_hi).shape == spec.shape


def test_zonal_rmse_measures_zonal_means_only():
    nlat, nlon, L = 4, 6, 3
    rng = np.random.default_rng(0)
    a = rng.standard_normal((nlat * nlon, 3 * L + 1))
    b = a.copy()
    # a zero-mean wave along each latitude leaves the zonal means unchanged
    wave = np.cos(2 * np.pi * np.arange(nlon) / nlon)
    b.reshape(nlat, nlon, -1)[:, :, :L] += wave[None, :, None]
    assert max(closure.zonal_rmse(a, b, nlat, nlon, L)) < 1e-12
    # a uniform 2 K offset of T shows as an RMSE of 2
    c = a.copy()
    c[:, 2 * L:3 * L] += 2.0
    ru, rt = closure.zonal_rmse(c, a, nlat, nlon, L)
    assert ru == 0.0 and abs(rt - 2.0) < 1e-12
