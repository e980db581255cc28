"""The single-precision host entry points (gd_*_f: float _Complex spectral,
float grid arrays, the layout of the reference's default r_kind = 4 build,
src/kinds.f90:100) against the double entry points on the same context.

The float arrays are converted on the device, so each result is the double
entry point's result rounded to float (the inputs are float-representable):
agreement to FP32 rounding, 2^-24 relative to the field's max-norm, checked
at 1e-6.  A state set in single precision and read back in double is the
float state exactly.
"""
import numpy as np
import pytest

from gdpy import core, inputs
from helpers import rand_spec, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "tf32x3", "f64_eddy"])
def test_float_transforms_match_double(prec):
    T, nlon, nlat = 42, 128, 64
    ak, bk = inputs.hybrid_coords(4)
    g = core.Dycore(T, nlon, nlat, 4, ak, bk, precision=prec)
    a = rand_spec(T, 3, seed=3, slope=-1.0).astype(np.complex64)
    b = rand_spec(T, 3, seed=4, slope=-1.0).astype(np.complex64)
    a64, b64 = a.astype(np.complex128), b.astype(np.complex128)
    grid = g.spectogrd(a)
    assert grid.dtype == np.float32
    assert rel(grid, g.spectogrd(a64)) < 1e-6
    gf = grid.astype(np.float32)
    sp = g.grdtospec(gf)
    assert sp.dtype == np.complex64
    assert rel(sp, g.grdtospec(gf.astype(np.float64))) < 1e-6
    u, v = g.getuv(a, b)
    u64, v64 = g.getuv(a64, b64)
    assert rel(u, u64) < 1e-6 and rel(v, v64) < 1e-6
    vr, dv = g.getvrtdivspec(u, v)
    vr64, dv64 = g.getvrtdivspec(u.astype(np.float64), v.astype(np.float64))
    assert rel(vr, vr64) < 1e-6 and rel(dv, dv64) < 1e-6
    gx, gy = g.getgrad(a)
    gx64, gy64 = g.getgrad(a64)
    assert rel(gx, gx64) < 1e-6 and rel(gy, gy64) < 1e-6
    g.close()


@pytest.mark.parametrize("prec", ["fp64", "tf32x3"])
def test_float_state_round_trip_and_step(prec):
    T, nlon, nlat, L, nt = 42, 128, 64, 20, 2
    ak, bk = inputs.hybrid_coords(L)
    st = inputs.smooth_random_state(T, L, ntrac=nt, seed=9)
    f = {k: np.asarray(v).astype(np.complex64) for k, v in st.items()}
    g = core.Dycore(T, nlon, nlat, L, ak, bk, ntrac=nt, dt=900.0, precision=prec)
    g.set_state(f["vrt"], f["div"], f["tv"], f["lnps"], trc=f["trc"])
    back = g.get_state()  # double read of a float-set state: exact
    for k in ("vrt", "div", "tv", "lnps", "trc"):
        np.testing.assert_array_equal(back[k], f[k].astype(np.complex128))
    g.advance(2)
    s32 = g.get_state(single=True)
    s64 = g.get_state()
    for k in ("vrt", "div", "tv", "lnps", "trc"):
        assert s32[k].dtype == np.complex64
        np.testing.assert_array_equal(s32[k], s64[k].astype(np.complex64))
    # the same steps from the double entry point give the same state
    h = core.Dycore(T, nlon, nlat, L, ak, bk, ntrac=nt, dt=900.0, precision=prec)
    h.set_state(*(f[k].astype(np.complex128) for k in ("vrt", "div", "tv", "lnps")),
                trc=f["trc"].astype(np.complex128))
    h.advance(2)
    s = h.get_state()
    for k in ("vrt", "div", "tv", "lnps", "trc"):
        np.testing.assert_array_equal(s[k], s64[k])
    g.close()
    h.close()
