"""Pins the FP64 oracle's dynamics: semi-implicit inverses against scipy's
LAPACK dgetrf/dgetri (the routines src/semimp_data.f90:248-249 calls), the
IMEX tableau conditions of src/semimp_data.f90:135-160, and physical
known answers of src/run.f90::advance with Held-Suarez forcing."""
import numpy as np
import pytest
from scipy.linalg import lapack

from gdpy import inputs


def f32(x):
    return float(np.float32(x))


def make(oracle_mod, T=42, nlon=128, nlat=64, nlev=20, **kw):
    ak, bk = inputs.hybrid_coords(nlev)
    return oracle_mod.Oracle(T, nlon, nlat, nlev, ak, bk, **kw)


def test_semimp_inverses_match_lapack(oracle_mod):
    o = make(oracle_mod, T=42, nlev=20, dt=1200.0)
    s = o.semimp()
    consts = [f32(1.0 / 6.0), f32(1.0 / 3.0), f32(1.0 / 4.0)]
    for si, c in enumerate(consts):
        for n in [0, 1, 7, 42]:
            y = np.eye(20) + (c * 1200.0) ** 2 * n * (n + 1) * s["ym"]
            lu, piv, info = lapack.dgetrf(y)
            assert info == 0
            inv, info = lapack.dgetri(lu, piv)
            assert info == 0
            np.testing.assert_allclose(s["d_hyb_m"][si, n], inv, rtol=1e-12, atol=1e-14)
    # ym = tor (x) sv + amhyb bmhyb (semimp_data.f90:225-234)
    ym = np.outer(s["tor_hyb"], s["svhyb"]) + s["amhyb"] @ s["bmhyb"]
    np.testing.assert_allclose(s["ym"], ym, rtol=1e-13)


def test_imex_tableau_conditions():
    a21, a31, a32 = f32(1 / 3), f32(1 / 6), f32(1 / 2)
    aa21, aa22, aa31, aa32, aa33 = f32(1 / 6), f32(1 / 6), f32(1 / 3), 0.0, f32(1 / 3)
    b1, b2, b3 = 0.5, -0.5, 1.0
    bb1, bb2, bb3, bb4 = f32(3 / 8), 0.0, f32(3 / 8), f32(1 / 4)
    assert abs(a21 - (aa21 + aa22)) < 1e-5 and abs(a31 + a32 - (aa31 + aa32 + aa33)) < 1e-5
    assert abs(b1 + b2 + b3 - 1) < 1e-5 and abs(bb1 + bb2 + bb3 + bb4 - 1) < 1e-5
    assert abs(a21 * b2 + (a31 + a32) * b3 - 0.5) < 1e-5
    assert abs((aa21 + aa22) * bb2 + (aa31 + aa32 + aa33) * bb3 + bb4 - 0.5) < 1e-5


def test_isothermal_rest_is_steady_adiabatic(oracle_mod):
    o = make(oracle_mod, T=21, nlon=64, nlat=32, nlev=8, adiabatic=True, heldsuarez=False)
    st = inputs.hs_rest_state(21, 8, amp=0.0)
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    t = o.getdyntend(1)
    for k in ("dvrt", "ddiv", "dtv"):
        assert np.abs(t[k]).max() < 1e-12 * 300
    assert np.abs(t["dlnps"]).max() < 1e-16


@pytest.mark.parametrize("T,nlon,nlat", [(42, 128, 64), (62, 192, 94), (126, 384, 190)])
def test_balanced_jet_is_steady_adiabatic(oracle_mod, T, nlon, nlat):
    # a known answer for the whole of getdyntend: the barotropic jet u = 35
    # sin^2(2 phi) on an isothermal atmosphere, ln ps in gradient-wind balance
    # (the pressure-gradient force is -R T grad ln ps on every hybrid level), is
    # a steady state of the adiabatic equations, and the discrete tendencies
    # keep it to round-off (measured ddiv 2e-14 .. 2e-13 of f |vrt|, dvrt
    # ~1e-17, dTv and dlnps zero)
    L = 8
    o = make(oracle_mod, T=T, nlon=nlon, nlat=nlat, nlev=L, adiabatic=True, heldsuarez=False)
    st = inputs.balanced_jet_state(T, nlat, L, seed=0, tnoise=0.0)
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    t = o.getdyntend(1)
    scale = 2 * inputs.OMEGA * np.abs(st["vrt"]).max()
    assert np.abs(t["ddiv"]).max() < 1e-11 * scale
    assert np.abs(t["dvrt"]).max() < 1e-14 * scale
    assert np.abs(t["dtv"]).max() < 1e-14 * 300
    assert np.abs(t["dlnps"]).max() < 1e-16


def test_hs_step_mass_and_zonal_symmetry(oracle_mod):
    T, nlev = 21, 8
    o = make(oracle_mod, T=T, nlon=64, nlat=32, nlev=nlev, dt=1200.0)
    st = inputs.hs_rest_state(T, nlev, amp=0.0)
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    o.advance(3)
    s = o.get_state()
    deg, order = inputs.degree_order(T)
    for k in ("vrt", "div", "tv"):
        assert np.all(np.isfinite(s[k]))
        assert np.abs(s[k][:, order > 0]).max() < 1e-12 * max(1.0, np.abs(s[k]).max())
    # HS forcing spins up zonal flow from rest
    assert np.abs(s["vrt"][:, order == 0]).max() > 0
    d = o.diag()
    np.testing.assert_allclose(d["pdryini"], 1.0e5, rtol=1e-12)
    # dry-mass fixer: the global mean of exp(lnps) returns to pdryini
    ps = np.exp(o.spectogrd(s["lnps"][None])[0])
    aw = o.grid_info()["areawts"]
    pmean = (ps * aw[:, None]).sum()
    np.testing.assert_allclose(pmean, d["pdryini"], rtol=1e-10)


def test_hs_noise_case_runs(oracle_mod):
    o = make(oracle_mod, T=42, nlev=20, dt=1200.0)
    st = inputs.hs_rest_state(42, 20, seed=7)
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    o.advance(2)
    d = o.diag()
    assert np.isfinite(d["spdmax"]) and 900 < d["psmin"] <= d["psmax"] < 1100
