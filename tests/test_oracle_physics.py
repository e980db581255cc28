"""Pins the oracle's DCMIP simple physics (src/simple_physics_v5_1.f90, Reed
and Jablonowski 2012) before it is used to check the GPU.

- An independent numpy restatement, vectorised over columns, that solves the
  implicit boundary-layer diffusion as a banded linear system with scipy's
  solve_banded (the reference eliminates it by hand, bottom up), must give
  the oracle's columns to 1e-12.
- Large-scale condensation conserves moist enthalpy level by level
  (cp dT + L dq = 0) and the precipitation rate is the column integral of
  the condensation.
- The implicit diffusion is in flux form: it conserves the pressure-weighted
  column sums of u and v apart from the surface drag on the lowest level.
"""
import numpy as np
import pytest
from scipy.linalg import solve_banded

G, RAIR, CPAIR, LV, RH2O = 9.80616, 287.0, 1.0045e3, 2.5e6, 461.5
EPS, ZVIR = RAIR / RH2O, RH2O / RAIR - 1.0
C, SST, T0, E0, RHOW = 0.0011, 302.15, 273.16, 610.78, 1000.0
CD0, CD1, CM, V20, P0 = 0.0007, 0.000065, 0.002, 20.0, 1.0e5
PBLTOP, PBLCONST = 85000.0, 10000.0


def columns(ncol, n, seed, strong=False):
    rng = np.random.default_rng(seed)
    ps = 1.0e5 + 1500 * rng.standard_normal(ncol)
    eta = np.linspace(0, 1, n + 1) ** 1.3
    ak = 2000.0 * np.sin(np.pi * eta) * (1 - eta)
    bk = eta
    pint = ak[None, :] + bk[None, :] * ps[:, None]
    pint[:, 0] = 0.0
    pmid = 0.5 * (pint[:, 1:] + pint[:, :-1])
    pmid[:, 0] = 0.6 * pint[:, 1]
    sig = pmid / ps[:, None]
    t = 300.0 * sig ** 0.19 + 3 * rng.standard_normal((ncol, n))
    qsat = EPS * E0 / pmid * np.exp(-LV / RH2O * (1 / t - 1 / T0))
    q = qsat * (0.6 + 0.6 * rng.random((ncol, n)))  # some levels supersaturated
    w = 25.0 if strong else 8.0
    u = w * (0.5 + rng.random((ncol, n)))
    v = 0.5 * w * rng.standard_normal((ncol, n))
    lat = np.deg2rad(rng.uniform(-80, 80, ncol))
    return lat, t, q, u, v, pmid, pint, ps


def np_simple(dtime, lat, t, q, u, v, pmid, pint, ps, test, turbflux):
    t, q, u, v = t.copy(), q.copy(), u.copy(), v.copy()
    ncol, n = t.shape
    pdel = pint[:, 1:] - pint[:, :-1]
    za = RAIR / G * t[:, -1] * (1 + ZVIR * q[:, -1]) * 0.5 * (np.log(ps) - np.log(pint[:, n - 1]))
    if test == 1:
        pi = np.pi
        etav = (1 - 0.252) * 0.5 * pi
        q0 = float(np.float32(0.021))
        s, c = np.sin(lat), np.cos(lat)
        tsurf = (288.0 + pi * 35.0 / RAIR * 1.5 * np.sin(etav) * np.sqrt(np.cos(etav)) *
                 ((-2 * s ** 6 * (c ** 2 + 1 / 3) + 10 / 63) * 35.0 * np.cos(etav) ** 1.5 +
                  (8 / 5 * c ** 3 * (s ** 2 + 2 / 3) - pi / 4) * 6371220.0 * 7.29212e-5 * 0.5)) / \
                (1 + ZVIR * q0 * np.exp(-(lat / (2 * pi / 9)) ** 4))
    else:
        tsurf = np.full(ncol, SST)
    qsat = EPS * E0 / pmid * np.exp(-LV / RH2O * (1 / t - 1 / T0))
    tmp = np.where(q > qsat, (q - qsat) / dtime / (1 + LV / CPAIR * (EPS * LV * qsat / (RAIR * t ** 2))), 0.0)
    t += LV / CPAIR * tmp * dtime
    q -= tmp * dtime
    precl = (tmp * pdel).sum(axis=1) / (G * RHOW)
    if not turbflux:
        return t, q, u, v, precl
    wind = np.hypot(u[:, -1], v[:, -1])
    cd = np.where(wind < V20, CD0 + CD1 * wind, CM)
    kms, kes = cd * wind * za, C * wind * za
    taper = np.where(pint >= PBLTOP, 1.0, np.exp(-((PBLTOP - pint) ** 2) / PBLCONST ** 2))
    km, ke = kms[:, None] * taper, kes[:, None] * taper  # interfaces 0..n (n: the surface)
    qsats = EPS * E0 / ps * np.exp(-LV / RH2O * (1 / tsurf - 1 / T0))
    u[:, -1] /= 1 + cd * wind * dtime / za
    v[:, -1] /= 1 + cd * wind * dtime / za
    t[:, -1] = (t[:, -1] + C * wind * tsurf * dtime / za) / (1 + C * wind * dtime / za)
    q[:, -1] = (q[:, -1] + C * wind * qsats * dtime / za) / (1 + C * wind * dtime / za)
    rho = pint[:, 1:n] / (RAIR * (t[:, 1:] + t[:, :-1]) / 2)
    x = dtime * G * G * rho * rho / (pmid[:, 1:] - pmid[:, :-1])  # interfaces 1..n-1
    kap = RAIR / CPAIR
    theta = (P0 / pmid) ** kap * t
    out = []
    for k_i, fields in ((km, (u, v)), (ke, (theta, q))):
        ca = np.zeros((ncol, n))
        cc = np.zeros((ncol, n))
        ca[:, :-1] = 1 / pdel[:, :-1] * k_i[:, 1:n] * x
        cc[:, 1:] = 1 / pdel[:, 1:] * k_i[:, 1:n] * x
        for f in fields:
            sol = np.empty_like(f)
            for i in range(ncol):
                ab = np.zeros((3, n))
                ab[0, 1:] = -ca[i, :-1]  # superdiagonal
                ab[1] = 1 + ca[i] + cc[i]
                ab[2, :-1] = -cc[i, 1:]  # subdiagonal
                sol[i] = solve_banded((1, 1), ab, f[i])
            out.append(sol)
    u, v, theta, q = out
    t = theta * (pmid / P0) ** kap
    return t, q, u, v, precl


@pytest.mark.parametrize("test,turbflux,strong", [(0, True, False), (0, True, True), (1, True, False),
                                                  (1, False, False)])
def test_oracle_columns_match_banded_solve(oracle_mod, test, turbflux, strong):
    args = columns(40, 30, seed=3 + test, strong=strong)
    a = oracle_mod.simple_columns(1200.0, *args, test, turbflux)
    b = np_simple(1200.0, *args, test, turbflux)
    for x, y, name in zip(a, b, ("t", "q", "u", "v", "precl")):
        np.testing.assert_allclose(x, y, rtol=1e-12, atol=1e-15 * np.abs(y).max(), err_msg=name)
    assert (a[4] > 0).any()  # condensation happened


def test_condensation_conserves_moist_enthalpy(oracle_mod):
    lat, t, q, u, v, pmid, pint, ps = columns(30, 24, seed=11)
    dt = 900.0
    t1, q1, u1, v1, precl = oracle_mod.simple_columns(dt, lat, t, q, u, v, pmid, pint, ps, 0, False)
    np.testing.assert_allclose(CPAIR * (t1 - t) + LV * (q1 - q), 0.0, atol=1e-8)
    pdel = np.diff(pint, axis=1)
    np.testing.assert_allclose(precl, ((q - q1) / dt * pdel).sum(axis=1) / (G * RHOW), rtol=1e-12)
    np.testing.assert_array_equal(u1, u)
    np.testing.assert_array_equal(v1, v)
    qsat1 = EPS * E0 / pmid * np.exp(-LV / RH2O * (1 / t1 - 1 / T0))
    cond = q1 < q
    assert cond.any()
    np.testing.assert_allclose(q1[cond], qsat1[cond], rtol=0.02)  # adjusted to saturation (linearised)


def test_diffusion_conserves_column_momentum_but_the_surface_drag(oracle_mod):
    lat, t, q, u, v, pmid, pint, ps = columns(20, 26, seed=12)
    dt = 1200.0
    t1, q1, u1, v1, _ = oracle_mod.simple_columns(dt, lat, t, q, u, v, pmid, pint, ps, 0, True)
    pdel = np.diff(pint, axis=1)
    za = RAIR / G * t[:, -1] * (1 + ZVIR * q[:, -1]) * 0.5 * (np.log(ps) - np.log(pint[:, -2]))
    wind = np.hypot(u[:, -1], v[:, -1])
    cd = np.where(wind < V20, CD0 + CD1 * wind, CM)
    for a, a1 in ((u, u1), (v, v1)):
        s = a.copy()
        s[:, -1] = a[:, -1] / (1 + cd * wind * dt / za)
        np.testing.assert_allclose((pdel * a1).sum(axis=1), (pdel * s).sum(axis=1), rtol=1e-12)
        assert not np.allclose(a1, s)  # mixing did act
