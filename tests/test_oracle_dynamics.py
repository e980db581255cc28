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


def test_hs_forcing_vs_numpy_restatement(oracle_mod):
    # the physics plugin of the Held-Suarez build (phy_run_hs.f90:42-77)
    # restated in numpy on the oracle's own transforms: Phillips layer
    # pressure from the interfaces p = ak + bk ps (top to bottom) for the
    # fields stored bottom to top, Teq = max(200, (p/p0)^(2/7) (315 - 60
    # sin^2 phi - 10 ln(p/p0) cos^2 phi)), blprof = max(0, (p/ps - 0.7) / 0.3),
    # dTv = (ka + (ks - ka) blprof cos^4 phi)(Teq - Tv), dvrt, ddiv = -kf
    # blprof (vrt, div), with the reference's single-precision constants
    # (measured: the tendencies within 9.4e-15 of their largest value, the
    # layer pressures within 3.6e-15)
    T, nlon, nlat, L = 42, 128, 64, 20
    ak, bk = inputs.hybrid_coords(L)
    o = oracle_mod.Oracle(T, nlon, nlat, L, ak, bk, dt=1200.0)
    st = inputs.hs_rest_state(T, L, seed=4, amp=2.0e-5)
    rng = np.random.default_rng(4)
    st["div"] = st["vrt"][::-1] * 0.3
    st["tv"] = st["tv"] + 0.0
    st["tv"][:, 1:30] += 0.5 * (rng.standard_normal((L, 29)) + 1j * rng.standard_normal((L, 29)))
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    o.getdyntend(3, inverse_only=True)  # the grid fields the plugin reads, as after getdyntend
    t = o.getphytend()
    prs_oracle = o.get_grid("prs")
    f32 = np.float32
    kappa = float(f32(287.05)) / float(f32(1004.6))
    sigbot = float(f32(0.7))
    kf = float(f32(1.0) / (f32(1.0) * f32(86400.0)))
    ka = float(f32(1.0) / (f32(40.0) * f32(86400.0)))
    ks = float(f32(1.0) / (f32(4.0) * f32(86400.0)))
    expo = float(f32(2.0) / f32(7.0))
    p0 = 1.0e5
    lat = o.grid_info()["lats"][:, None]
    sl, cl = np.sin(lat), np.cos(lat)
    ps = np.exp(o.spectogrd(st["lnps"][None])[0])
    vrtg, divg, tvg = o.spectogrd(st["vrt"]), o.spectogrd(st["div"]), o.spectogrd(st["tv"])
    pk = [ak[i] + bk[i] * ps for i in range(L + 1)]  # interfaces, top to bottom
    want = {k: np.zeros((L, o.nlm), np.complex128) for k in ("dtv", "dvrt", "ddiv")}
    for b in range(L):  # field level b (bottom to top) is layer L - 1 - b
        lo, up = pk[L - b], pk[L - 1 - b]
        prs = ((lo ** kappa * lo - up ** kappa * up) / ((kappa + 1.0) * (lo - up))) ** (1.0 / kappa)
        np.testing.assert_allclose(prs_oracle[b], prs, rtol=1e-13)  # calc_pressdata's Phillips pressure
        bl = np.maximum(0.0, (prs / ps - sigbot) / (1.0 - sigbot))
        teq = np.maximum(200.0, (prs / p0) ** expo * (315.0 - 60.0 * sl ** 2 - 10.0 * np.log(prs / p0) * cl ** 2))
        want["dtv"][b] = o.grdtospec(((ka + (ks - ka) * bl * cl ** 4) * (teq - tvg[b]))[None])[0]
        want["dvrt"][b] = o.grdtospec((-(bl * kf) * vrtg[b])[None])[0]
        want["ddiv"][b] = o.grdtospec((-(bl * kf) * divg[b])[None])[0]
    for k in ("dtv", "dvrt", "ddiv"):
        np.testing.assert_allclose(t[k], want[k], rtol=0, atol=1e-12 * np.abs(want[k]).max())
    assert np.abs(t["dlnps"]).max() == 0


def test_getomega_vs_numpy_restatement(oracle_mod):
    # getomega (dyn_run.f90:307-373) restated in numpy on the oracle's grid
    # winds and divergence and its transforms: cg = V . grad ln ps, the
    # top-down sums db (div dp) and cb (cg dbk), dlnps/dt = -db_N/ps - cb_N,
    # etadot at the interior interfaces, and omega/p from the workb / workc
    # terms with rlnp, alfa (pressure_data.f90:90-97; alfa at the top is the
    # single-precision log 2), dbk and ck (dyn_init.f90:58-60)
    # (measured 7.5e-16, 5.3e-16 and 2.3e-15 of the largest value)
    T, nlon, nlat, L = 42, 128, 64, 20
    ak, bk = inputs.hybrid_coords(L)
    o = oracle_mod.Oracle(T, nlon, nlat, L, ak, bk, dt=1200.0)
    st = inputs.hs_rest_state(T, L, seed=6, amp=2.0e-5)
    st["div"] = 0.4 * st["vrt"][::-1]
    st["lnps"] = st["lnps"].copy()
    rng = np.random.default_rng(6)
    st["lnps"][1:40] += 2e-3 * rng.standard_normal(39)
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    o.getdyntend(3, inverse_only=True)
    ug, vg, divg = o.get_grid("ug"), o.get_grid("vg"), o.get_grid("divg")  # bottom to top
    ps = np.exp(o.spectogrd(st["lnps"][None])[0])
    gx, gy = o.getgrad(st["lnps"][None])
    gx, gy = gx[0], gy[0]
    pk = np.array([ak[i] + bk[i] * ps for i in range(L + 1)])  # interfaces, top to bottom
    dpk = pk[1:] - pk[:-1]
    dbk = bk[1:] - bk[:-1]
    ck = ak[1:] * bk[:-1] - ak[:-1] * bk[1:]
    rlnp = np.zeros_like(dpk)
    alfa = np.zeros_like(dpk)
    alfa[0] = float(np.log(np.float32(2.0)))
    rlnp[1:] = np.log(pk[2:] / pk[1:-1])
    alfa[1:] = 1.0 - (pk[1:-1] / dpk[1:]) * rlnp[1:]
    cg = np.array([ug[L - 1 - k] * gx + vg[L - 1 - k] * gy for k in range(L)])  # top to bottom
    db = np.cumsum(np.array([divg[L - 1 - k] * dpk[k] for k in range(L)]), axis=0)
    cb = np.cumsum(np.array([cg[k] * dbk[k] for k in range(L)]), axis=0)
    dlnpsdt = -db[L - 1] / ps - cb[L - 1]
    etadot = np.zeros((L + 1,) + ps.shape)
    for k in range(L - 1):
        etadot[k + 1] = -ps * (bk[k + 1] * dlnpsdt + cb[k]) - db[k]
    workb = np.zeros_like(dpk)
    workc = np.zeros_like(dpk)
    workb[0] = alfa[0] * (divg[L - 1] * dpk[0] + ps * cb[0] * dbk[0])
    workc[0] = ps * cg[0] * dbk[0]
    for k in range(1, L):
        workb[k] = rlnp[k] * (db[k - 1] + ps * cb[k - 1]) + alfa[k] * (divg[L - 1 - k] * dpk[k] + ps * cg[k] * dbk[k])
        workc[k] = ps * cg[k] * (dbk[k] + ck[k] * rlnp[k] / dpk[k])
    dlnpdtg = np.array([(workc[L - 1 - b] - workb[L - 1 - b]) / dpk[L - 1 - b] for b in range(L)])  # bottom to top
    for name, want in (("dlnpsdt", dlnpsdt), ("etadot", etadot), ("dlnpdtg", dlnpdtg)):
        got = o.get_grid(name).reshape(want.shape)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max(), err_msg=name)


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


# ---- getdyntend restated in numpy (dyn_run.f90:160-305, 375-603) ----------
# Fields are numpy arrays [level][lat][lon]: 3-D grid fields bottom (0) to top,
# interface quantities (pk, etadot) and layer coefficients (dpk, dbk, rlnp,
# alfa) top (0) to bottom, as in the reference.
def _np_getvadv(q, etadot, dpk):
    L = q.shape[0]
    v = np.zeros_like(q)
    for t in range(L):  # layer t from the top is field level L - 1 - t
        acc = 0.0
        if t <= L - 2:
            acc = acc + etadot[t + 1] * (q[L - 2 - t] - q[L - 1 - t])
        if t >= 1:
            acc = acc + etadot[t] * (q[L - 1 - t] - q[L - t])
        v[L - 1 - t] = (0.5 / dpk[t]) * acc
    return v


def _np_getvadv_tracers(q, etadot, dpk):
    L = q.shape[0]
    half = np.zeros((L + 1,) + q.shape[1:])
    d = np.zeros_like(half)
    for k in range(1, L):
        half[k] = 0.5 * (q[L - 1 - k] + q[L - k])
        d[k] = q[L - 1 - k] - q[L - k]
    half[0], half[L] = q[L - 1], q[0]
    two_t = 2.0 * q[L - 1] - q[L - 2]
    d[0] = np.where(q[L - 1] >= 0, q[L - 1] - np.maximum(0.0, two_t), q[L - 1] - np.minimum(0.0, two_t))
    two_b = 2.0 * q[0] - q[1]
    d[L] = np.where(q[0] >= 0, np.maximum(0.0, two_b) - q[0], np.minimum(0.0, two_b) - q[0])
    tiny = np.finfo(np.float64).tiny
    for k in range(1, L):
        d[k] = np.where(np.abs(d[k]) < tiny, np.copysign(tiny, d[k]), d[k])
    for k in range(1, L):  # Thuburn's limiter (phi + |phi|) / (1 + |phi|), upwind by etadot
        up = etadot[k] > 0.0
        phi = np.where(up, d[k - 1], d[k + 1]) / d[k]
        qu = np.where(up, q[L - k], q[L - 1 - k])
        half[k] = qu + (phi + np.abs(phi)) / (1.0 + np.abs(phi)) * (half[k] - qu)
    v = np.zeros_like(q)
    for t in range(L):
        v[L - 1 - t] = (1.0 / dpk[t]) * ((half[t + 1] * etadot[t + 1] - half[t] * etadot[t]) +
                                         q[L - 1 - t] * (etadot[t] - etadot[t + 1]))
    return v


def _np_getpresgrad(tv, tx, ty, phx, phy, lx, ly, ps, pk, dpk, bk, dbk, rlnp, alfa, rd):
    L = tv.shape[0]
    cofb1 = [-(1.0 / dpk[0]) * (alfa[0] * dbk[0])] + \
        [-(1.0 / dpk[t]) * (bk[t] * rlnp[t] + alfa[t] * dbk[t]) for t in range(1, L)]
    cofa = [-(1.0 / dpk[t]) * (bk[t + 1] * pk[t] / pk[t + 1] - bk[t] + rlnp[t] * (bk[t] - pk[t] * dbk[t] / dpk[t]))
            for t in range(L)]
    cofb2 = [None] * L
    px3u, px3v = [None] * L, [None] * L
    cofb2[L - 1] = 0.0 * ps
    px3u[L - 1] = px3v[L - 1] = 0.0 * ps
    for k in range(1, L):  # bottom-up sums over the layers below
        cofb2[L - 1 - k] = cofb2[L - k] - rd * (bk[L + 1 - k] / pk[L + 1 - k] - bk[L - k] / pk[L - k]) * tv[k - 1]
        px3u[L - 1 - k] = px3u[L - k] - rd * rlnp[L - k] * tx[k - 1]
        px3v[L - 1 - k] = px3v[L - k] - rd * rlnp[L - k] * ty[k - 1]
    gx, gy = np.zeros_like(tv), np.zeros_like(tv)
    for t in range(L):
        b = L - 1 - t
        gx[b] = cofb1[t] * rd * tv[b] * ps * lx - phx + cofb2[t] * ps * lx + px3u[t] - rd * alfa[t] * tx[b] \
            - cofa[t] * rd * tv[b] * ps * lx
        gy[b] = cofb1[t] * rd * tv[b] * ps * ly - phy + cofb2[t] * ps * ly + px3v[t] - rd * alfa[t] * ty[b] \
            - cofa[t] * rd * tv[b] * ps * ly
    return gx, gy


def test_getdyntend_vs_numpy_restatement(oracle_mod):
    # the whole tendency computation of getdyntend (dyn_run.f90:160-305) in
    # numpy on the oracle's grid fields and transforms: getpresgrad
    # (:375-451), getvadv (:453-476), getvadv_tracers with Thuburn's limiter
    # (:478-603), the energy conversion with the humidity factor, the flux
    # form of the vorticity and divergence tendencies (getvrtdivspec of (Fu,
    # Fv) gives (ddiv, -dvrt)), the kinetic-energy Laplacian and the tracer
    # tendencies, with the reference's single-precision constants (measured
    # within 5e-16 of each field's largest value; a limiter upwinded the wrong
    # way misses the tracer tendencies by 46 %, R_d off by 1e-7 the divergence
    # tendency by 1e-8)
    T, nlon, nlat, L, nt = 42, 128, 64, 20, 2
    ak, bk = inputs.hybrid_coords(L)
    o = oracle_mod.Oracle(T, nlon, nlat, L, ak, bk, ntrac=nt, dt=1200.0)
    st = inputs.smooth_random_state(T, L, ntrac=nt, seed=8)
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=st["trc"])
    got = o.getdyntend(1)
    f32 = np.float32
    rd, cp, cvap = float(f32(287.05)), float(f32(1004.6)), float(f32(1846.0))
    kappa, omega, a = rd / cp, float(f32(7.2921e-5)), float(f32(6.3712e6))
    ug, vg, vrtg, tvg = o.get_grid("ug"), o.get_grid("vg"), o.get_grid("vrtg"), o.get_grid("tvg")
    trcg = o.get_grid("trcg").reshape(nt, L, nlat, nlon)
    dlnpdtg, dlnpsdt = o.get_grid("dlnpdtg"), o.get_grid("dlnpsdt")[0]
    etadot = o.get_grid("etadot")  # top to bottom, checked against getomega above
    phx, phy = o.get_grid("dphisdx")[0], o.get_grid("dphisdy")[0]
    ps = np.exp(o.spectogrd(st["lnps"][None])[0])
    lx, ly = (g[0] for g in o.getgrad(st["lnps"][None]))
    tx, ty = o.getgrad(st["tv"])
    pk = [ak[i] + bk[i] * ps for i in range(L + 1)]
    dpk = [pk[t + 1] - pk[t] for t in range(L)]
    dbk = bk[1:] - bk[:-1]
    rlnp = [0.0 * ps + float(f32(99999.99))] + [np.log(pk[t + 1] / pk[t]) for t in range(1, L)]
    alfa = [0.0 * ps + float(np.log(f32(2.0)))] + [1.0 - (pk[t] / dpk[t]) * rlnp[t] for t in range(1, L)]
    gx, gy = _np_getpresgrad(tvg, tx, ty, phx, phy, lx, ly, ps, pk, dpk, bk, dbk, rlnp, alfa, rd)
    vu, vv, vt = (_np_getvadv(f, etadot, dpk) for f in (ug, vg, tvg))
    vq = kappa * dlnpdtg * tvg / (1.0 + (cvap / cp - 1.0) * trcg[0])
    fcor = (2.0 * omega * np.sin(o.grid_info()["lats"]))[:, None]
    vv, vu = vv - gy, vu - gx
    dtv = o.grdtospec(-ug * tx - vg * ty - vt + vq)
    ddiv, mdvrt = o.getvrtdivspec(ug * (vrtg + fcor) + vv, vg * (vrtg + fcor) - vu)
    deg, _ = inputs.degree_order(T)
    lap = -deg * (deg + 1.0)
    ddiv = ddiv - (lap / a ** 2) * o.grdtospec(0.5 * (ug ** 2 + vg ** 2))
    dtrc = []
    for q in range(nt):
        qx, qy = o.getgrad(st["trc"][q])
        dtrc.append(o.grdtospec(-ug * qx - vg * qy - _np_getvadv_tracers(trcg[q], etadot, dpk)))
    want = dict(dvrt=-mdvrt, ddiv=ddiv, dtv=dtv, dtrc=np.array(dtrc), dlnps=o.grdtospec(dlnpsdt[None])[0])
    for k, w in want.items():
        np.testing.assert_allclose(got[k], w, rtol=0, atol=1e-12 * np.abs(w).max(), err_msg=k)


def _np_advance_dynamics(ev, st, dt, semi, damp, T):
    """One IMEX RK3 step of run.f90:194-501 (dynamics and the forward-implicit
    damping) in numpy; ev evaluates getdyntend at a spectral state."""
    f32 = np.float32
    a21, a31, a32 = float(f32(1.0) / f32(3.0)), float(f32(1.0) / f32(6.0)), float(f32(1.0) / f32(2.0))
    aa21 = aa22 = float(f32(1.0) / f32(6.0))
    aa31, aa32, aa33 = float(f32(1.0) / f32(3.0)), 0.0, float(f32(1.0) / f32(3.0))
    b1, b2, b3 = float(f32(1.0) / f32(2.0)), float(f32(-1.0) / f32(2.0)), 1.0
    bb1, bb2, bb3, bb4 = float(f32(3.0) / f32(8.0)), 0.0, float(f32(3.0) / f32(8.0)), float(f32(1.0) / f32(4.0))
    A, B, sv, tor, D = semi["amhyb"], semi["bmhyb"], semi["svhyb"], semi["tor_hyb"], semi["d_hyb_m"]
    deg, _ = inputs.degree_order(T)
    lap = -deg * (deg + 1.0)
    o = {k: st[k].copy() for k in ("vrt", "div", "tv", "lnps", "trc")}

    def tend(s, stage):
        ev.set_state(s["vrt"], s["div"], s["tv"], s["lnps"], trc=s["trc"] if s["trc"].size else None)
        return ev.getdyntend(stage)

    def lin(s):  # the linear terms the semi-implicit scheme treats implicitly
        return dict(ddiv=-lap * (A @ s["tv"] + tor[:, None] * s["lnps"][None, :]), dtv=-(B @ s["div"]),
                    dlnps=-(sv @ s["div"]))

    def solve(s, c, mats):  # implicit part for the updated divergence, back-substitution
        rhs = s["div"] - c * lap * dt * (A @ s["tv"] + tor[:, None] * s["lnps"][None, :])
        div = np.einsum("nkj,jn->kn", mats[deg], rhs)
        s["div"] = div
        s["tv"] = s["tv"] - c * dt * (B @ div)
        s["lnps"] = s["lnps"] - c * dt * (sv @ div)

    keys = (("ddiv", "div"), ("dtv", "tv"), ("dlnps", "lnps"))
    t0 = tend(o, 1)
    l0 = lin(o)
    for k, _ in keys:
        t0[k] = t0[k] - l0[k]
    s = {"vrt": o["vrt"] + a21 * dt * t0["dvrt"], "trc": o["trc"] + a21 * dt * t0["dtrc"]}
    for k, f in keys:
        s[f] = o[f] + dt * (a21 * t0[k] + aa21 * l0[k])
    solve(s, aa22, D[0])
    t1 = tend(s, 2)
    l1 = lin(s)
    for k, _ in keys:
        t1[k] = t1[k] - l1[k]
    s2 = {"vrt": o["vrt"] + dt * (a31 * t0["dvrt"] + a32 * t1["dvrt"]),
          "trc": o["trc"] + dt * (a31 * t0["dtrc"] + a32 * t1["dtrc"])}
    for k, f in keys:
        s2[f] = o[f] + dt * (a31 * t0[k] + aa31 * l0[k] + a32 * t1[k] + aa32 * l1[k])
    solve(s2, aa33, D[1])
    t2 = tend(s2, 3)
    l2 = lin(s2)
    for k, _ in keys:
        t2[k] = t2[k] - l2[k]
    s3 = {"vrt": o["vrt"] + dt * (b1 * t0["dvrt"] + b2 * t1["dvrt"] + b3 * t2["dvrt"]),
          "trc": o["trc"] + dt * (b1 * t0["dtrc"] + b2 * t1["dtrc"] + b3 * t2["dtrc"])}
    for k, f in keys:
        s3[f] = o[f] + dt * (b1 * t0[k] + bb1 * l0[k] + b2 * t1[k] + bb2 * l1[k] + b3 * t2[k] + bb3 * l2[k])
    solve(s3, bb4, D[2])
    dis, dp, mp = damp["disspec"], damp["diff_prof"], damp["dmp_prof"]
    fvd = 1.0 - (dis[None, :] * dp[:, None] - mp[:, None]) * dt
    ftq = 1.0 - dis[None, :] * dp[:, None] * dt
    s3["vrt"], s3["div"], s3["tv"] = s3["vrt"] / fvd, s3["div"] / fvd, s3["tv"] / ftq
    s3["trc"] = s3["trc"] / ftq[None]
    return s3


def test_advance_vs_numpy_restatement(oracle_mod):
    # one adiabatic step of advance (run.f90:194-501): the explicit and
    # implicit tableaux of the IMEX RK3 scheme (semimp_data.f90:74-88), the
    # linear terms taken out of each stage's tendencies, the per-degree solve
    # against d_hyb_m with back-substitution, and the forward-implicit
    # damping, in numpy on the oracle's getdyntend and matrices; 64 levels,
    # so that the sponge (dmp_prof, above sigma = 0.002) acts (measured within
    # 2e-15 of each field's largest value; the stage-2 inverse in stage 1 or
    # the sponge's sign flipped miss by 4e-3 and 8e-3)
    T, nlon, nlat, L, nt, dt = 42, 128, 64, 64, 2, 1200.0
    ak, bk = inputs.hybrid_coords(L)
    kw = dict(ntrac=nt, dt=dt, adiabatic=True, heldsuarez=False)
    o = oracle_mod.Oracle(T, nlon, nlat, L, ak, bk, **kw)
    ev = oracle_mod.Oracle(T, nlon, nlat, L, ak, bk, **kw)
    st = inputs.smooth_random_state(T, L, ntrac=nt, seed=11)
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=st["trc"])
    o.advance(1)
    got = o.get_state()
    want = _np_advance_dynamics(ev, st, dt, o.semimp(), o.damp(), T)
    for k in ("vrt", "div", "tv", "lnps", "trc"):
        np.testing.assert_allclose(got[k], want[k], rtol=0, atol=1e-12 * np.abs(want[k]).max(), err_msg=k)


def test_advance_with_forcing_vs_numpy_restatement(oracle_mod):
    # one Held-Suarez step: the dynamics as above, then the time-split physics
    # (run.f90:509-538: the grid updated by an inverse-only pass, getphytend
    # applied over dt) and the dry-mass fixer (dyn_run.f90:605-634: ps scaled
    # by pcorr = pdryini / sum(areawts ps), its log analysed, the ln ps
    # tendency (ws - lnps) / dt applied); measured within 2e-15 of each field's
    # largest value
    T, nlon, nlat, L, nt, dt = 42, 128, 64, 20, 1, 1200.0
    ak, bk = inputs.hybrid_coords(L)
    kw = dict(ntrac=nt, dt=dt)
    o = oracle_mod.Oracle(T, nlon, nlat, L, ak, bk, **kw)
    ev = oracle_mod.Oracle(T, nlon, nlat, L, ak, bk, **kw)
    st = inputs.smooth_random_state(T, L, ntrac=nt, seed=12)
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=st["trc"])
    o.advance(1)
    got = o.get_state()
    pdryini = o.diag()["pdryini"]
    s = _np_advance_dynamics(ev, st, dt, o.semimp(), o.damp(), T)
    ev.set_state(s["vrt"], s["div"], s["tv"], s["lnps"], trc=s["trc"])
    ev.getdyntend(3, inverse_only=True)
    ph = ev.getphytend()
    s["vrt"] = s["vrt"] + dt * ph["dvrt"]
    s["div"] = s["div"] + dt * ph["ddiv"]
    s["tv"] = s["tv"] + dt * ph["dtv"]
    s["trc"] = s["trc"] + dt * ph["dtrc"]
    psg = ev.get_grid("psg")[0]
    aw = ev.grid_info()["areawts"]
    pcorr = pdryini / (aw[:, None] * psg).sum()
    ws = ev.grdtospec(np.log(psg * pcorr)[None])[0]
    s["lnps"] = s["lnps"] + dt * ((ws - s["lnps"]) / dt)
    for k in ("vrt", "div", "tv", "lnps", "trc"):
        np.testing.assert_allclose(got[k], s[k], rtol=0, atol=1e-12 * np.abs(s[k]).max(), err_msg=k)
