"""DCMIP-2012 initial states -- TEST INFRASTRUCTURE ONLY.

A numpy restatement, vectorised over points, of the analytic initial states
the reference evaluates in src/dcmip_initial_conditions_test_4_v3.f90
(moist baroclinic instability) and src/dcmip_initial_conditions_test_5_v1.f90
(tropical cyclone), and of the dcmip_ics driver (src/dyn_init.f90:330-416)
on top of the FP64 oracle's transforms.  Only tests use it, to check the
library's host evaluation (gd_dcmip_point) and its gd_dcmip_ics state.
"""
import numpy as np

PI = 4.0 * np.arctan(1.0)
A, RD, G, OMEGA = 6371220.0, 287.0, 9.80616, 7.29212e-5


def _lat_polys(lat):
    s, c = np.sin(lat), np.cos(lat)
    return -2.0 * s ** 6 * (c ** 2 + 1.0 / 3.0) + 10.0 / 63.0, 8.0 / 5.0 * c ** 3 * (s ** 2 + 2.0 / 3.0) - PI / 4.0


def test4(lon, lat, p, moist=True):
    """(u, v, T, phis, ps, q, q1, q2) of the baroclinic wave at pressure p."""
    p0, kappa, eta_t, u0, T0, eta0 = 1.0e5, 2.0 / 7.0, 0.2, 35.0, 288.0, 0.252
    radius, amp = 10.0, 1.0
    plon, plat = np.deg2rad(20.0), np.deg2rad(40.0)
    dT, gam = 480000.0, 0.005
    aom, expo = A * OMEGA, RD * gam / G
    lon, lat, p = np.broadcast_arrays(np.asarray(lon, float), np.asarray(lat, float), np.asarray(p, float))
    eta = p / p0
    P1, P2 = _lat_polys(lat)
    tmean = T0 * eta ** expo + np.where(eta < eta_t, dT * (eta_t - np.minimum(eta, eta_t)) ** 5, 0.0)
    phv = (eta - eta0) * 0.5 * PI
    tdev = eta * PI * u0 / RD * 1.5 * np.sin(phv) * np.cos(phv) ** 0.5 * (
        P1 * u0 * np.cos(phv) ** 1.5 + P2 * aom * 0.5)
    t = tmean + tdev
    ct_s = u0 * np.cos((1.0 - eta0) * PI * 0.5) ** 1.5
    phis = (P1 * ct_s + P2 * aom) * ct_s
    K = np.sin(plat) * np.sin(lat) + np.cos(plat) * np.cos(lat) * np.cos(lon - plon)
    r = np.arccos(K)
    u = amp * np.exp(-(r * radius) ** 2) + np.cos(phv) ** 1.5 * 4.0 * u0 * np.sin(lat) ** 2 * np.cos(lat) ** 2
    if moist:
        q = 0.021 * np.exp(-(lat / (2.0 * PI / 9.0)) ** 4) * np.exp(-((eta - 1.0) * p0 / 34000.0) ** 2)
        t = t / (1.0 + 0.608 * q)
    else:
        q = np.zeros_like(t)
    enu = phv
    ct = u0 * np.cos(enu) ** 1.5
    Y = P1 * 2.0 * ct + P2 * aom
    q1 = tmean * eta ** (-kappa) + 0.75 * PI * u0 / RD * eta ** (1 - kappa) * np.sin(enu) * np.sqrt(np.cos(enu)) * Y
    # Ertel PV (the centre, antipode and pole cases of the reference)
    s, c = np.sin(lat), np.cos(lat)
    DK = np.sin(plat) * c - np.cos(plat) * s * np.cos(lon - plon)
    zbg = -4.0 / A * ct * s * c * (2.0 - 5.0 * s ** 2)
    eps = 1e-6
    centre = (np.abs(lat - plat) <= eps) & (np.abs(lon - plon) <= eps)
    special = ((np.abs(lat + plat) <= eps) & (np.abs(lon - (plon + PI)) <= eps)) | (np.abs(lat - PI / 2) <= eps) | (
        np.abs(lat + PI / 2) <= eps)
    with np.errstate(divide="ignore", invalid="ignore"):
        general = zbg + amp / A * np.exp(-(r * radius) ** 2) * (np.tan(lat) - 2.0 * radius ** 2 * r * DK / np.sqrt(1.0 - K ** 2))
    zeta = np.where(centre, zbg + amp / A * np.tan(lat), np.where(special, zbg, general))
    dudeta = -u0 * np.sin(2.0 * lat) ** 2 * 3.0 * PI / 4.0 * np.sqrt(np.cos(enu)) * np.sin(enu)
    dmt = T0 * (expo - kappa) * eta ** (expo - kappa - 1.0)
    dmt = dmt - np.where(eta < eta_t, dT * (5.0 * (eta_t - eta) ** 4 * eta ** (-kappa)
                                            + kappa * (eta_t - eta) ** 5 * eta ** (-kappa - 1.0)), 0.0)
    e1k = eta ** (1.0 - kappa)
    dthde = (dmt + 0.75 * PI * u0 / RD * (1 - kappa) * eta ** (-kappa) * np.sin(enu) * np.sqrt(np.cos(enu)) * Y
             + 3.0 / 8.0 * PI * PI / RD * e1k * ct * Y
             - 3.0 / 16.0 * PI * PI * u0 / RD * e1k * np.sin(enu) ** 2 * np.cos(enu) ** (-0.5) * Y
             - 9.0 / 8.0 * PI * PI * u0 * u0 / RD * e1k * np.sin(enu) ** 2 * np.cos(enu) * P1)
    d1 = 2.0 * ct * (-12.0 * c * s ** 5 * (c ** 2 + 1.0 / 3.0) + 4.0 * c * s ** 7)
    d2 = aom * (-24.0 / 5.0 * s * c ** 2 * (s ** 2 + 2.0 / 3.0) + 16.0 / 5.0 * c ** 4 * s)
    dthdphi = 0.75 * PI * u0 / RD * e1k * np.sin(enu) * np.sqrt(np.cos(enu)) * (d1 + d2)
    q2 = np.abs(G / p0 * (-dudeta * dthdphi / A - (zeta + 2.0 * OMEGA * s) * dthde))
    return u, np.zeros_like(u), t, phis, np.full_like(u, p0), q, q1, q2


def test5(lon, lat, p):
    """(u, v, T, phis, ps, q) of the tropical cyclone at pressure p."""
    omega, deg = 7.292115e-5, 180.0 / PI
    rp, dp, zp, q0, gam, Ts0, p00 = 282000.0, 1115.0, 7000.0, 0.021, 0.007, 302.15, 101500.0
    clat, clon, zq1, zq2, eppr, eppz = 10.0, 180.0, 3000.0, 8000.0, 1.5, 2.0
    ztrop, qtrop, rfpi, ctv = 15000.0, 1e-11, 1.0e6, 0.608
    expo = RD * gam / G
    T0 = Ts0 * (1.0 + ctv * q0)
    lon, lat, p = np.broadcast_arrays(np.asarray(lon, float), np.asarray(lat, float), np.asarray(p, float))
    f = 2.0 * omega * np.sin(clat / deg)
    gr = A * np.arccos(np.sin(clat / deg) * np.sin(lat) + np.cos(clat / deg) * np.cos(lat) * np.cos(lon - clon / deg))
    ps = p00 - dp * np.exp(-(gr / rp) ** eppr)
    h = (T0 / gam) * (1.0 - (p / ps) ** expo)
    gk = G / (RD * gam)

    def F(z):
        return p - (p00 - dp * np.exp(-(gr / rp) ** eppr) * np.exp(-(z / zp) ** eppz)) * ((T0 - gam * z) / T0) ** gk

    def dF(z):
        e = np.exp(-(gr / rp) ** eppr) * np.exp(-(z / zp) ** eppz)
        return (-eppz * z * dp * e / (zp * zp) * ((T0 - gam * z) / T0) ** gk
                + G / (RD * T0) * (p00 - dp * e) * ((T0 - gam * z) / T0) ** (gk - 1.0))

    z = h.copy()
    active = gr < rfpi
    zn = z.copy()
    for n in range(2, 21 + 1):  # the reference's iteration count and stopping rule
        znew = z - F(z) / dF(z)
        zn = np.where(active, znew, zn)
        stop = (n > 20) | ~(np.abs(znew - z) / np.abs(znew) > 1e-11)
        z = np.where(active & ~stop, znew, z)
        active = active & ~stop
        if not active.any():
            break
    h = np.where(gr < rfpi, zn, h)
    d1 = np.sin(clat / deg) * np.cos(lat) - np.cos(clat / deg) * np.sin(lat) * np.cos(lon - clon / deg)
    d2 = np.cos(clat / deg) * np.sin(lon - clon / deg)
    d = np.maximum(1e-25, np.sqrt(d1 ** 2 + d2 ** 2))
    er, ez = np.exp((gr / rp) ** eppr), np.exp((h / zp) ** eppz)
    vt = -f * gr / 2 + np.sqrt((f * gr / 2) ** 2 - eppr * (gr / rp) ** eppr * RD * (T0 - gam * h)
                               / (eppz * h * RD * (T0 - gam * h) / (G * zp ** eppz) + (1 - p00 / dp * er * ez)))
    trop = h > ztrop
    q = np.where(trop, qtrop, q0 * np.exp(-h / zq1) * np.exp(-(h / zq2) ** eppz))
    t = (T0 - gam * h) / (1 + ctv * q) / (1 + eppz * RD * (T0 - gam * h) * h / (G * zp ** eppz * (1 - p00 / dp * er * ez)))
    t = np.where(trop, T0 - gam * ztrop, t)
    u = np.where(trop, 0.0, d1 / d * vt)
    v = np.where(trop, 0.0, d2 / d * vt)
    return u, v, t, np.zeros_like(u), ps, q


def layer_pressure(ak, bk, ps, kappa):
    """prs of calc_pressdata, [L][...] bottom to top."""
    pk = ak[:, None] + bk[:, None] * ps.ravel()[None, :]
    pu, pl = pk[:-1], pk[1:]
    prs = ((pl ** kappa * pl - pu ** kappa * pu) / ((kappa + 1.0) * (pl - pu))) ** (1.0 / kappa)
    return prs[::-1].reshape((len(ak) - 1,) + ps.shape)


def ics(oracle, testcase, ak, bk, ntrac, dry, fvirt, kappa, grav):
    """dcmip_ics on an oracle_py.Oracle: the spectral state (vrt, div, tv, trc, lnps, topo)."""
    info = oracle.grid_info()
    nlat, nlon = oracle.nlat, oracle.nlon
    lat = np.repeat(info["lats"][:, None], nlon, axis=1)
    lon = np.repeat((2 * PI * np.arange(nlon) / nlon)[None, :], nlat, axis=0)
    tc = testcase // 10
    if tc == 4:
        ps = np.full((nlat, nlon), 1.0e5)
    else:
        ps0 = np.exp(np.full((nlat, nlon), np.log(1.015e5)))
        ps = test5(lon, lat, layer_pressure(ak, bk, ps0, kappa)[0])[4]
    lnpsg = np.log(ps)
    prs = layer_pressure(ak, bk, np.exp(lnpsg), kappa)
    L = len(ak) - 1
    if tc == 4:
        u, v, t, phis, _, q, q1, q2 = test4(lon[None], lat[None], prs, moist=not dry)
    else:
        u, v, t, phis, _, q = test5(lon[None], lat[None], prs)
    tv = t if dry else t * (1 + fvirt * q)
    trc = np.zeros((ntrac, L, nlat, nlon))
    if not dry:
        trc[0] = q
    if tc == 4:
        trc[1], trc[2] = q1, q2
    vrt, div = oracle.getvrtdivspec(u, v)
    return dict(vrt=vrt, div=div, tv=oracle.grdtospec(tv), trc=oracle.grdtospec(trc.reshape(-1, nlat, nlon)).reshape(
        ntrac, L, -1), lnps=oracle.grdtospec(lnpsg)[0], topo=oracle.grdtospec(phis[0] / grav)[0])
