"""Pins the FP64 CPU oracle's transforms (the role SHTns plays for
src/shtns.f90) against scipy / numpy and analytic known answers.

The reference ships no golden vectors for this path; these known-answer
tests fix the convention of src/shtns.f90:110 (orthonormal, no
Condon-Shortley phase) and the physical contract of getuv / getvrtdivspec /
getgrad (src/shtns.f90:233-352).
"""
import numpy as np
import pytest
from scipy.special import gammaln, lpmv, roots_legendre

from gdpy import inputs
from sht_numpy import ShtNumpy

A = inputs.RERTH


def make(oracle_mod, T=21, nlon=64, nlat=32, nlev=2):
    ak, bk = inputs.hybrid_coords(nlev)
    return oracle_mod.Oracle(T, nlon, nlat, nlev, ak, bk, dt=1200.0)


def rand_spec(T, nb, seed=1):
    rng = np.random.default_rng(seed)
    deg, order = inputs.degree_order(T)
    a = rng.standard_normal((nb, deg.size)) + 1j * rng.standard_normal((nb, deg.size))
    a[:, order == 0] = a[:, order == 0].real
    return a


@pytest.mark.parametrize("nlat,nlon", [(32, 64), (64, 128), (190, 384), (576, 1152)])
def test_gauss_nodes_weights_vs_scipy(oracle_mod, nlat, nlon):
    o = make(oracle_mod, T=21, nlon=nlon, nlat=nlat)
    gi = o.grid_info()
    x, w = roots_legendre(nlat)
    np.testing.assert_allclose(np.sin(gi["lats"]), x[::-1], rtol=0, atol=2e-15)
    # scipy's polar weights carry up to ~2e-9 relative error at n = 576 (its
    # n > 150 branch is asymptotic); the oracle's are checked against
    # mpmath below and are ~1e-11 or better.
    np.testing.assert_allclose(gi["gauwts"], w[::-1], rtol=5e-9 if nlat > 150 else 2e-12)
    np.testing.assert_allclose(gi["gauwts"].sum(), 2.0, rtol=1e-14)
    np.testing.assert_allclose(gi["areawts"].sum() * o.nlon, 1.0, rtol=1e-14)


@pytest.mark.parametrize("N,nlon,tol", [(32, 64, 1e-13), (576, 1152, 2e-11)])
def test_polar_gauss_weight_vs_mpmath(oracle_mod, N, nlon, tol):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 50
    o = make(oracle_mod, T=21, nlon=nlon, nlat=N)
    gi = o.grid_info()

    def pn(t):
        p0, p1 = mp.mpf(1), t
        for k in range(1, N):
            p0, p1 = p1, ((2 * k + 1) * t * p1 - k * p0) / (k + 1)
        return p0, p1

    for j in (0, 1, 5):
        r = mp.mpf(np.sin(gi["lats"][j]))
        for _ in range(8):
            pm1, p = pn(r)
            r = r - p / (N * (r * p - pm1) / (r * r - 1))
        pm1, p = pn(r)
        dp = N * (r * p - pm1) / (r * r - 1)
        wr = float(2 / ((1 - r ** 2) * dp ** 2))
        assert abs(gi["gauwts"][j] - wr) / wr < tol
        assert abs(float(np.sin(gi["lats"][j]) - r)) < 1e-16


def test_legendre_tables_vs_scipy(oracle_mod):
    T, nlat = 42, 64
    o = make(oracle_mod, T=T, nlon=128, nlat=nlat)
    mu = np.sin(o.grid_info()["lats"][: nlat // 2])
    for m in [0, 1, 2, 7, 20, 42]:
        P, H = o.legendre(m)
        for n in range(m, T + 1):
            norm = np.sqrt((2 * n + 1) / (4 * np.pi) * np.exp(gammaln(n - m + 1) - gammaln(n + m + 1)))
            ref = norm * (-1.0) ** m * lpmv(m, n, mu)
            np.testing.assert_allclose(P[:, n - m], ref, rtol=1e-10, atol=1e-13)


@pytest.mark.parametrize("m", [0, 1, 37, 300, 573, 574])
def test_legendre_tables_t574_vs_mpmath(oracle_mod, m):
    # the headline truncation, where scipy's lpmv cannot follow the high orders:
    # the orthonormal functions (no Condon-Shortley phase) by the same
    # three-term recurrence carried out in 60-digit arithmetic, at latitudes
    # from the pole row to the equator row; the oracle's FP64 values within
    # 1e-12 of each order's largest value (measured 2e-15 at m = 0, 1.3e-14
    # at m = 574; a Condon-Shortley phase would miss odd orders by 2).  The
    # derivative table dP/dphi against cos(phi) dP/dmu = ((n+1) eps_n P_{n-1}
    # - n eps_{n+1} P_{n+1}) / cos(phi), eps_n = sqrt((n^2 - m^2) / (4 n^2 - 1))
    # (measured at most 2.7e-13, at the row next to the pole for m = 0)
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 60
    T, nlat = 574, 576
    o = make(oracle_mod, T=T, nlon=1152, nlat=nlat)
    mus = np.sin(o.grid_info()["lats"][: nlat // 2])
    P, H = o.legendre(m)
    rows = [0, 1, 2, 40, 144, 250, nlat // 2 - 1]
    ref = np.zeros((len(rows), T - m + 1))
    refh = np.zeros_like(ref)
    eps = lambda n: mp.sqrt(mp.mpf(n * n - m * m) / (4 * n * n - 1))
    for a, j in enumerate(rows):
        mu = mp.mpf(float(mus[j]))
        s2 = 1 - mu * mu
        # P_m^m = sqrt((2m+1) / (4 pi (2m)!)) (2m-1)!! (1 - mu^2)^(m/2)
        pmm = mp.sqrt((2 * m + 1) / (4 * mp.pi * mp.factorial(2 * m))) * mp.fac2(2 * m - 1) * s2 ** (mp.mpf(m) / 2)
        pv = {m: pmm}
        p0, p1 = None, pmm
        for n in range(m + 1, T + 2):  # one degree past T for the derivative identity
            an = mp.sqrt(mp.mpf(4 * n * n - 1) / (n * n - m * m))
            bn = mp.sqrt(mp.mpf((n - 1) ** 2 - m * m) / (4 * (n - 1) ** 2 - 1)) if n > m + 1 else mp.mpf(0)
            p2 = an * (mu * p1 - (bn * p0 if p0 is not None else 0))
            p0, p1 = p1, p2
            pv[n] = p2
        for n in range(m, T + 1):
            ref[a, n - m] = float(pv[n])
            pm1 = pv[n - 1] if n - 1 >= m else 0
            refh[a, n - m] = float(((n + 1) * eps(n) * pm1 - n * eps(n + 1) * pv[n + 1]) / mp.sqrt(s2))
    for got, want in ((P[rows, :], ref), (H[rows, :], refh)):
        scale = np.abs(want).max()
        assert scale > 0
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * scale)


def test_t574_transforms_vs_numpy_fft(oracle_mod):
    # the oracle's full T574 scalar transforms (Legendre sums over its tables,
    # which the test above pins, and its own longitude FFTs) against numpy's
    # FFT over the same tables, order by order: synthesis g = F_0 + 2 Re sum
    # F_m e^{i m lambda}, analysis a_nm = sum_j 2 pi w_j P_nm(mu_j) F_m(mu_j)
    # (measured 9.9e-16 and 6.1e-16 of the largest value, round trip 2.5e-14)
    T, nlon, nlat = 574, 1152, 576
    o = make(oracle_mod, T=T, nlon=nlon, nlat=nlat)
    gi = o.grid_info()
    W = 2 * np.pi * gi["gauwts"]
    deg, order = inputs.degree_order(T)
    rng = np.random.default_rng(7)
    a = (rng.standard_normal(deg.size) + 1j * rng.standard_normal(deg.size)) / (1.0 + deg)
    a[order == 0] = a[order == 0].real
    g = o.spectogrd(a[None, :])[0]
    F = np.zeros((nlon // 2 + 1, nlat), np.complex128)
    off = 0
    half = nlat // 2
    for m in range(T + 1):
        P, _ = o.legendre(m)  # northern rows x degrees n = m .. T
        cnt = T - m + 1
        am = a[off:off + cnt]
        sgn = (-1.0) ** np.arange(cnt)  # P(-mu) = (-1)^(n-m) P(mu)
        F[m, :half] = P @ am
        F[m, half:] = ((P * sgn) @ am)[::-1]
        off += cnt
    gn = nlon * np.fft.irfft(F, n=nlon, axis=0).T  # [lat][lon]
    scale = np.abs(gn).max()
    np.testing.assert_allclose(g.reshape(nlat, nlon), gn, rtol=0, atol=1e-12 * scale)
    # analysis of the same grid
    b = o.grdtospec(gn[None])[0]
    Fg = np.fft.rfft(gn, axis=1).T / nlon  # [m][lat]
    bn = np.zeros_like(a)
    off = 0
    for m in range(T + 1):
        P, _ = o.legendre(m)
        cnt = T - m + 1
        sgn = (-1.0) ** np.arange(cnt)
        bn[off:off + cnt] = (P.T * W[:half]) @ Fg[m, :half] + ((P * sgn).T * W[half:][::-1]) @ Fg[m, half:][::-1]
        off += cnt
    np.testing.assert_allclose(b, bn, rtol=0, atol=1e-12 * np.abs(bn).max())
    np.testing.assert_allclose(bn, a, rtol=0, atol=1e-11 * np.abs(a).max())  # the round trip


def test_t574_vector_transforms_vs_numpy_fft(oracle_mod):
    # getuv and getvrtdivspec at T574 against the formulas of sht_numpy (U =
    # -H s + (i m / cos) P c, V = (i m / cos) P s + H c with s, c = a invlap
    # (vrt, div); vrt = (P (i m / cos) V + H U) / a, div = (P (i m / cos) U - H V)
    # / a under the quadrature) over the oracle's pinned tables, P mirrored
    # with (-1)^(n-m) and H = dP/dphi with the opposite sign, and numpy's FFT
    # (measured 2.4e-13 and 4.2e-14 of the largest value; the FP64 round trip
    # itself loses to 4e-12 at T574)
    T, nlon, nlat = 574, 1152, 576
    o = make(oracle_mod, T=T, nlon=nlon, nlat=nlat)
    gi = o.grid_info()
    W = 2 * np.pi * gi["gauwts"]
    cs = np.cos(gi["lats"])
    deg, order = inputs.degree_order(T)
    rng = np.random.default_rng(9)

    def rs():
        x = (rng.standard_normal(deg.size) + 1j * rng.standard_normal(deg.size)) / (1.0 + deg) ** 2
        x[order == 0] = x[order == 0].real
        x[0] = 0
        return x

    vrt, div = rs(), rs()
    il = np.zeros(deg.size)
    il[1:] = -1.0 / (deg[1:] * (deg[1:] + 1.0))
    s, c = A * il * vrt, A * il * div
    U = np.zeros((nlon // 2 + 1, nlat), complex)
    V = np.zeros_like(U)
    tabs = []
    off = 0
    for m in range(T + 1):
        P, H = o.legendre(m)
        cnt = T - m + 1
        sg = (-1.0) ** np.arange(cnt)
        Pf, Hf = np.vstack([P, (P * sg)[::-1]]), np.vstack([H, (-H * sg)[::-1]])
        tabs.append((Pf, Hf))
        imc = 1j * m / cs
        sm, cm = s[off:off + cnt], c[off:off + cnt]
        U[m] = -Hf @ sm + imc * (Pf @ cm)
        V[m] = imc * (Pf @ sm) + Hf @ cm
        off += cnt
    un = nlon * np.fft.irfft(U, n=nlon, axis=0).T
    vn = nlon * np.fft.irfft(V, n=nlon, axis=0).T
    u, v = o.getuv(vrt[None], div[None])
    np.testing.assert_allclose(u[0], un, rtol=0, atol=1e-12 * np.abs(un).max())
    np.testing.assert_allclose(v[0], vn, rtol=0, atol=1e-12 * np.abs(vn).max())
    Ug, Vg = np.fft.rfft(un, axis=1).T / nlon, np.fft.rfft(vn, axis=1).T / nlon
    vr, dv = np.zeros_like(vrt), np.zeros_like(div)
    off = 0
    for m in range(T + 1):
        Pf, Hf = tabs[m]
        cnt = T - m + 1
        imc = 1j * m / cs
        vr[off:off + cnt] = ((Pf.T * W) @ (imc * Vg[m]) + (Hf.T * W) @ Ug[m]) / A
        dv[off:off + cnt] = ((Pf.T * W) @ (imc * Ug[m]) - (Hf.T * W) @ Vg[m]) / A
        off += cnt
    v2, d2 = o.getvrtdivspec(un[None], vn[None])
    np.testing.assert_allclose(v2[0], vr, rtol=0, atol=1e-12 * np.abs(vr).max())
    np.testing.assert_allclose(d2[0], dv, rtol=0, atol=1e-12 * np.abs(dv).max())
    np.testing.assert_allclose(vr, vrt, rtol=0, atol=2e-11 * np.abs(vrt).max())


def test_orthonormality_under_gauss_quadrature(oracle_mod):
    T, nlat = 42, 64
    o = make(oracle_mod, T=T, nlon=128, nlat=nlat)
    w = o.grid_info()["gauwts"][: nlat // 2]
    for m in [0, 3, 17, 42]:
        P, _ = o.legendre(m)
        # both hemispheres: parity (-1)^(n-m)
        n = np.arange(m, T + 1)
        sgn = (-1.0) ** (n - m)
        G = 2 * np.pi * (P.T * w) @ P + 2 * np.pi * ((P * sgn).T * w) @ (P * sgn)
        np.testing.assert_allclose(G, np.eye(T - m + 1), atol=1e-13)


@pytest.mark.parametrize("T,nlon,nlat", [(21, 64, 32), (42, 128, 64), (62, 192, 94)])
def test_round_trip(oracle_mod, T, nlon, nlat):
    o = make(oracle_mod, T=T, nlon=nlon, nlat=nlat)
    a = rand_spec(T, 3)
    g = o.spectogrd(a)
    b = o.grdtospec(g)
    np.testing.assert_allclose(b, a, atol=1e-12 * np.abs(a).max())
    vrt, div = rand_spec(T, 2, 5), rand_spec(T, 2, 6)
    vrt[:, 0] = 0
    div[:, 0] = 0
    u, v = o.getuv(vrt, div)
    vrt2, div2 = o.getvrtdivspec(u, v)
    np.testing.assert_allclose(vrt2, vrt, atol=1e-12 * np.abs(vrt).max())
    np.testing.assert_allclose(div2, div, atol=1e-12 * np.abs(div).max())


def test_cpp_oracle_matches_numpy_oracle(oracle_mod):
    T, nlon, nlat = 21, 64, 32
    o = make(oracle_mod, T=T, nlon=nlon, nlat=nlat)
    s = ShtNumpy(T, nlon, nlat, A)
    a, b = rand_spec(T, 1, 11)[0], rand_spec(T, 1, 12)[0]
    g = o.spectogrd(a)[0]
    np.testing.assert_allclose(g, s.spectogrd(a), atol=1e-12 * np.abs(g).max())
    np.testing.assert_allclose(o.grdtospec(g)[0], s.grdtospec(g), atol=1e-12 * np.abs(a).max())
    u, v = o.getuv(a, b)
    us, vs = s.getuv(a, b)
    np.testing.assert_allclose(u[0], us, atol=1e-12 * np.abs(us).max())
    np.testing.assert_allclose(v[0], vs, atol=1e-12 * np.abs(vs).max())
    gx, gy = o.getgrad(a)
    gxs, gys = s.getgrad(a)
    np.testing.assert_allclose(gx[0], gxs, atol=1e-12 * np.abs(gxs).max())
    np.testing.assert_allclose(gy[0], gys, atol=1e-12 * np.abs(gys).max())
    rng = np.random.default_rng(3)
    ug, vg = rng.standard_normal((nlat, nlon)), rng.standard_normal((nlat, nlon))
    vr, dv = o.getvrtdivspec(ug, vg)
    vrs, dvs = s.getvrtdivspec(ug, vg)
    np.testing.assert_allclose(vr[0], vrs, atol=1e-12 * np.abs(vrs).max())
    np.testing.assert_allclose(dv[0], dvs, atol=1e-12 * np.abs(dvs).max())


def test_solid_body_rotation_and_gradients(oracle_mod):
    T, nlon, nlat = 21, 64, 32
    o = make(oracle_mod, T=T, nlon=nlon, nlat=nlat)
    gi = o.grid_info()
    phi = gi["lats"][:, None] * np.ones(nlon)
    lam = 2 * np.pi * np.arange(nlon)[None, :] / nlon * np.ones((nlat, 1))
    U0 = 20.0
    # u = U0 cos(phi), v = 0  <=>  vrt = 2 U0 sin(phi) / a, i.e. n=1,m=0 coefficient
    vrt = np.zeros(o.nlm, np.complex128)
    vrt[1] = 2 * U0 / A * np.sqrt(4 * np.pi / 3)
    u, v = o.getuv(vrt, np.zeros_like(vrt))
    np.testing.assert_allclose(u[0], U0 * np.cos(phi), atol=1e-12 * U0)
    np.testing.assert_allclose(v[0], 0.0, atol=1e-12 * U0)
    vr, dv = o.getvrtdivspec(U0 * np.cos(phi), 0 * phi)
    np.testing.assert_allclose(vr[0], vrt, atol=1e-13 * abs(vrt[1]))
    np.testing.assert_allclose(dv[0], 0, atol=1e-13 * abs(vrt[1]))
    # f = cos(phi) cos(lambda): grad = (-sin(lambda)/a, -sin(phi) cos(lambda)/a)
    f = np.cos(phi) * np.cos(lam)
    fs = o.grdtospec(f)[0]
    gx, gy = o.getgrad(fs)
    np.testing.assert_allclose(gx[0], -np.sin(lam) / A, atol=1e-12 / A)
    np.testing.assert_allclose(gy[0], -np.sin(phi) * np.cos(lam) / A, atol=1e-12 / A)
    # no Condon-Shortley phase: Y_1^1 coefficient of cos(phi)cos(lambda) is positive
    k11 = T + 1  # m=1, n=1
    assert fs[k11].real > 0
    # Laplacian eigenvalues (lap = -n(n+1))
    np.testing.assert_array_equal(gi["lap"], -gi["degree"] * (gi["degree"] + 1.0))
