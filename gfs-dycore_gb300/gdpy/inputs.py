"""Synthetic inputs for the GFS spectral dycore step.

The reference takes its hybrid coordinate (ak, bk) and its initial state
from a sigma file header and body (src/dyn_init.f90:45-61); those files are
not distributed with jswhit/gfs-dycore, so every configuration here is
seeded and generated:

* ``hybrid_coords``: a documented L-level hybrid sigma-pressure set with the
  model top at p = 0 (the reference's calc_pressdata special-cases the top
  layer, src/pressure_data.f90:87-89, which presumes pk(1) = 0).
* ``hs_rest_state``: isothermal 300 K at rest, ps = 1000 hPa, plus seeded
  Gaussian vorticity noise in total wavenumbers 1..20 (grid RMS 1e-6 1/s).
* ``smooth_random_state``: vorticity, divergence, temperature, ln(ps) and
  passive tracers with seeded spectral amplitudes ~ n**-2.
* ``balanced_jet_state``: barotropic zonal jet u = 35 sin^2(2 phi) m/s on an
  isothermal 300 K atmosphere with ln(ps) in gradient-wind balance (for an
  isothermal atmosphere without orography the pressure-gradient force is
  R T grad(ln ps) on every hybrid surface, so the balance holds at all
  levels), plus 1 K seeded temperature noise in wavenumbers 1..42.

Spectral coefficients use the transform library's convention: orthonormal
harmonics without Condon-Shortley phase, m-major triangular order, m > 0
coefficients standing for the (+m, -m) pair of a real field
(src/shtns.f90:110, :149-150).  Arrays are ``complex128[nlev, nlm]``.
"""
import numpy as np

RERTH = float(np.float32(6.3712e6))
OMEGA = float(np.float32(7.2921e-5))
RD = float(np.float32(287.05))


def nlm_of(T):
    return (T + 1) * (T + 2) // 2


def degree_order(T):
    deg = np.concatenate([np.arange(m, T + 1) for m in range(T + 1)])
    order = np.concatenate([np.full(T - m + 1, m) for m in range(T + 1)])
    return deg, order


def hybrid_coords(nlev, eta_c=0.2, p0=1.0e5):
    """Interfaces top (k=0) to bottom (k=nlev), as ak/bk in init_dyn.

    eta_k = (1 - cos(pi k / nlev)) / 2 (thin layers at top and bottom),
    bk = ((eta - eta_c) / (1 - eta_c))**2 below eta_c else 0,
    ak = p0 (eta - bk), so ak + bk p0 = p0 eta; top pk = 0, bottom pk = ps.
    """
    k = np.arange(nlev + 1, dtype=np.float64)
    eta = 0.5 * (1.0 - np.cos(np.pi * k / nlev))
    bk = np.where(eta > eta_c, ((eta - eta_c) / (1.0 - eta_c)) ** 2, 0.0)
    ak = p0 * (eta - bk)
    ak[0] = 0.0
    bk[0] = 0.0
    ak[-1] = 0.0
    bk[-1] = 1.0
    return ak, bk


def _legendre_m0(T, mu):
    """Orthonormal P_n^0(mu) and d/dphi for n = 0..T (rows) at nodes mu."""
    s = np.sqrt((1 - mu) * (1 + mu))
    P = np.zeros((T + 1, mu.size))
    H = np.zeros_like(P)
    P[0] = 1.0 / np.sqrt(2.0)
    if T >= 1:
        P[1] = np.sqrt(3.0) * mu * P[0]
    for n in range(2, T + 1):
        a = np.sqrt((4.0 * n * n - 1) / (n * n))
        b = np.sqrt(((n - 1.0) ** 2) / (4.0 * (n - 1) ** 2 - 1))
        P[n] = a * (mu * P[n - 1] - b * P[n - 2])
    for n in range(1, T + 1):
        c = np.sqrt(n * n * (2 * n + 1.0) / (2 * n - 1.0))
        H[n] = (-n * mu * P[n] + c * P[n - 1]) / s
    return P / np.sqrt(2 * np.pi), H / np.sqrt(2 * np.pi)


def _rms_normalise(coef, deg, order, rms):
    """Scale coefficients so the grid RMS of the field equals rms."""
    w = np.where(order == 0, 1.0, 2.0)
    ms = np.sum(w * np.abs(coef) ** 2) / (4 * np.pi)
    return coef * (rms / np.sqrt(ms)) if ms > 0 else coef


def _noise(rng, T, nmin, nmax, slope=0.0):
    deg, order = degree_order(T)
    c = rng.standard_normal(deg.size) + 1j * rng.standard_normal(deg.size)
    c[order == 0] = c[order == 0].real
    band = (deg >= nmin) & (deg <= nmax)
    amp = np.where(band, np.maximum(deg, 1).astype(float) ** slope, 0.0)
    return c * amp, deg, order


def _const(T, value):
    c = np.zeros(nlm_of(T), np.complex128)
    c[0] = value * np.sqrt(4 * np.pi)
    return c


def hs_rest_state(T, nlev, seed=0, amp=1.0e-6, nmax=20):
    rng = np.random.default_rng(seed)
    nlm = nlm_of(T)
    vrt = np.zeros((nlev, nlm), np.complex128)
    for k in range(nlev):
        c, deg, order = _noise(rng, T, 1, min(nmax, T))
        vrt[k] = _rms_normalise(c, deg, order, amp)
    div = np.zeros_like(vrt)
    tv = np.tile(_const(T, 300.0), (nlev, 1))
    lnps = _const(T, np.log(1.0e5))
    return dict(vrt=vrt, div=div, tv=tv, lnps=lnps, trc=np.zeros((0, nlev, nlm), np.complex128))


def smooth_random_state(T, nlev, ntrac=3, seed=0):
    rng = np.random.default_rng(seed)
    nlm = nlm_of(T)
    out = {}
    spec = dict(vrt=(0.0, 1.0e-5), div=(0.0, 1.0e-6), tv=(280.0, 5.0))
    for name, (mean, rms) in spec.items():
        a = np.zeros((nlev, nlm), np.complex128)
        for k in range(nlev):
            c, deg, order = _noise(rng, T, 1, T, slope=-2.0)
            a[k] = _rms_normalise(c, deg, order, rms) + _const(T, mean)
        out[name] = a
    c, deg, order = _noise(rng, T, 1, T, slope=-2.0)
    out["lnps"] = _rms_normalise(c, deg, order, 0.01) + _const(T, np.log(1.0e5))
    trc = np.zeros((ntrac, nlev, nlm), np.complex128)
    for q in range(ntrac):
        for k in range(nlev):
            c, deg, order = _noise(rng, T, 1, T, slope=-2.0)
            trc[q, k] = _rms_normalise(c, deg, order, 1.0e-4) + _const(T, 1.0e-3 * (q + 1))
    out["trc"] = trc
    return out


def balanced_jet_state(T, nlat, nlev, seed=0, u0=35.0, tnoise=1.0, ntrac=0):
    from numpy.polynomial.legendre import leggauss

    x, w = leggauss(nlat)
    mu, w = x[::-1], w[::-1]
    W = 2 * np.pi * w
    phi = np.arcsin(mu)
    P, H = _legendre_m0(T, mu)
    deg, order = degree_order(T)
    nlm = nlm_of(T)
    # vorticity of u = u0 sin^2(2 phi): -(1/(a cos)) d(u cos)/dphi
    s2, c2 = np.sin(2 * phi), np.cos(2 * phi)
    vrt_g = -(u0 / RERTH) * (4 * s2 * c2 - s2 * s2 * np.tan(phi))
    vrt0 = (P * (W * vrt_g)).sum(axis=1)  # n = 0..T, m = 0 block
    vrt0[0] = 0.0
    # spectral-consistent u: u = -(1/a) dPsi/dphi, Psi = a^2 invlap vrt
    n = np.arange(T + 1, dtype=float)
    il = np.zeros(T + 1)
    il[1:] = -1.0 / (n[1:] * (n[1:] + 1))
    u = -(H * (RERTH * il * vrt0)[:, None]).sum(axis=0)
    f = 2 * OMEGA * mu
    G = -(RERTH * f * u + u * u * np.tan(phi)) / (RD * 300.0)  # d lnps / d phi
    lnps0 = np.zeros(T + 1)
    lnps0[1:] = (H[1:] * (W * G)).sum(axis=1) / (n[1:] * (n[1:] + 1))
    lnps = np.zeros(nlm, np.complex128)
    lnps[: T + 1] = lnps0
    lnps[0] = np.log(1.0e5) * np.sqrt(4 * np.pi)
    vrt = np.zeros((nlev, nlm), np.complex128)
    vrt[:, : T + 1] = vrt0
    rng = np.random.default_rng(seed)
    tv = np.zeros((nlev, nlm), np.complex128)
    for k in range(nlev):
        c, d_, o_ = _noise(rng, T, 1, min(42, T))
        tv[k] = _rms_normalise(c, d_, o_, tnoise) + _const(T, 300.0)
    trc = np.zeros((ntrac, nlev, nlm), np.complex128)
    for q in range(ntrac):
        trc[q] = _const(T, 1.0e-3 * (q + 1))
    return dict(vrt=vrt, div=np.zeros_like(vrt), tv=tv, lnps=lnps, trc=trc)
