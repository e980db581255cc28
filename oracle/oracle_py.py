"""ctypes wrapper of the FP64 CPU oracle -- TEST INFRASTRUCTURE ONLY.

Used by tests/, by ``__graft_entry__.smoke()`` as the oracle and by
``bench.py``'s CPU-baseline leg; the product never imports it.  The oracle
restates the jswhit/gfs-dycore time step (src/shtns.f90, src/dyn_run.f90,
src/run.f90, src/semimp_data.f90, src/pressure_data.f90,
src/phy_run_hs.f90) in C++ (gd_oracle.cpp).

Arrays use the reference layouts: spectral ``complex128[nlev, nlm]``
(Fortran ``complex(ndimspec,nlevs)``), grid ``float64[nlev, nlat, nlon]``.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")


def build():
    """Compile the oracle with its Makefile (g++, OpenMP)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


class OraConfig(ctypes.Structure):
    _fields_ = [
        ("ntrunc", ctypes.c_int), ("nlon", ctypes.c_int), ("nlat", ctypes.c_int),
        ("nlev", ctypes.c_int), ("ntrac", ctypes.c_int), ("dt", ctypes.c_double),
        ("explicit_", ctypes.c_int), ("adiabatic", ctypes.c_int),
        ("heldsuarez", ctypes.c_int), ("massfix", ctypes.c_int), ("dry", ctypes.c_int),
        ("ndiss", ctypes.c_int), ("efold", ctypes.c_double), ("hdif_fac", ctypes.c_double),
        ("hdif_fac2", ctypes.c_double), ("fshk", ctypes.c_double),
        ("taustratdamp", ctypes.c_double), ("pdryini", ctypes.c_double),
        ("nthreads", ctypes.c_int), ("dcmip", ctypes.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        L.ora_create.restype = vp
        L.ora_create.argtypes = [ctypes.POINTER(OraConfig), dp, dp]
        L.ora_destroy.argtypes = [vp]
        L.ora_nlm.argtypes = [vp]
        L.ora_nlm.restype = ctypes.c_int
        L.ora_get_grid.restype = ctypes.c_int
        for name in ["ora_set_state", "ora_get_state", "ora_spectogrd", "ora_grdtospec",
                     "ora_getuv", "ora_getvrtdivspec", "ora_getgrad", "ora_getdyntend",
                     "ora_grid_info", "ora_legendre", "ora_semimp", "ora_damp", "ora_diag",
                     "ora_getphytend", "ora_get_grid"]:
            getattr(L, name).restype = getattr(L, name).restype or None
        L.ora_advance.argtypes = [vp, ctypes.c_double, ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """FP64 CPU dycore; mirrors init_dyn / getdyntend / advance."""

    def __init__(self, ntrunc, nlon, nlat, nlev, ak, bk, ntrac=0, dt=1200.0,
                 explicit=False, adiabatic=False, heldsuarez=True, massfix=True,
                 dry=True, nthreads=0, pdryini=0.0, **kw):
        L = lib()
        c = OraConfig()
        L.ora_default_config(ctypes.byref(c))
        c.ntrunc, c.nlon, c.nlat, c.nlev, c.ntrac = ntrunc, nlon, nlat, nlev, ntrac
        c.dt = dt
        c.explicit_ = int(explicit)
        c.adiabatic = int(adiabatic)
        c.heldsuarez = int(heldsuarez)
        c.massfix = int(massfix)
        c.dry = int(dry)
        c.nthreads = nthreads
        c.pdryini = pdryini
        for k, v in kw.items():
            setattr(c, k, v)
        self.cfg = c
        self.ak = np.ascontiguousarray(ak, dtype=np.float64)
        self.bk = np.ascontiguousarray(bk, dtype=np.float64)
        self.h = L.ora_create(ctypes.byref(c), self.ak.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                              self.bk.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        self.nlm = L.ora_nlm(self.h)
        self.ntrunc, self.nlon, self.nlat, self.nlev, self.ntrac = ntrunc, nlon, nlat, nlev, ntrac

    def __del__(self):
        if getattr(self, "h", None):
            lib().ora_destroy(self.h)
            self.h = None

    # ---- state ----
    def set_state(self, vrt, div, tv, lnps, trc=None, topo=None):
        c128 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.complex128)
        self._keep = [c128(x) for x in (vrt, div, tv, trc, lnps, topo)]
        lib().ora_set_state(self.h, *[_p(x) for x in self._keep])

    def get_state(self):
        L, n = self.nlev, self.nlm
        vrt = np.zeros((L, n), np.complex128)
        div = np.zeros_like(vrt)
        tv = np.zeros_like(vrt)
        trc = np.zeros((max(self.ntrac, 1), L, n), np.complex128)
        lnps = np.zeros(n, np.complex128)
        lib().ora_get_state(self.h, _p(vrt), _p(div), _p(tv), _p(trc), _p(lnps))
        return dict(vrt=vrt, div=div, tv=tv, trc=trc[: self.ntrac], lnps=lnps)

    # ---- transforms (batched over leading axis) ----
    def _gshape(self, nb):
        return (nb, self.nlat, self.nlon)

    def spectogrd(self, spec):
        spec = np.ascontiguousarray(np.atleast_2d(spec), np.complex128)
        g = np.zeros(self._gshape(spec.shape[0]))
        lib().ora_spectogrd(self.h, spec.shape[0], _p(spec), _p(g))
        return g

    def grdtospec(self, grid):
        grid = np.ascontiguousarray(grid, np.float64).reshape(-1, self.nlat, self.nlon)
        s = np.zeros((grid.shape[0], self.nlm), np.complex128)
        lib().ora_grdtospec(self.h, grid.shape[0], _p(grid), _p(s))
        return s

    def getuv(self, vrt, div):
        vrt = np.ascontiguousarray(np.atleast_2d(vrt), np.complex128)
        div = np.ascontiguousarray(np.atleast_2d(div), np.complex128)
        u = np.zeros(self._gshape(vrt.shape[0]))
        v = np.zeros_like(u)
        lib().ora_getuv(self.h, vrt.shape[0], _p(vrt), _p(div), _p(u), _p(v))
        return u, v

    def getvrtdivspec(self, u, v):
        u = np.ascontiguousarray(u, np.float64).reshape(-1, self.nlat, self.nlon)
        v = np.ascontiguousarray(v, np.float64).reshape(-1, self.nlat, self.nlon)
        vrt = np.zeros((u.shape[0], self.nlm), np.complex128)
        div = np.zeros_like(vrt)
        lib().ora_getvrtdivspec(self.h, u.shape[0], _p(u), _p(v), _p(vrt), _p(div))
        return vrt, div

    def getgrad(self, spec):
        spec = np.ascontiguousarray(np.atleast_2d(spec), np.complex128)
        gx = np.zeros(self._gshape(spec.shape[0]))
        gy = np.zeros_like(gx)
        lib().ora_getgrad(self.h, spec.shape[0], _p(spec), _p(gx), _p(gy))
        return gx, gy

    # ---- dynamics ----
    def getdyntend(self, rkstage=1, inverse_only=False):
        L, n = self.nlev, self.nlm
        d = [np.zeros((L, n), np.complex128) for _ in range(3)]
        dtrc = np.zeros((max(self.ntrac, 1), L, n), np.complex128)
        dl = np.zeros(n, np.complex128)
        lib().ora_getdyntend(self.h, rkstage, int(inverse_only), _p(d[0]), _p(d[1]), _p(d[2]),
                             _p(dtrc), _p(dl))
        return dict(dvrt=d[0], ddiv=d[1], dtv=d[2], dtrc=dtrc[: self.ntrac], dlnps=dl)

    def getphytend(self):
        L, n = self.nlev, self.nlm
        d = [np.zeros((L, n), np.complex128) for _ in range(3)]
        dtrc = np.zeros((max(self.ntrac, 1), L, n), np.complex128)
        dl = np.zeros(n, np.complex128)
        lib().ora_getphytend(self.h, _p(d[0]), _p(d[1]), _p(d[2]), _p(dtrc), _p(dl))
        return dict(dvrt=d[0], ddiv=d[1], dtv=d[2], dtrc=dtrc[: self.ntrac], dlnps=dl)

    def set_sppt(self, pattern, sigtop=0.05, sigbot=0.10):
        """Attach a PatternOracle as stochastically perturbed physics."""
        self._sppt = pattern
        L = lib()
        L.ora_set_sppt.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
        L.ora_set_sppt(self.h, pattern.h, sigtop, sigbot)

    def advance(self, nsteps=1, t=0.0):
        lib().ora_advance(self.h, ctypes.c_double(t), nsteps)

    def get_grid(self, name):
        L = self.nlev
        shapes = dict(ug=L, vg=L, vrtg=L, divg=L, tvg=L, dlnpdtg=L, prs=L, etadot=L + 1,
                      trcg=max(self.ntrac, 1) * L, lnpsg=1, psg=1, dlnpsdt=1, dphisdx=1, dphisdy=1,
                      precip=1, apcp=1, pwat=1)
        out = np.zeros((shapes[name], self.nlat, self.nlon))
        rc = lib().ora_get_grid(self.h, name.encode(), _p(out))
        assert rc == 0
        return out

    def grid_info(self):
        lats = np.zeros(self.nlat)
        gw = np.zeros(self.nlat)
        aw = np.zeros(self.nlat)
        deg = np.zeros(self.nlm, np.int32)
        order = np.zeros(self.nlm, np.int32)
        lap = np.zeros(self.nlm)
        ilap = np.zeros(self.nlm)
        lib().ora_grid_info(self.h, _p(lats), _p(gw), _p(aw), _p(deg), _p(order), _p(lap), _p(ilap))
        return dict(lats=lats, gauwts=gw, areawts=aw, degree=deg, order=order, lap=lap, invlap=ilap)

    def legendre(self, m):
        K = self.ntrunc - m + 1
        P = np.zeros((self.nlat // 2, K))
        H = np.zeros_like(P)
        lib().ora_legendre(self.h, m, _p(P), _p(H))
        return P, H

    def semimp(self):
        L, T = self.nlev, self.ntrunc
        a = np.zeros((L, L))
        b = np.zeros((L, L))
        sv = np.zeros(L)
        tor = np.zeros(L)
        d = np.zeros((3, T + 1, L, L))
        ym = np.zeros((L, L))
        lib().ora_semimp(self.h, _p(a), _p(b), _p(sv), _p(tor), _p(d), _p(ym))
        return dict(amhyb=a, bmhyb=b, svhyb=sv, tor_hyb=tor, d_hyb_m=d, ym=ym)

    def damp(self):
        dis = np.zeros(self.nlm)
        dp = np.zeros(self.nlev)
        mp = np.zeros(self.nlev)
        lib().ora_damp(self.h, _p(dis), _p(dp), _p(mp))
        return dict(disspec=dis, diff_prof=dp, dmp_prof=mp)

    def set_iau(self, fhrs, delthrs=6.0, vrt=None, div=None, tv=None, trc=None, lnps=None):
        """IAU increments with a leading file axis (iau_module.f90); fhrs=None detaches."""
        L = lib()
        L.ora_set_iau.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_double] + [
            ctypes.c_void_p] * 5
        if fhrs is None:
            L.ora_set_iau(self.h, 0, None, delthrs, None, None, None, None, None)
            return
        c = lambda a: None if a is None else np.ascontiguousarray(a, np.complex128)
        self._iau = [np.ascontiguousarray(fhrs, np.float64)] + [c(x) for x in (vrt, div, tv, trc, lnps)]
        L.ora_set_iau(self.h, len(self._iau[0]), *[_p(self._iau[0])], delthrs, *[_p(x) for x in self._iau[1:]])

    def getiauforcing(self, t):
        L_, n = self.nlev, self.nlm
        d = [np.zeros((L_, n), np.complex128) for _ in range(3)]
        dtrc = np.zeros((max(self.ntrac, 1), L_, n), np.complex128)
        dl = np.zeros(n, np.complex128)
        L = lib()
        L.ora_getiauforcing.argtypes = [ctypes.c_void_p, ctypes.c_double] + [ctypes.c_void_p] * 5
        L.ora_getiauforcing(self.h, t, _p(d[0]), _p(d[1]), _p(d[2]), _p(dtrc) if self.ntrac else None, _p(dl))
        return dict(dvrt=d[0], ddiv=d[1], dtv=d[2], dtrc=dtrc[: self.ntrac], dlnps=dl)

    def dfi(self, ntdfi, t=0.0):
        L = lib()
        L.ora_dfi.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
        L.ora_dfi(self.h, t, ntdfi)

    def diag(self):
        o = np.zeros(5)
        lib().ora_diag(self.h, _p(o))
        return dict(spdmax=o[0], psmin=o[1], psmax=o[2], pstend=o[3], pdryini=o[4])


def dfi_weights(ntdfi):
    w = np.zeros(2 * ntdfi + 1)
    lib().ora_dfi_weights(int(ntdfi), _p(w))
    return w


def simple_columns(dtime, lat, t, q, u, v, pmid, pint, ps, test, turbflux):
    """simple_physics_v5_1.f90 on independent columns (top to bottom);
    returns updated (t, q, u, v) and precl."""
    arr = lambda a: np.ascontiguousarray(a, np.float64).copy()
    t, q, u, v = arr(t), arr(q), arr(u), arr(v)
    ncol, n = t.shape
    precl = np.zeros(ncol)
    lib().ora_simple_columns(ncol, n, ctypes.c_double(dtime), _p(arr(lat)), _p(t), _p(q), _p(u), _p(v),
                             _p(arr(pmid)), _p(arr(pint)), _p(arr(ps)), _p(precl), int(test), int(turbflux))
    return t, q, u, v, precl


# ---- stochastic pattern generator (gd_pattern_oracle.cpp) --------------------
def _pattern_lib():
    L = lib()
    if getattr(L, "_pattern_ready", False):
        return L
    vp, fp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)
    dp = vp  # arrays are passed as raw pointers
    L.ora_mt_uniform.argtypes = [ctypes.c_int, ctypes.c_int, fp]
    L.ora_mt_gauss.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), fp]
    L.ora_mt_kat.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
    L.ora_mt_kat.restype = ctypes.c_uint32
    L.ora_pattern_create.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int]
    L.ora_pattern_create.restype = vp
    L.ora_pattern_destroy.argtypes = [vp]
    L.ora_pattern_start.argtypes = [vp]
    L.ora_pattern_advance.argtypes = [vp, ctypes.c_int]
    L.ora_pattern_get.argtypes = [vp, dp]
    L.ora_pattern_getnoise.argtypes = [vp, dp]
    L.ora_pattern_spectra.argtypes = [vp, dp, dp, dp]
    L.ora_pattern_varspec.argtypes = [vp, ctypes.c_int]
    L.ora_pattern_varspec.restype = ctypes.c_double
    L.ora_pattern_getvarspectrum.argtypes = [vp, ctypes.c_int, dp]
    L._pattern_ready = True
    return L


def mt_uniform(seed, n):
    """w3lib random_setseed(seed) then random_number of n values (float32)."""
    out = np.zeros(n, np.float32)
    _pattern_lib().ora_mt_uniform(seed, n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return out


def mt_gauss(seed, counts):
    """random_setseed(seed) then one random_gauss call per entry of counts."""
    counts = np.ascontiguousarray(counts, np.int32)
    out = np.zeros(int(counts.sum()), np.float32)
    _pattern_lib().ora_mt_gauss(seed, len(counts), counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return out


def mt_kat():
    """(this MT19937's 10000th output, std::mt19937's) from the standard seed 5489."""
    z = ctypes.c_uint32(0)
    y = _pattern_lib().ora_mt_kat(ctypes.byref(z))
    return int(y), int(z.value)


class PatternOracle:
    """Single-precision restatement of patterngenerator.f90 (random_pattern)."""

    def __init__(self, lscale, delt, tscale, stdev, iseed, jcap, normalization=2 * np.float32(np.pi),
                 nfields=1):
        L = _pattern_lib()
        self.jcap, self.nfields = jcap, nfields
        self.nlm = (jcap + 1) * (jcap + 2) // 2
        self.h = L.ora_pattern_create(lscale, delt, tscale, stdev, iseed, jcap, float(normalization), nfields)

    def __del__(self):
        if getattr(self, "h", None):
            _pattern_lib().ora_pattern_destroy(self.h)
            self.h = None

    def start(self):
        _pattern_lib().ora_pattern_start(self.h)

    def advance(self, nsteps=1):
        _pattern_lib().ora_pattern_advance(self.h, nsteps)

    def get(self):
        out = np.zeros((self.nfields, self.nlm), np.complex128)
        _pattern_lib().ora_pattern_get(self.h, _p(out))
        return out

    def getnoise(self):
        out = np.zeros(self.nlm, np.complex128)
        _pattern_lib().ora_pattern_getnoise(self.h, _p(out))
        return out

    def spectra(self):
        vs = np.zeros(self.nlm)
        v1 = np.zeros(self.jcap + 1)
        phi = np.zeros(1)
        _pattern_lib().ora_pattern_spectra(self.h, _p(vs), _p(v1), _p(phi))
        return vs, v1, float(phi[0])

    def varspec(self, field=0):
        return _pattern_lib().ora_pattern_varspec(self.h, field)

    def getvarspectrum(self, field=0):
        out = np.zeros(self.jcap + 1)
        _pattern_lib().ora_pattern_getvarspectrum(self.h, field, _p(out))
        return out
