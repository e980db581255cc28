"""ctypes binding of libgdcore.so (include/gd_api.h).

``Dycore`` mirrors the reference's dynamics interface -- init_dyn,
getdyntend, getphytend, advance, finalize_dyn (src/dyn_init.f90,
src/dyn_run.f90, src/phy_run_hs.f90, src/run.f90) -- and the shtns.f90
transform facade, with the reference's array layouts:
spectral ``complex128[nlev, nlm]`` and grid ``float64[nlev, nlat, nlon]``.

Errors raise ``GdError`` carrying the library status and message; there is
no fallback path: if the CUDA library cannot be loaded or the device cannot
be initialised the call fails.
"""
import ctypes
import os

import numpy as np

from . import build as _build

GD_OK = 0
GD_ERR_ARG = -1
GD_ERR_CUDA = -2
GD_ERR_STATE = -3
GD_ERR_NOMEM = -4
GD_ERR_UNSUPPORTED = -5
GD_ERR_NUMERIC = -6
GD_ERR_IO = -7

PREC = {"fp64": 0, "fp32": 1, "tf32x3": 2, "bf16x3": 3, "f64_tf32x3": 4, "f64_eddy": 5}

API_FUNCTIONS = [
    "gd_default_config", "gd_init", "gd_finalize", "gd_set_state", "gd_get_state", "gd_get_topo",
    "gd_set_state_f", "gd_get_state_f", "gd_spectogrd_f", "gd_grdtospec_f", "gd_getuv_f", "gd_getvrtdivspec_f",
    "gd_getgrad_f",
    "gd_getdyntend", "gd_getphytend", "gd_advance", "gd_spectogrd", "gd_grdtospec",
    "gd_getuv", "gd_getvrtdivspec", "gd_getgrad", "gd_grid_info", "gd_get_grid", "gd_diag",
    "gd_set_stream", "gd_sync", "gd_launch_count", "gd_last_error", "gd_profile_step",
    "gd_diag_static",
    "gd_pattern_init", "gd_pattern_start", "gd_pattern_advance", "gd_pattern_getnoise", "gd_pattern_get",
    "gd_pattern_set", "gd_pattern_spectra", "gd_pattern_destroy", "gd_pattern_set_stream", "gd_pattern_sync",
    "gd_pattern_launch_count", "gd_pattern_last_error", "gd_set_sppt", "gd_ensemble_advance",
    "gd_sigio_head_init", "gd_sigio_read_head", "gd_sigio_read", "gd_sigio_write", "gd_sigio_config",
    "gd_read_sig", "gd_write_sig", "gd_sigio_last_error", "gd_dcmip_ics",
    "gd_dcmip_point", "gd_set_iau", "gd_set_iau_files", "gd_dfi", "gd_dfi_weights",
    "gd_mlp_init", "gd_mlp_destroy", "gd_mlp_nparams", "gd_mlp_get_params", "gd_mlp_set_params",
    "gd_mlp_set_norm", "gd_mlp_forward", "gd_mlp_loss_grad", "gd_mlp_train_step", "gd_mlp_set_stream",
    "gd_mlp_sync", "gd_mlp_last_error", "gd_set_closure", "gd_closure_features", "gd_autotune",
]
PHASES = ["legendre_synth", "fft_synth", "columns", "fft_anal", "legendre_anal", "semi_implicit",
          "physics", "other", "column_physics"]


class GdConfig(ctypes.Structure):
    _fields_ = [
        ("ntrunc", ctypes.c_int), ("nlon", ctypes.c_int), ("nlat", ctypes.c_int),
        ("nlev", ctypes.c_int), ("ntrac", ctypes.c_int), ("dt", ctypes.c_double),
        ("precision", ctypes.c_int), ("explicit_", ctypes.c_int), ("adiabatic", ctypes.c_int),
        ("heldsuarez", ctypes.c_int), ("massfix", ctypes.c_int), ("dry", ctypes.c_int),
        ("ndiss", ctypes.c_int), ("efold", ctypes.c_double), ("hdif_fac", ctypes.c_double),
        ("hdif_fac2", ctypes.c_double), ("fshk", ctypes.c_double),
        ("taustratdamp", ctypes.c_double), ("pdryini", ctypes.c_double), ("device", ctypes.c_int),
        ("dcmip", ctypes.c_int),
    ]


class GdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gd error {code}: {msg}")
        self.code = code


_lib = None


def load(build_if_missing=True):
    """Load the in-tree libgdcore.so (building it first if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise OSError(f"{_build.LIB} is not built")
        _build.build()
    L = ctypes.CDLL(_build.LIB)
    vp = ctypes.c_void_p
    L.gd_init.argtypes = [ctypes.POINTER(GdConfig), vp, vp, ctypes.POINTER(vp)]
    L.gd_finalize.argtypes = [vp]
    L.gd_last_error.restype = ctypes.c_char_p
    L.gd_last_error.argtypes = [vp]
    L.gd_launch_count.restype = ctypes.c_longlong
    L.gd_launch_count.argtypes = [vp]
    L.gd_advance.argtypes = [vp, ctypes.c_double, ctypes.c_int]
    L.gd_set_stream.argtypes = [vp, vp]
    for f in ["gd_set_state_f", "gd_get_state_f", "gd_spectogrd_f", "gd_grdtospec_f", "gd_getuv_f",
              "gd_getvrtdivspec_f", "gd_getgrad_f"]:
        getattr(L, f).restype = ctypes.c_int
    for f in ["gd_set_state", "gd_get_state", "gd_get_topo", "gd_getdyntend", "gd_getphytend", "gd_spectogrd",
              "gd_grdtospec", "gd_getuv", "gd_getvrtdivspec", "gd_getgrad", "gd_grid_info",
              "gd_get_grid", "gd_diag", "gd_sync", "gd_profile_step"]:
        getattr(L, f).restype = ctypes.c_int
    L.gd_diag_static.restype = ctypes.c_int
    L.gd_diag_static.argtypes = [vp, vp, ctypes.c_int, vp, vp, vp, ctypes.c_int, ctypes.c_int, vp, vp]
    d, i = ctypes.c_double, ctypes.c_int
    L.gd_pattern_init.argtypes = [d, d, d, d, i, i, i, i, d, i, i, ctypes.POINTER(vp)]
    for f in ["gd_pattern_start", "gd_pattern_destroy", "gd_pattern_sync"]:
        getattr(L, f).argtypes = [vp]
    L.gd_pattern_advance.argtypes = [vp, i]
    for f in ["gd_pattern_getnoise", "gd_pattern_get", "gd_pattern_set", "gd_pattern_set_stream"]:
        getattr(L, f).argtypes = [vp, vp]
    L.gd_pattern_spectra.argtypes = [vp, vp, vp, vp]
    L.gd_pattern_launch_count.restype = ctypes.c_longlong
    L.gd_pattern_launch_count.argtypes = [vp]
    L.gd_pattern_last_error.restype = ctypes.c_char_p
    L.gd_pattern_last_error.argtypes = [vp]
    L.gd_set_sppt.argtypes = [vp, vp, d, d]
    L.gd_ensemble_advance.argtypes = [ctypes.POINTER(vp), i, d, i]
    cp = ctypes.c_char_p
    L.gd_sigio_head_init.argtypes = [vp]
    L.gd_sigio_read_head.argtypes = [cp, vp]
    L.gd_sigio_read.argtypes = [cp, i, i, i, vp, vp, vp, vp, vp, vp, vp]
    L.gd_sigio_write.argtypes = [cp, vp, i, vp, vp, vp, vp, vp, vp]
    L.gd_sigio_config.argtypes = [vp, vp, vp, vp]
    L.gd_read_sig.argtypes = [vp, cp, vp]
    L.gd_write_sig.argtypes = [vp, cp, d, vp]
    L.gd_sigio_last_error.restype = ctypes.c_char_p
    L.gd_sigio_last_error.argtypes = []
    L.gd_dcmip_ics.argtypes = [vp, i]
    L.gd_dcmip_point.argtypes = [i, i, d, d, d, vp]
    L.gd_set_iau.argtypes = [vp, i, vp, d, vp, vp, vp, vp, vp]
    L.gd_set_iau_files.argtypes = [vp, i, vp, d, ctypes.POINTER(cp), ctypes.POINTER(cp)]
    L.gd_dfi.argtypes = [vp, d, i]
    L.gd_dfi_weights.argtypes = [i, vp]
    f = ctypes.c_float
    L.gd_mlp_init.argtypes = [i, i, i, i, ctypes.c_ulonglong, i, ctypes.POINTER(vp)]
    L.gd_mlp_destroy.argtypes = [vp]
    L.gd_mlp_nparams.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
    L.gd_mlp_get_params.argtypes = [vp, vp]
    L.gd_mlp_set_params.argtypes = [vp, vp]
    L.gd_mlp_set_norm.argtypes = [vp, vp, vp, vp, vp]
    L.gd_mlp_forward.argtypes = [vp, vp, i, vp]
    L.gd_mlp_loss_grad.argtypes = [vp, vp, vp, i, vp, vp]
    L.gd_mlp_train_step.argtypes = [vp, vp, vp, i, f, vp]
    L.gd_mlp_set_stream.argtypes = [vp, vp]
    L.gd_mlp_sync.argtypes = [vp]
    L.gd_mlp_last_error.restype = ctypes.c_char_p
    L.gd_mlp_last_error.argtypes = [vp]
    L.gd_set_closure.argtypes = [vp, vp]
    L.gd_closure_features.argtypes = [vp, vp]
    L.gd_autotune.argtypes = [vp, vp]
    _lib = L
    return L


def default_config(**kw):
    c = GdConfig()
    load().gd_default_config(ctypes.byref(c))
    for k, v in kw.items():
        if k == "precision" and isinstance(v, str):
            v = PREC[v]
        setattr(c, k, v)
    return c


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def dfi_weights(ntdfi):
    """gd_dfi_weights: the Lanczos weights of the digital filter."""
    w = np.zeros(2 * ntdfi + 1)
    rc = load().gd_dfi_weights(int(ntdfi), _p(w))
    if rc != GD_OK:
        raise GdError(rc, "gd_dfi_weights: ntdfi must be >= 1")
    return w


def dcmip_point(testcase, lon, lat, p, moist=True):
    """gd_dcmip_point: (u, v, T, phis, ps, q, q1, q2) of a DCMIP-2012 case at one point."""
    out = np.zeros(8)
    rc = load().gd_dcmip_point(int(testcase), int(moist), float(lon), float(lat), float(p), _p(out))
    if rc != GD_OK:
        raise GdError(rc, "gd_dcmip_point: bad arguments")
    return out


class Dycore:
    """One device context (gd_ctx) of the GB300 spectral dycore."""

    def __init__(self, ntrunc, nlon, nlat, nlev, ak, bk, ntrac=0, dt=1200.0, precision="fp64",
                 explicit=False, adiabatic=False, heldsuarez=True, massfix=True, dry=True,
                 device=0, **kw):
        L = load()
        self.cfg = default_config(ntrunc=ntrunc, nlon=nlon, nlat=nlat, nlev=nlev, ntrac=ntrac,
                                  dt=dt, precision=precision, explicit_=int(explicit),
                                  adiabatic=int(adiabatic), heldsuarez=int(heldsuarez),
                                  massfix=int(massfix), dry=int(dry), device=device, **kw)
        self.ak = np.ascontiguousarray(ak, np.float64)
        self.bk = np.ascontiguousarray(bk, np.float64)
        h = ctypes.c_void_p()
        rc = L.gd_init(ctypes.byref(self.cfg), _p(self.ak), _p(self.bk), ctypes.byref(h))
        if rc != GD_OK:
            raise GdError(rc, L.gd_last_error(None).decode())
        self.h = h
        self.ntrunc, self.nlon, self.nlat, self.nlev, self.ntrac = ntrunc, nlon, nlat, nlev, ntrac
        self.nlm = (ntrunc + 1) * (ntrunc + 2) // 2

    def close(self):
        if getattr(self, "h", None):
            load().gd_finalize(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        if rc != GD_OK:
            raise GdError(rc, load().gd_last_error(self.h).decode())

    # ---- state ----
    def set_state(self, vrt, div, tv, lnps, trc=None, topo=None):
        """complex64 arrays go through gd_set_state_f (single-precision host
        layout), anything else through gd_set_state."""
        f = self._single(vrt)
        ct = np.complex64 if f else np.complex128
        c = lambda a: None if a is None else np.ascontiguousarray(a, ct)
        arr = [c(x) for x in (vrt, div, tv, trc, lnps, topo)]
        fn = load().gd_set_state_f if f else load().gd_set_state
        self._chk(fn(self.h, *[_p(x) for x in arr]))

    def get_state(self, single=False):
        L, n = self.nlev, self.nlm
        ct = np.complex64 if single else np.complex128
        vrt = np.zeros((L, n), ct)
        div = np.zeros_like(vrt)
        tv = np.zeros_like(vrt)
        trc = np.zeros((max(self.ntrac, 1), L, n), ct)
        lnps = np.zeros(n, ct)
        fn = load().gd_get_state_f if single else load().gd_get_state
        self._chk(fn(self.h, _p(vrt), _p(div), _p(tv), _p(trc), _p(lnps)))
        return dict(vrt=vrt, div=div, tv=tv, trc=trc[: self.ntrac], lnps=lnps)

    def get_topo(self):
        """Orography (complex [nlm], m) of the last set_state."""
        out = np.zeros(self.nlm, np.complex128)
        self._chk(load().gd_get_topo(self.h, _p(out)))
        return out

    def dcmip_ics(self, testcase):
        """DCMIP-2012 test 4x (baroclinic wave) or 5x (tropical cyclone) initial state (gd_dcmip_ics)."""
        self._chk(load().gd_dcmip_ics(self.h, int(testcase)))

    def set_iau(self, fhrs, delthrs=6.0, vrt=None, div=None, tv=None, trc=None, lnps=None):
        """gd_set_iau: increments with a leading file axis; fhrs=None detaches."""
        if fhrs is None:
            self._chk(load().gd_set_iau(self.h, 0, None, ctypes.c_double(delthrs), None, None, None, None, None))
            return
        fh = np.ascontiguousarray(fhrs, np.float64)
        c = lambda a: None if a is None else np.ascontiguousarray(a, np.complex128)
        self._iau = [fh] + [c(x) for x in (vrt, div, tv, trc, lnps)]
        self._chk(load().gd_set_iau(self.h, len(fh), _p(fh), ctypes.c_double(delthrs),
                                    *[_p(x) for x in self._iau[1:]]))

    def set_iau_files(self, fhrs, fg, anl, delthrs=6.0):
        """gd_set_iau_files: increments from first-guess / analysis sigma files."""
        fh = np.ascontiguousarray(fhrs, np.float64)
        arr = lambda names: (ctypes.c_char_p * len(names))(*[str(x).encode() for x in names])
        self._chk(load().gd_set_iau_files(self.h, len(fh), _p(fh), ctypes.c_double(delthrs), arr(fg), arr(anl)))

    def dfi(self, ntdfi, t=0.0):
        """gd_dfi: the digital filter over 2 ntdfi steps from time t."""
        self._chk(load().gd_dfi(self.h, ctypes.c_double(t), int(ntdfi)))

    def read_sig(self, path):
        """readin_sig + init_dyn's ln(ps) conversion (gd_read_sig); returns the header."""
        from . import sigio

        return sigio.read_into(self, path)

    def write_sig(self, path, fhour, head):
        """wrtout_sig (gd_write_sig) with head, a sigio.SigHead."""
        from . import sigio

        sigio.write_from(self, path, fhour, head)

    # ---- dynamics ----
    def getdyntend(self, rkstage=1, inverse_only=False):
        L, n = self.nlev, self.nlm
        d = [np.zeros((L, n), np.complex128) for _ in range(3)]
        dtrc = np.zeros((max(self.ntrac, 1), L, n), np.complex128)
        dl = np.zeros(n, np.complex128)
        self._chk(load().gd_getdyntend(self.h, rkstage, int(inverse_only), _p(d[0]), _p(d[1]),
                                       _p(d[2]), _p(dtrc), _p(dl)))
        return dict(dvrt=d[0], ddiv=d[1], dtv=d[2], dtrc=dtrc[: self.ntrac], dlnps=dl)

    def getphytend(self):
        L, n = self.nlev, self.nlm
        d = [np.zeros((L, n), np.complex128) for _ in range(3)]
        dtrc = np.zeros((max(self.ntrac, 1), L, n), np.complex128)
        dl = np.zeros(n, np.complex128)
        self._chk(load().gd_getphytend(self.h, _p(d[0]), _p(d[1]), _p(d[2]), _p(dtrc) if self.ntrac else None,
                                       _p(dl)))
        return dict(dvrt=d[0], ddiv=d[1], dtv=d[2], dtrc=dtrc[: self.ntrac], dlnps=dl)

    def set_sppt(self, pattern, sigtop=0.05, sigbot=0.10):
        """Attach a Pattern as stochastically perturbed physics (None detaches)."""
        self._sppt = pattern  # keep the generator alive while attached
        self._chk(load().gd_set_sppt(self.h, pattern.h if pattern is not None else None, sigtop, sigbot))

    def autotune(self):
        """Times the candidate tile shapes on this context and keeps the fastest;
        returns {"synth_tile": latitude tile of the synthesis GEMM (0 without the
        tensor-core path), "column_levels_per_warp": ..., "a_slots": A-operand
        slots in tensor memory of the Legendre GEMMs (0 without them)}."""
        out = np.zeros(3, np.int32)
        self._chk(load().gd_autotune(self.h, _p(out)))
        return {"synth_tile": int(out[0]), "column_levels_per_warp": int(out[1]), "a_slots": int(out[2])}

    def set_closure(self, net):
        """Attach a trained Mlp as the learned per-column closure (None detaches)."""
        self._closure = net  # keep the net alive while attached
        self._chk(load().gd_set_closure(self.h, net.h if net is not None else None))

    def closure_features(self):
        """Raw closure inputs of the current state: float32 [nlat*nlon, 3 nlev + 1]
        (u, v, Tv at the levels bottom to top, then ps in Pa)."""
        out = np.zeros((self.nlat * self.nlon, 3 * self.nlev + 1), np.float32)
        self._chk(load().gd_closure_features(self.h, _p(out)))
        return out

    def advance(self, nsteps=1, t=0.0):
        self._chk(load().gd_advance(self.h, ctypes.c_double(t), int(nsteps)))

    def sync(self):
        self._chk(load().gd_sync(self.h))

    def set_stream(self, stream_handle):
        self._chk(load().gd_set_stream(self.h, ctypes.c_void_p(stream_handle)))

    def profile_step(self):
        """One eager step; returns {phase: milliseconds}."""
        ms = np.zeros(len(PHASES))
        self._chk(load().gd_profile_step(self.h, _p(ms), len(PHASES)))
        return dict(zip(PHASES, ms.tolist()))

    def launch_count(self):
        return load().gd_launch_count(self.h)

    # ---- transforms ----
    # Transforms: complex128 / float64 arrays use the double entry points;
    # complex64 / float32 arrays the single-precision ones (gd_*_f), which
    # copy the float arrays as they are and convert on the device.
    @staticmethod
    def _single(a):
        return np.asarray(a).dtype in (np.complex64, np.float32)

    def _g(self, nb, single=False):
        return np.zeros((nb, self.nlat, self.nlon), np.float32 if single else np.float64)

    def spectogrd(self, spec):
        f = self._single(spec)
        spec = np.ascontiguousarray(np.atleast_2d(spec), np.complex64 if f else np.complex128)
        g = self._g(spec.shape[0], f)
        fn = load().gd_spectogrd_f if f else load().gd_spectogrd
        self._chk(fn(self.h, spec.shape[0], _p(spec), _p(g)))
        return g

    def grdtospec(self, grid):
        f = self._single(grid)
        grid = np.ascontiguousarray(grid, np.float32 if f else np.float64).reshape(-1, self.nlat, self.nlon)
        s = np.zeros((grid.shape[0], self.nlm), np.complex64 if f else np.complex128)
        fn = load().gd_grdtospec_f if f else load().gd_grdtospec
        self._chk(fn(self.h, grid.shape[0], _p(grid), _p(s)))
        return s

    def getuv(self, vrt, div):
        f = self._single(vrt)
        ct = np.complex64 if f else np.complex128
        vrt = np.ascontiguousarray(np.atleast_2d(vrt), ct)
        div = np.ascontiguousarray(np.atleast_2d(div), ct)
        u, v = self._g(vrt.shape[0], f), self._g(vrt.shape[0], f)
        fn = load().gd_getuv_f if f else load().gd_getuv
        self._chk(fn(self.h, vrt.shape[0], _p(vrt), _p(div), _p(u), _p(v)))
        return u, v

    def getvrtdivspec(self, u, v):
        f = self._single(u)
        rt = np.float32 if f else np.float64
        u = np.ascontiguousarray(u, rt).reshape(-1, self.nlat, self.nlon)
        v = np.ascontiguousarray(v, rt).reshape(-1, self.nlat, self.nlon)
        vrt = np.zeros((u.shape[0], self.nlm), np.complex64 if f else np.complex128)
        div = np.zeros_like(vrt)
        fn = load().gd_getvrtdivspec_f if f else load().gd_getvrtdivspec
        self._chk(fn(self.h, u.shape[0], _p(u), _p(v), _p(vrt), _p(div)))
        return vrt, div

    def getgrad(self, spec):
        f = self._single(spec)
        spec = np.ascontiguousarray(np.atleast_2d(spec), np.complex64 if f else np.complex128)
        gx, gy = self._g(spec.shape[0], f), self._g(spec.shape[0], f)
        fn = load().gd_getgrad_f if f else load().gd_getgrad
        self._chk(fn(self.h, spec.shape[0], _p(spec), _p(gx), _p(gy)))
        return gx, gy

    def grid_info(self):
        lats, gw, aw = np.zeros(self.nlat), np.zeros(self.nlat), np.zeros(self.nlat)
        deg, order = np.zeros(self.nlm, np.int32), np.zeros(self.nlm, np.int32)
        lap, ilap = np.zeros(self.nlm), np.zeros(self.nlm)
        self._chk(load().gd_grid_info(self.h, _p(lats), _p(gw), _p(aw), _p(deg), _p(order),
                                      _p(lap), _p(ilap)))
        return dict(lats=lats, gauwts=gw, areawts=aw, degree=deg, order=order, lap=lap, invlap=ilap)

    def get_grid(self, name):
        L = self.nlev
        rows = dict(ug=L, vg=L, vrtg=L, divg=L, tvg=L, dlnpdtg=L, prs=L, etadot=L + 1,
                    trcg=max(self.ntrac, 1) * L, lnpsg=1, psg=1, dlnpsdt=1, dphisdx=1, dphisdy=1, sppt=1,
                    precip=1, apcp=1, pwat=1)
        out = np.zeros((rows[name], self.nlat, self.nlon))
        self._chk(load().gd_get_grid(self.h, name.encode(), _p(out)))
        return out

    def diag(self):
        o = np.zeros(5)
        self._chk(load().gd_diag(self.h, _p(o)))
        return dict(spdmax=o[0], psmin=o[1], psmax=o[2], pstend=o[3], pdryini=o[4])


class Pattern:
    """One stochastic pattern generator (gd_pattern): patterngenerator.f90's
    random_pattern with its own Mersenne-twister stream and nfields patterns."""

    def __init__(self, lscale, delt, tscale, stdev, iseed, jcap, nlon=0, nlat=0, normalization=None,
                 nfields=1, device=0):
        L = load()
        if normalization is None:
            normalization = 2.0 * float(np.float32(np.pi))  # stoch_data.f90: 2.*pi in r_kind
        h = ctypes.c_void_p()
        rc = L.gd_pattern_init(lscale, delt, tscale, stdev, iseed, nlon, nlat, jcap, normalization, nfields,
                               device, ctypes.byref(h))
        if rc != GD_OK:
            raise GdError(rc, L.gd_pattern_last_error(None).decode())
        self.h = h
        self.jcap, self.nfields = jcap, nfields
        self.nlm = (jcap + 1) * (jcap + 2) // 2

    def _chk(self, rc):
        if rc != GD_OK:
            raise GdError(rc, load().gd_pattern_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            load().gd_pattern_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def start(self):
        self._chk(load().gd_pattern_start(self.h))

    def advance(self, nsteps=1):
        self._chk(load().gd_pattern_advance(self.h, nsteps))

    def getnoise(self):
        out = np.zeros(self.nlm, np.complex128)
        self._chk(load().gd_pattern_getnoise(self.h, _p(out)))
        return out

    def get(self):
        out = np.zeros((self.nfields, self.nlm), np.complex128)
        self._chk(load().gd_pattern_get(self.h, _p(out)))
        return out

    def set(self, spec):
        a = np.ascontiguousarray(spec, np.complex128).reshape(self.nfields, self.nlm)
        self._chk(load().gd_pattern_set(self.h, _p(a)))

    def spectra(self):
        vs = np.zeros(self.nlm)
        v1 = np.zeros(self.jcap + 1)
        phi = np.zeros(1)
        self._chk(load().gd_pattern_spectra(self.h, _p(vs), _p(v1), _p(phi)))
        return vs, v1, float(phi[0])

    def set_stream(self, stream):
        self._chk(load().gd_pattern_set_stream(self.h, ctypes.c_void_p(stream)))

    def sync(self):
        self._chk(load().gd_pattern_sync(self.h))

    def launch_count(self):
        return load().gd_pattern_launch_count(self.h)


def ensemble_advance(members, nsteps=1):
    """gd_ensemble_advance: step all members, overlapping on the GPU."""
    arr = (ctypes.c_void_p * len(members))(*[m.h.value if hasattr(m.h, "value") else m.h for m in members])
    rc = load().gd_ensemble_advance(arr, len(members), 0.0, nsteps)
    if rc != GD_OK:
        raise GdError(rc, "gd_ensemble_advance failed: " + "; ".join(
            load().gd_last_error(m.h).decode() for m in members))


class Mlp:
    """The learned closure's network (gd_mlp): nin -> nhidden (GELU) x nlayers
    -> nout, BF16 weights with FP32 accumulation, trained by the library's own
    forward/backward kernels.  Batches are torch CUDA float32 tensors
    [ncols, nin] / [ncols, nout] on the net's device."""

    def __init__(self, nin, nhidden, nlayers, nout, seed=1, device=0):
        L = load()
        h = ctypes.c_void_p()
        rc = L.gd_mlp_init(nin, nhidden, nlayers, nout, seed, device, ctypes.byref(h))
        if rc != GD_OK:
            raise GdError(rc, L.gd_mlp_last_error(None).decode())
        self.h = h
        self.nin, self.nhidden, self.nlayers, self.nout, self.device = nin, nhidden, nlayers, nout, device
        n = ctypes.c_longlong()
        self._chk(L.gd_mlp_nparams(h, ctypes.byref(n)))
        self.nparams = n.value

    def _chk(self, rc):
        if rc != GD_OK:
            raise GdError(rc, load().gd_mlp_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            load().gd_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def layer_shapes(self):
        """(fout, fin) of each linear layer, in the packed parameter order."""
        sizes = [self.nin] + [self.nhidden] * self.nlayers + [self.nout]
        return [(sizes[i + 1], sizes[i]) for i in range(len(sizes) - 1)]

    def get_params(self):
        out = np.zeros(self.nparams, np.float32)
        self._chk(load().gd_mlp_get_params(self.h, _p(out)))
        return out

    def set_params(self, params):
        a = np.ascontiguousarray(params, np.float32)
        if a.size != self.nparams:
            raise ValueError("parameter count")
        self._chk(load().gd_mlp_set_params(self.h, _p(a)))

    def set_norm(self, in_mu, in_sd, out_mu, out_sd):
        arrs = [np.ascontiguousarray(x, np.float32) for x in (in_mu, in_sd, out_mu, out_sd)]
        self._norm = arrs
        self._chk(load().gd_mlp_set_norm(self.h, *[_p(x) for x in arrs]))

    def _batch(self, x, width, name):
        import torch

        if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.float32 and x.is_contiguous()
                and x.dim() == 2 and x.shape[1] == width and x.device.index == self.device):
            raise ValueError(f"{name}: a contiguous float32 CUDA tensor [ncols, {width}] on device {self.device}")
        return x

    def forward(self, x):
        import torch

        self._batch(x, self.nin, "x")
        y = torch.empty((x.shape[0], self.nout), dtype=torch.float32, device=x.device)
        self._chk(load().gd_mlp_forward(self.h, ctypes.c_void_p(x.data_ptr()), int(x.shape[0]),
                                        ctypes.c_void_p(y.data_ptr())))
        self.sync()
        return y

    def loss_grad(self, x, t):
        self._batch(x, self.nin, "x")
        self._batch(t, self.nout, "t")
        loss = np.zeros(1, np.float32)
        g = np.zeros(self.nparams, np.float32)
        self._chk(load().gd_mlp_loss_grad(self.h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(t.data_ptr()),
                                          int(x.shape[0]), _p(loss), _p(g)))
        return float(loss[0]), g

    def train_step(self, x, t, lr, want_loss=False):
        self._batch(x, self.nin, "x")
        self._batch(t, self.nout, "t")
        loss = np.zeros(1, np.float32)
        self._chk(load().gd_mlp_train_step(self.h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(t.data_ptr()),
                                           int(x.shape[0]), ctypes.c_float(lr), _p(loss) if want_loss else None))
        return float(loss[0]) if want_loss else None

    def sync(self):
        self._chk(load().gd_mlp_sync(self.h))
