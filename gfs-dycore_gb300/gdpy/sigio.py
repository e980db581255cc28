"""GFS sigma files through libgdcore.so (gd_sigio_* / gd_read_sig / gd_write_sig).

``SigHead`` is the C ``gd_sighead`` (the reference's ``type sigio_head``,
src/sigio_module.f90:337-379).  ``read_head`` / ``read`` / ``write`` mirror
sigio_srhead, readin_sig and wrtout_sig's copyspecout + sigio_swohdc
(src/dyn_init.f90:93-191); ``config`` is the header-to-model mapping of
src/params.f90:250-264 and src/dyn_init.f90:52-66.  Spectral arrays are
``complex128``: ``[levs, nlm]`` for vrt/div/tv, ``[ntrac, levs, nlm]`` for
tracers, ``[nlm]`` for ln(ps) (in cb, as stored in the file) and orography.
"""
import ctypes

import numpy as np

from . import core

MAXLEVS = 256
MAXTRAC = 100
FILL = -9999.0
_f, _i, _c = ctypes.c_float, ctypes.c_int, ctypes.c_char


class SigHead(ctypes.Structure):
    _fields_ = [
        ("clabsig", _c * 32), ("fhour", _f), ("idate", _i * 4),
        ("si", _f * 101), ("sl", _f * 100), ("ak", _f * 101), ("bk", _f * 101),
        *[(n, _i) for n in ("jcap", "levs", "itrun", "iorder", "irealf", "igen", "latf", "lonf", "latb",
                            "lonb", "latr", "lonr", "ntrac", "icen2")],
        ("iens", _i * 2),
        *[(n, _i) for n in ("idpp", "idsl", "idvc", "idvm", "idvt", "idrun", "idusr")],
        ("pdryini", _f),
        *[(n, _i) for n in ("ncldt", "ixgr", "ivs", "nvcoord")],
        ("vcoord", (_f * (MAXLEVS + 1)) * 3),
        ("cfvars", (_c * 8) * (5 + MAXTRAC)),
        *[(n, _i) for n in ("nxgr", "nxss", "nhead", "ndata")],
        ("cpi", _f * (MAXTRAC + 1)), ("ri", _f * (MAXTRAC + 1)),
    ]

    @property
    def vcoord_array(self):
        """vcoord(levs+1, nvcoord) of the Fortran header as float32[nvcoord, levs+1]."""
        v = np.ctypeslib.as_array(self.vcoord)
        return v[: max(self.nvcoord, 0), : self.levs + 1].copy()

    def set_vcoord(self, v):
        v = np.asarray(v, np.float32)
        self.nvcoord = v.shape[0]
        for j in range(v.shape[0]):
            for k in range(v.shape[1]):
                self.vcoord[j][k] = float(v[j, k])

    @property
    def label(self):
        """clabsig as its 32 raw bytes."""
        return ctypes.string_at(ctypes.addressof(self) + SigHead.clabsig.offset, 32)

    @property
    def cfvar_names(self):
        """The 5+ntrac cfvars entries as 8-byte strings."""
        base = ctypes.addressof(self) + SigHead.cfvars.offset
        return [ctypes.string_at(base + 8 * i, 8) for i in range(5 + max(self.ntrac, 0))]

    def set_cfvars(self, names):
        base = ctypes.addressof(self) + SigHead.cfvars.offset
        for i, n in enumerate(names):
            b = n.encode() if isinstance(n, str) else bytes(n)
            ctypes.memmove(base + 8 * i, b.ljust(8)[:8], 8)


def _err():
    return core.load().gd_sigio_last_error().decode()


def _check(rc):
    if rc != core.GD_OK:
        raise core.GdError(rc, _err())


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def head_init():
    """The default-initialised sigio_head (fill values, blank labels)."""
    h = SigHead()
    _check(core.load().gd_sigio_head_init(ctypes.byref(h)))
    return h


def read_head(path):
    h = SigHead()
    _check(core.load().gd_sigio_read_head(str(path).encode(), ctypes.byref(h)))
    return h


def read(path, jcap=None, levs=None, ntrac=None):
    """readin_sig: header and renormalised spectral fields.  Sizes default to
    the file's own."""
    if jcap is None or levs is None or ntrac is None:
        h0 = read_head(path)
        jcap = h0.jcap if jcap is None else jcap
        levs = h0.levs if levs is None else levs
        ntrac = h0.ntrac if ntrac is None else ntrac
    nlm = (jcap + 1) * (jcap + 2) // 2
    out = dict(vrt=np.zeros((levs, nlm), np.complex128), div=np.zeros((levs, nlm), np.complex128),
               tv=np.zeros((levs, nlm), np.complex128), trc=np.zeros((ntrac, levs, nlm), np.complex128),
               lnps=np.zeros(nlm, np.complex128), topo=np.zeros(nlm, np.complex128))
    h = SigHead()
    _check(core.load().gd_sigio_read(str(path).encode(), jcap, levs, ntrac, ctypes.byref(h), _p(out["vrt"]),
                                     _p(out["div"]), _p(out["tv"]), _p(out["trc"]) if ntrac else None,
                                     _p(out["lnps"]), _p(out["topo"])))
    return h, out


def _c128(a, shape):
    if a is None:
        return None
    a = np.ascontiguousarray(a, np.complex128)
    if a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


def write(path, head, vrt=None, div=None, tv=None, trc=None, lnps=None, topo=None):
    """copyspecout + sigio_swohdc.  head is updated (nxgr, nxss, nhead, ndata)."""
    L, nlm = head.levs, (head.jcap + 1) * (head.jcap + 2) // 2
    ntrac = 0 if trc is None else np.asarray(trc).shape[0]
    arrs = [_c128(vrt, (L, nlm)), _c128(div, (L, nlm)), _c128(tv, (L, nlm)),
            _c128(trc, (ntrac, L, nlm)) if ntrac else None, _c128(lnps, (nlm,)), _c128(topo, (nlm,))]
    _check(core.load().gd_sigio_write(str(path).encode(), ctypes.byref(head), ntrac, *[_p(a) for a in arrs]))


def config(head, **kw):
    """(GdConfig, ak, bk) for a model run on the file's grid; kw overrides
    other config fields (dt, precision, ntrac ...)."""
    cfg = core.default_config(**kw)
    ak = np.zeros(head.levs + 1)
    bk = np.zeros(head.levs + 1)
    _check(core.load().gd_sigio_config(ctypes.byref(head), ctypes.byref(cfg), _p(ak), _p(bk)))
    return cfg, ak, bk


def hybrid_head(jcap, levs, ntrac, lonb, latb, ak, bk, irealf=1, fhour=0.0, idate=(0, 1, 1, 2000), ivs=200509):
    """A header for a hybrid-coordinate model state that did not come from a
    file (the reference always writes the header it read).  ak, bk [levs+1]
    top to bottom as gd_init takes them; the file holds them bottom to top."""
    h = head_init()
    h.ivs, h.fhour, h.jcap, h.levs, h.ntrac, h.irealf = ivs, fhour, jcap, levs, ntrac, irealf
    for i, v in enumerate(idate):
        h.idate[i] = v
    h.itrun, h.iorder, h.igen = 1, 2, 0
    h.latf = h.latb = h.latr = latb
    h.lonf = h.lonb = h.lonr = lonb
    h.icen2, h.iens[0], h.iens[1] = 0, 0, 0
    h.idpp, h.idsl, h.idvc, h.idvm, h.idvt, h.idrun, h.idusr = 0, 0, 2, 0, 21, 0, 0
    h.pdryini, h.ncldt, h.ixgr = 0.0, 0, 0
    h.set_vcoord(np.stack([np.asarray(ak, np.float64)[::-1], np.asarray(bk, np.float64)[::-1]]))
    h.set_cfvars(["hs", "ps", "t", "d", "z"] + [f"q{n + 1}" for n in range(ntrac)])
    return h


def read_into(dycore, path):
    """gd_read_sig: load path into a Dycore (ln ps to Pa, orography set)."""
    h = SigHead()
    L = core.load()
    rc = L.gd_read_sig(dycore.h, str(path).encode(), ctypes.byref(h))
    if rc != core.GD_OK:
        raise core.GdError(rc, L.gd_last_error(dycore.h).decode())
    return h


def write_from(dycore, path, fhour, head):
    """gd_write_sig: the Dycore's state to path with head (fhour, pdryini set)."""
    L = core.load()
    rc = L.gd_write_sig(dycore.h, str(path).encode(), ctypes.c_double(fhour), ctypes.byref(head))
    if rc != core.GD_OK:
        raise core.GdError(rc, L.gd_last_error(dycore.h).decode())
