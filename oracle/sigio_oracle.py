"""Sigma-file oracle -- TEST INFRASTRUCTURE ONLY.

A pure-Python restatement of the GFS sigma-file format as
src/sigio_module.f90 reads and writes it, and of the spectral
renormalisation of readin_sig / wrtout_sig (src/dyn_init.f90:93-191).  Only
tests use it, to check the library's reader and writer byte for byte.

- Records: Fortran unformatted sequential, big-endian, a 4-byte length
  before and after each payload (convert='big_endian' in sigio_sropen /
  sigio_swopen, sigio_module.f90:430-456).
- Header 200509 (sigio_swhead, :585-610; sigio_srhead, :478-506): label
  'GFS SIG ' + ivs, nhead, ndata, 0, 0, 0; lhead(nhead) + ldata(ndata);
  50 words fhour..ixgr + 18 zeros; vcoord; cfvars; cpi and ri when
  mod(idvm/10,10) == 3.  After reading, si, sl, ak, bk and pdryini are the
  fill value (:501-506).
- Header 198410 (:507-570 read, :612-673 write): the 32-byte ON85 label and
  fhour, idate(4), sisl(201), ext(44); ext words map to the integer fields
  by truncation (ntrac at least 1); sisl holds si/sl or ak/bk by idvc.
- sigio_adhead (:1323-1382): nxgr/nxss by ixgr, nhead, ndata, lhead, ldata.
- Data (sigio_srdata / sigio_swdata, :755-915): hs, ps, t(levs),
  (d, z)(levs), q(ntrac, levs), xgr(nxgr), xss; 4-byte words unless
  irealf == 2, values carried in single precision.
- copyspecin / copyspecout (dyn_init.f90:93-118): times / divided by
  sqrt(2 pi) with the reference's single-rounded con_pi.
- sigio_modpr (:1207-1321) layer values at ps = 1 for the 198410 writer.

Headers are plain dicts; vcoord is float32[nvcoord, levs+1].
"""
import math
import struct

import numpy as np

FILL = float(np.float32(-9999.0))
IFILL = -9999
PI_REF = float(np.float32(3.1415926535897931))
RENORM = math.sqrt(2.0 * PI_REF)
F32 = np.float32

INT_FIELDS = ["jcap", "levs", "itrun", "iorder", "irealf", "igen", "latf", "lonf", "latb", "lonb", "latr",
              "lonr", "ntrac", "nvcoord", "icen2", "iens0", "iens1", "idpp", "idsl", "idvc", "idvm", "idvt",
              "idrun", "idusr"]


def default_head():
    """type sigio_head's default initialisation (sigio_module.f90:337-379)."""
    h = dict(clabsig=b" " * 32, fhour=FILL, idate=[IFILL] * 4, si=np.full(101, FILL, F32),
             sl=np.full(100, FILL, F32), ak=np.full(101, FILL, F32), bk=np.full(101, FILL, F32),
             pdryini=FILL, ncldt=IFILL, ixgr=IFILL, ivs=IFILL, vcoord=np.zeros((0, 0), F32), cfvars=[],
             nxgr=IFILL, nxss=IFILL, nhead=IFILL, ndata=IFILL, cpi=None, ri=None)
    for k in INT_FIELDS:
        h[k] = IFILL
    return h


# ----------------------------------------------------------------- records
def pack_records(recs):
    out = bytearray()
    for r in recs:
        n = struct.pack(">i", len(r))
        out += n + bytes(r) + n
    return bytes(out)


def unpack_records(buf):
    recs, i = [], 0
    while i < len(buf):
        (n,) = struct.unpack_from(">i", buf, i)
        assert n >= 0 and i + 8 + n <= len(buf), "bad record marker"
        recs.append(bytes(buf[i + 4:i + 4 + n]))
        (m,) = struct.unpack_from(">i", buf, i + 4 + n)
        assert m == n, "trailing marker differs"
        i += 8 + n
    return recs


def thermo3(h):
    q = abs(h["idvm"]) // 10 % 10  # mod(idvm/10,10): only the value 3 matters
    return h["idvm"] >= 0 and q == 3


def adhead(h):
    """Sets nxgr, nxss, nhead, ndata; returns (lhead, ldata)."""
    L = h["levs"]
    nxgr, nxss = {1: (2 * L + 1, 0), 2: (4 * L + 3, 0), 3: (3 * L + 1, 0), 4: (4 * L + 3, 1),
                  5: (3 * L + 1, 1)}.get(h["ixgr"], (0, 0))
    h["nxgr"], h["nxss"] = nxgr, nxss
    nspec = 2 + (3 + h["ntrac"]) * L
    nc = (h["jcap"] + 1) * (h["jcap"] + 2)
    lspec = 4 * h["irealf"] * nc
    lgrid = 4 * h["irealf"] * h["lonb"] * h["latb"]
    if h["ivs"] == 200509:
        h["nhead"] = 7 if thermo3(h) else 5
        h["ndata"] = nspec + nxgr + (1 if nxss > 0 else 0)
        lhead = [32, 4 * (h["nhead"] + h["ndata"]), 200, 4 * (L + 1) * h["nvcoord"], 8 * (5 + h["ntrac"])]
        if thermo3(h):
            lhead += [4 * (h["ntrac"] + 1)] * 2
        ldata = [lspec] * nspec + [lgrid] * nxgr + [4 * h["irealf"] * nxss] * (h["ndata"] - nspec - nxgr)
    else:
        h["nhead"], h["ndata"] = 2, nspec + nxgr
        lhead = [32, 1000]
        ldata = [lspec] * nspec + [lgrid] * nxgr
    return lhead, ldata


# ------------------------------------------------------------------ header
def modpr_layers(si, levs, idsl):
    """sigio_modpr's pm at ps = 1 for sigma interfaces si[0..levs]."""
    id2 = 1 if idsl in (0, 1) else 2 if idsl == 2 else 0
    pm = np.zeros(levs, F32)
    if id2 == 0:
        return pm, False
    rocp = float(F32(287.05) / F32(1004.6))
    rocpr = 1 / rocp
    pid = 1.0
    pidk = pid ** rocp if id2 == 1 else 0.0
    for k in range(levs):
        piu = float(F32(si[k + 1]) * F32(1.0))
        piuk = 0.0
        if id2 == 1:
            piuk = piu ** rocp
            pmk = (pid * pidk - piu * piuk) / ((rocp + 1) * (pid - piu))
            pmm = pmk ** rocpr
        else:
            pmm = (pid + piu) / 2
        pm[k] = F32(pmm)
        pid, pidk = piu, piuk
    return pm, True


def head_records(h):
    """sigio_swhead's records for header h (h gets nxgr.. set)."""
    lhead, ldata = adhead(h)
    if h["ivs"] >= 200509:
        r1 = b"GFS SIG " + struct.pack(">6i", h["ivs"], h["nhead"], h["ndata"], 0, 0, 0)
        r2 = struct.pack(f">{len(lhead) + len(ldata)}i", *lhead, *ldata)
        ints = [h[k] for k in INT_FIELDS]
        r3 = (struct.pack(">f4i", h["fhour"], *h["idate"]) + struct.pack(">24i", *ints) +
              struct.pack(">f2i", h["pdryini"], h["ncldt"], h["ixgr"]) + struct.pack(">18i", *[0] * 18))
        v = np.asarray(h["vcoord"], F32)
        rv = v.astype(">f4").tobytes()  # row j = vcoord(:, j+1): Fortran column order
        rc = b"".join(c.ljust(8)[:8] for c in h["cfvars"])
        recs = [r1, r2, r3, rv, rc]
        if thermo3(h):
            recs += [np.asarray(h["cpi"], ">f4").tobytes(), np.asarray(h["ri"], ">f4").tobytes()]
        return recs
    L = h["levs"]
    sisl = np.zeros(201, F32)
    v = np.asarray(h["vcoord"], F32)
    if h["idvc"] in (0, 1):
        if h["nvcoord"] == 1 and v[0, 0] == 1.0:
            sisl[:L + 1] = v[0, :L + 1]
            sisl[L + 1:2 * L + 1] = modpr_layers(v[0], L, h["idsl"])[0]
        else:
            sisl[:L + 1] = h["si"][:L + 1]
            sisl[L + 1:2 * L + 1] = h["sl"][:L]
    elif h["idvc"] in (2, 3):
        if h["nvcoord"] == 2 and v[1, 0] == 1.0:
            sisl[:L + 1], sisl[L + 1:2 * L + 2] = v[0, :L + 1], v[1, :L + 1]
        elif h["idvc"] == 2:
            sisl[:L + 1], sisl[L + 1:2 * L + 2] = h["ak"][:L + 1], h["bk"][:L + 1]
    ext = np.zeros(44, F32)
    order = ["jcap", "levs", "itrun", "iorder", "irealf", "igen", "lonf", "latf", "lonb", "latb", "lonr",
             "latr", "ntrac", "icen2", "iens0", "iens1", "idpp", "idsl", "idvc", "idvm", "idvt", "idrun",
             "idusr"]
    ext[:23] = [h[k] for k in order]
    ext[23], ext[24], ext[25] = h["pdryini"], h["ncldt"], h["ixgr"]
    r2 = struct.pack(">f4i", h["fhour"], *h["idate"]) + sisl.astype(">f4").tobytes() + ext.astype(">f4").tobytes()
    return [h["clabsig"].ljust(32)[:32], r2]


def parse_head(recs):
    """sigio_srhead: (header, number of header records)."""
    h = default_head()
    r1 = recs[0]
    if r1[:8] == b"GFS SIG ":
        (h["ivs"],) = struct.unpack_from(">i", r1, 8)
        assert h["ivs"] == 200509
        r3 = recs[2]
        h["fhour"], *idate = struct.unpack_from(">f4i", r3, 0)
        h["idate"] = idate
        for i, k in enumerate(INT_FIELDS):
            (h[k],) = struct.unpack_from(">i", r3, 20 + 4 * i)
        h["pdryini"], h["ncldt"], h["ixgr"] = struct.unpack_from(">f2i", r3, 20 + 4 * 24)
        L, nv = h["levs"], h["nvcoord"]
        h["vcoord"] = np.frombuffer(recs[3], ">f4", nv * (L + 1)).astype(F32).reshape(nv, L + 1)
        h["cfvars"] = [recs[4][8 * i:8 * i + 8] for i in range(5 + h["ntrac"])]
        n = 5
        if thermo3(h):
            h["cpi"] = np.frombuffer(recs[5], ">f4", h["ntrac"] + 1).astype(F32)
            h["ri"] = np.frombuffer(recs[6], ">f4", h["ntrac"] + 1).astype(F32)
            n = 7
        h["clabsig"] = b" " * 32
        for k in ("si", "sl", "ak", "bk"):
            h[k] = np.full_like(h[k], FILL)
        h["pdryini"] = FILL
    else:
        h["clabsig"] = r1[:32]
        r2 = recs[1]
        h["fhour"], *idate = struct.unpack_from(">f4i", r2, 0)
        h["idate"] = idate
        sisl = np.frombuffer(r2, ">f4", 201, 20).astype(F32)
        ext = np.frombuffer(r2, ">f4", 44, 20 + 4 * 201).astype(F32)
        order = ["jcap", "levs", "itrun", "iorder", "irealf", "igen", "lonf", "latf", "lonb", "latb", "lonr",
                 "latr"]
        for i, k in enumerate(order):
            h[k] = int(ext[i])
        h["ntrac"] = int(max(ext[12], F32(1)))
        h["icen2"], h["iens0"], h["iens1"] = int(ext[13]), int(ext[14]), int(ext[15])
        for i, k in enumerate(["idpp", "idsl", "idvc", "idvm", "idvt", "idrun", "idusr"]):
            h[k] = int(ext[16 + i])
        h["pdryini"] = float(ext[23])
        h["ncldt"], h["ixgr"] = int(ext[24]), int(ext[25])
        L = h["levs"]
        if h["idvc"] in (0, 1):
            h["si"][:L + 1] = sisl[:L + 1]
            h["sl"][:L] = sisl[L + 1:2 * L + 1]
            h["nvcoord"] = 1
            h["vcoord"] = sisl[None, :L + 1].copy()
        elif h["idvc"] in (2, 3):
            if h["idvc"] == 2:
                h["ak"][:L + 1] = sisl[:L + 1]
                h["bk"][:L + 1] = sisl[L + 1:2 * L + 2]
            h["nvcoord"] = 2
            h["vcoord"] = np.stack([sisl[:L + 1], sisl[L + 1:2 * L + 2]])
        h["cfvars"] = [b" " * 8] * (5 + h["ntrac"])
        h["ivs"] = 198410
        n = 2
    adhead(h)
    return h, n


# -------------------------------------------------------------------- data
def spec_out(c, dbl):
    """copyspecout of complex coefficients into one record's bytes."""
    c = np.asarray(c, np.complex128)
    r = np.empty(2 * c.size, np.float64)
    r[0::2], r[1::2] = c.real, c.imag
    v = (r / RENORM).astype(F32)
    return v.astype(">f8").tobytes() if dbl else v.astype(">f4").tobytes()


def spec_in(rec, nc, dbl):
    """One record, as sigio_srdata hands it on (float), times sqrt(2 pi)."""
    v = np.frombuffer(rec, ">f8" if dbl else ">f4", nc).astype(F32).astype(np.float64) * RENORM
    return v[0::2] + 1j * v[1::2]


def data_records(h, fields, ntrac):
    """sigio_swdata's records of the model fields (zeros where absent)."""
    L = h["levs"]
    nlm = (h["jcap"] + 1) * (h["jcap"] + 2) // 2
    dbl = h["irealf"] == 2
    z = np.zeros(nlm, np.complex128)
    g = lambda k, *ix: fields[k][ix] if fields.get(k) is not None else z
    recs = [spec_out(g("topo"), dbl), spec_out(g("lnps"), dbl)]
    recs += [spec_out(g("tv", k), dbl) for k in range(L)]
    for k in range(L):
        recs += [spec_out(g("div", k), dbl), spec_out(g("vrt", k), dbl)]
    for n in range(h["ntrac"]):
        for k in range(L):
            recs.append(spec_out(fields["trc"][n, k] if n < ntrac else z, dbl))
    w = 8 if dbl else 4
    recs += [bytes(w * h["lonb"] * h["latb"])] * h["nxgr"]
    if h["nxss"] > 0:
        recs.append(bytes(w * h["nxss"]))
    return recs


def parse_data(h, recs, ntrac=None):
    """sigio_srdata + copyspecin of the data records."""
    L = h["levs"]
    nc = (h["jcap"] + 1) * (h["jcap"] + 2)
    dbl = h["irealf"] == 2
    ntrac = h["ntrac"] if ntrac is None else ntrac
    it = iter(recs)
    out = dict(topo=spec_in(next(it), nc, dbl), lnps=spec_in(next(it), nc, dbl))
    out["tv"] = np.array([spec_in(next(it), nc, dbl) for _ in range(L)])
    d, z = [], []
    for _ in range(L):
        d.append(spec_in(next(it), nc, dbl))
        z.append(spec_in(next(it), nc, dbl))
    out["div"], out["vrt"] = np.array(d), np.array(z)
    q = [[spec_in(next(it), nc, dbl) for _ in range(L)] for _ in range(h["ntrac"])]
    out["trc"] = np.array(q[:ntrac]).reshape(ntrac, L, nc // 2)
    out["extra"] = list(it)
    return out


def file_bytes(h, fields, ntrac):
    return pack_records(head_records(h) + data_records(h, fields, ntrac))


def read_file(path):
    recs = unpack_records(open(path, "rb").read())
    h, n = parse_head(recs)
    return h, parse_data(h, recs[n:]), recs
