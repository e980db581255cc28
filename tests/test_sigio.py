"""Sigma-file reader and writer (gd_sigio_*) against the oracle restatement of
src/sigio_module.f90 and dyn_init.f90's copyspecin / copyspecout.

Host-only entry points: no GPU is touched.  The reference ships no sample
sigma file (its dcmip_test/sanl.dat is a link to a file that is not in the
tree), so the format is pinned three ways: files the library writes are
byte-identical to the oracle's; the oracle's files read back field for
field; and a written 200509 file's own record-length table (lhead, ldata of
sigio_adhead) matches its record markers.
"""
import ctypes
import struct

import numpy as np
import pytest

import sigio_oracle as so
from gdpy import core, inputs, sigio
from helpers import renorm_float, sig_to_dict as to_dict


def rand_fields(jcap, levs, ntrac, seed):
    nlm = (jcap + 1) * (jcap + 2) // 2
    rng = np.random.default_rng(seed)
    c = lambda *s: rng.standard_normal(s) * 30 + 1j * rng.standard_normal(s) * 30
    return dict(vrt=c(levs, nlm), div=c(levs, nlm), tv=c(levs, nlm), trc=c(ntrac, levs, nlm), lnps=c(nlm),
                topo=c(nlm))


def make_head(jcap=12, levs=6, ntrac=2, ivs=200509, irealf=1, idvm=0, ixgr=0, lonb=40, latb=20):
    ak, bk = inputs.hybrid_coords(levs)
    h = sigio.hybrid_head(jcap, levs, ntrac, lonb, latb, ak, bk, irealf=irealf, fhour=6.0,
                          idate=(12, 7, 4, 2019), ivs=ivs)
    h.idvm, h.ixgr = idvm, ixgr
    if (idvm // 10) % 10 == 3:
        for i in range(ntrac + 1):
            h.cpi[i], h.ri[i] = 1000.0 + i, 287.0 + i
    if ivs != 200509:
        h.clabsig = b"LEGACY SIGMA FILE FROM UNIT TEST"
        h.pdryini = 98.25
    return h


CASES = [
    dict(ivs=200509, irealf=1),
    dict(ivs=200509, irealf=2),
    dict(ivs=200509, irealf=1, idvm=32),  # cpi and ri records
    dict(ivs=200509, irealf=1, ixgr=4),  # extra grid and scalar records
    dict(ivs=198410, irealf=1),
    dict(ivs=198410, irealf=2, ixgr=1),
]


# ------------------------------------------------------------------ tests
@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(f"{k}{v}" for k, v in c.items()))
def test_written_file_is_byte_identical_to_oracle(tmp_path, case):
    h = make_head(**case)
    f = rand_fields(h.jcap, h.levs, h.ntrac, seed=3)
    p = tmp_path / "s.sig"
    sigio.write(p, h, **f)
    d = to_dict(h)
    want = so.file_bytes(d, f, h.ntrac)
    got = p.read_bytes()
    assert len(got) == len(want)
    assert got == want


@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(f"{k}{v}" for k, v in c.items()))
def test_reader_matches_oracle_parse(tmp_path, case):
    h = make_head(**case)
    f = rand_fields(h.jcap, h.levs, h.ntrac, seed=4)
    p = tmp_path / "s.sig"
    p.write_bytes(so.file_bytes(to_dict(h), f, h.ntrac))
    oh, od, _ = so.read_file(p)
    g, out = sigio.read(p)
    gd = to_dict(g)
    for k in so.INT_FIELDS + ["ivs", "ncldt", "ixgr", "nxgr", "nxss", "nhead", "ndata"]:
        assert gd[k] == oh[k], k
    for k in ("fhour", "pdryini"):
        assert np.float32(gd[k]) == np.float32(oh[k]), k
    assert gd["idate"] == list(oh["idate"])
    assert gd["clabsig"] == oh["clabsig"]
    np.testing.assert_array_equal(gd["vcoord"], oh["vcoord"])
    for k in ("si", "sl", "ak", "bk"):
        np.testing.assert_array_equal(gd[k], oh[k])
    assert gd["cfvars"] == list(oh["cfvars"])
    if so.thermo3(oh):
        np.testing.assert_array_equal(gd["cpi"], oh["cpi"])
        np.testing.assert_array_equal(gd["ri"], oh["ri"])
    for k in ("vrt", "div", "tv", "trc", "lnps", "topo"):
        np.testing.assert_array_equal(out[k], od[k], err_msg=k)
        np.testing.assert_array_equal(out[k], renorm_float(f[k]), err_msg=k)


def test_record_length_table_describes_the_file(tmp_path):
    h = make_head(ivs=200509, irealf=2, idvm=32, ixgr=5)
    p = tmp_path / "s.sig"
    sigio.write(p, h, **rand_fields(h.jcap, h.levs, h.ntrac, 5))
    recs = so.unpack_records(p.read_bytes())
    ivs, nhead, ndata = struct.unpack_from(">3i", recs[0], 8)
    assert (ivs, nhead, ndata) == (200509, 7, h.ndata)
    table = struct.unpack(f">{nhead + ndata}i", recs[1])
    lhead, ldata = table[:nhead], table[nhead:]
    assert [len(r) for r in recs[:nhead]] == list(lhead)
    assert [len(r) for r in recs[nhead:]] == list(ldata)
    assert len(recs) == nhead + ndata


def test_modern_header_as_the_reference_reads_it(tmp_path):
    h = make_head()
    h.pdryini = 98.0
    p = tmp_path / "s.sig"
    sigio.write(p, h, **rand_fields(h.jcap, h.levs, h.ntrac, 6))
    g = sigio.read_head(p)
    # sigio_srhead replaces these after reading a 200509 header
    assert g.pdryini == so.FILL
    assert g.label == b" " * 32
    assert all(v == so.FILL for v in g.si) and all(v == so.FILL for v in g.bk)
    np.testing.assert_array_equal(g.vcoord_array, h.vcoord_array)


def test_legacy_header_words_truncate_and_ntrac_is_at_least_one(tmp_path):
    d = so.default_head()
    d.update(ivs=198410, clabsig=b"X" * 32, fhour=3.0, idate=[0, 1, 2, 2000], jcap=10, levs=4, itrun=1,
             iorder=2, irealf=1, igen=0, latf=16, lonf=32, latb=16, lonb=32, latr=16, lonr=32, ntrac=0,
             nvcoord=2, icen2=0, iens0=0, iens1=0, idpp=0, idsl=0, idvc=2, idvm=0, idvt=0, idrun=0, idusr=0,
             pdryini=97.5, ncldt=0, ixgr=0)
    ak, bk = inputs.hybrid_coords(4)
    d["vcoord"] = np.stack([ak[::-1], bk[::-1]]).astype(np.float32)
    d["vcoord"][1, 0] = 1.0
    recs = so.head_records(d)
    r2 = bytearray(recs[1])
    struct.pack_into(">f", r2, 20 + 4 * 201 + 4 * 2, 1.7)  # itrun written as 1.7
    recs[1] = bytes(r2)
    data = so.data_records(d, {}, 0)
    p = tmp_path / "s.sig"
    p.write_bytes(so.pack_records(recs + data))
    g = sigio.read_head(p)
    assert g.itrun == 1 and g.ntrac == 1 and g.ivs == 198410
    assert g.pdryini == np.float32(97.5)
    np.testing.assert_array_equal(np.ctypeslib.as_array(g.ak)[:5], d["vcoord"][0])
    np.testing.assert_array_equal(np.ctypeslib.as_array(g.bk)[:5], d["vcoord"][1])


def test_legacy_sigma_header_layer_values(tmp_path):
    """A 198410 sigma header whose vcoord(1,1) is 1 gets its layer values
    from sigio_modpr: Phillips layers (idsl 1) and mean layers (idsl 2)."""
    L = 8
    si = np.linspace(1.0, 0.0, L + 1).astype(np.float32) ** 1.5
    for idsl in (1, 2):
        h = sigio.head_init()
        h.ivs, h.jcap, h.levs, h.ntrac, h.irealf, h.idvc, h.idsl, h.ixgr = 198410, 5, L, 1, 1, 1, idsl, 0
        h.lonb, h.latb, h.idvm, h.fhour = 16, 8, 0, 0.0
        h.set_vcoord(si[None, :])
        p = tmp_path / f"s{idsl}.sig"
        sigio.write(p, h)
        recs = so.unpack_records(p.read_bytes())
        sl = np.frombuffer(recs[1], ">f4", L, 20 + 4 * (L + 1)).astype(np.float64)
        np.testing.assert_array_equal(sl.astype(np.float32), so.modpr_layers(si, L, idsl)[0])
        s0, s1 = si[:-1].astype(np.float64), si[1:].astype(np.float64)
        if idsl == 1:
            kap = 287.05 / 1004.6
            ref = ((s0 ** (kap + 1) - s1 ** (kap + 1)) / ((kap + 1) * (s0 - s1))) ** (1 / kap)
        else:
            ref = (s0 + s1) / 2
        np.testing.assert_allclose(sl, ref, rtol=2e-6)


def test_round_trip_is_float_rounding(tmp_path):
    h = make_head(irealf=2)
    f = rand_fields(h.jcap, h.levs, h.ntrac, 8)
    p = tmp_path / "a.sig"
    sigio.write(p, h, **f)
    g, out = sigio.read(p)
    for k in f:
        np.testing.assert_array_equal(out[k], renorm_float(f[k]))
    q = tmp_path / "b.sig"
    sigio.write(q, g, **{k: out[k] for k in f})
    assert so.unpack_records(q.read_bytes())[5:] == so.unpack_records(p.read_bytes())[5:]


def test_tracer_subset_and_missing_tracers(tmp_path):
    h = make_head(ntrac=3)
    f = rand_fields(h.jcap, h.levs, 3, 9)
    p = tmp_path / "s.sig"
    sigio.write(p, h, **f)
    _, out = sigio.read(p, ntrac=1)
    np.testing.assert_array_equal(out["trc"], renorm_float(f["trc"][:1]))
    # only one tracer given: the other tracer records are zeros
    f1 = dict(f, trc=f["trc"][:1])
    sigio.write(p, h, **f1)
    _, out = sigio.read(p)
    np.testing.assert_array_equal(out["trc"][0], renorm_float(f["trc"][0]))
    assert not out["trc"][1:].any()


def test_null_outputs_are_skipped(tmp_path):
    h = make_head()
    f = rand_fields(h.jcap, h.levs, h.ntrac, 10)
    p = tmp_path / "s.sig"
    sigio.write(p, h, **f)
    lnps = np.zeros((h.jcap + 1) * (h.jcap + 2) // 2, np.complex128)
    g = sigio.SigHead()
    L = core.load()
    rc = L.gd_sigio_read(str(p).encode(), h.jcap, h.levs, h.ntrac, ctypes.byref(g), None, None, None, None,
                         lnps.ctypes.data_as(ctypes.c_void_p), None)
    assert rc == core.GD_OK
    np.testing.assert_array_equal(lnps, renorm_float(f["lnps"]))


def test_config_from_header():
    L = 10
    ak, bk = inputs.hybrid_coords(L)
    h = sigio.hybrid_head(20, L, 1, 64, 32, ak, bk)
    cfg, a, b = sigio.config(h, dt=900.0)
    assert (cfg.ntrunc, cfg.nlon, cfg.nlat, cfg.nlev, cfg.dt) == (20, 64, 32, L, 900.0)
    np.testing.assert_array_equal(a, ak.astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(b, bk.astype(np.float32).astype(np.float64))
    for cb, pa in [(98.25, float(np.float32(98.25) * np.float32(1000.0))), (101.0, 0.0), (so.FILL, 0.0)]:
        h.pdryini = cb
        assert sigio.config(h)[0].pdryini == pa
    h.idvc = 1
    with pytest.raises(core.GdError) as e:
        sigio.config(h)
    assert e.value.code == core.GD_ERR_UNSUPPORTED


def _status(fn, *a):
    return getattr(core.load(), fn)(*a)


def test_errors_are_status_codes(tmp_path):
    h = make_head()
    p = tmp_path / "s.sig"
    sigio.write(p, h, **rand_fields(h.jcap, h.levs, h.ntrac, 11))
    good = p.read_bytes()
    with pytest.raises(core.GdError) as e:
        sigio.read_head(tmp_path / "missing.sig")
    assert e.value.code == core.GD_ERR_IO and "cannot open" in str(e.value)
    for bad in (good[:-100], good[:-1] + b"\x01", good[:12] + b"\x00\x03\x0f\x4a" + good[16:]):
        q = tmp_path / "bad.sig"
        q.write_bytes(bad)
        with pytest.raises(core.GdError) as e:
            sigio.read(q, h.jcap, h.levs, h.ntrac)
        assert e.value.code == core.GD_ERR_IO
    with pytest.raises(core.GdError) as e:
        sigio.read(p, h.jcap + 1, h.levs, h.ntrac)
    assert e.value.code == core.GD_ERR_ARG
    with pytest.raises(core.GdError) as e:
        sigio.read(p, h.jcap, h.levs, h.ntrac + 1)
    assert e.value.code == core.GD_ERR_ARG
    big = make_head()
    big.levs = sigio.MAXLEVS + 1
    with pytest.raises(core.GdError) as e:
        sigio.write(tmp_path / "x.sig", big)
    assert e.value.code == core.GD_ERR_UNSUPPORTED
    with pytest.raises(core.GdError) as e:
        f = rand_fields(h.jcap, h.levs, h.ntrac + 1, 12)
        sigio.write(tmp_path / "x.sig", h, **f)
    assert e.value.code == core.GD_ERR_ARG
    assert _status("gd_sigio_read_head", None, None) == core.GD_ERR_ARG
    assert _status("gd_read_sig", None, str(p).encode(), None) == core.GD_ERR_ARG
    assert _status("gd_write_sig", None, str(p).encode(), 0.0, None) == core.GD_ERR_ARG


def test_header_struct_defaults():
    h = sigio.head_init()
    assert h.jcap == -9999 and h.fhour == so.FILL and h.nvcoord == -9999
    assert h.label == b" " * 32
    assert ctypes.sizeof(sigio.SigHead) == 32 + 4 * (1 + 4 + 403 + 12 + 11 + 1 + 4 + 3 * 257) + 8 * 105 + 4 * (4 + 202)
