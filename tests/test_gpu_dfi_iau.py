"""Digital filter initialisation (gd_dfi) and the incremental analysis update
(gd_set_iau, gd_set_iau_files) on the GPU against the FP64 oracle.

Tolerances: FP64 states 1e-9 (divergence against the vorticity scale), the
same bar as the other multi-step FP64 checks; the file path of IAU against
the array path bit for bit (same increments); IAU outside its window
bit for bit against no IAU (the forcing adds zeros).
"""
import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu


def rel_div(a, b):
    return float(np.abs(a["div"] - b["div"]).max() / np.abs(b["vrt"]).max())


def pair(oracle_mod, T=42, L=20, ntrac=1, dt=600.0, precision="fp64", seed=4):
    from gdpy import core, inputs

    ak, bk = inputs.hybrid_coords(L)
    g = core.Dycore(T, 128, 64, L, ak, bk, ntrac=ntrac, dt=dt, precision=precision)
    o = oracle_mod.Oracle(T, 128, 64, L, ak, bk, ntrac=ntrac, dt=dt)
    st = inputs.smooth_random_state(T, L, ntrac=ntrac, seed=seed)
    for m in (g, o):
        m.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=st["trc"])
    return g, o, st


def increments(g, nf, seed=9, amp=1e-3):
    rng = np.random.default_rng(seed)
    L, n, nt = g.nlev, g.nlm, g.ntrac
    from gdpy import inputs

    deg, order = inputs.degree_order(g.ntrunc)
    damp = 1.0 / (1.0 + deg) ** 2

    def c(*s):
        x = (rng.standard_normal(s) + 1j * rng.standard_normal(s)) * damp
        x[..., order == 0] = x[..., order == 0].real
        return x

    return dict(vrt=1e-6 * amp * c(nf, L, n), div=1e-7 * amp * c(nf, L, n), tv=amp * c(nf, L, n),
                trc=1e-4 * amp * c(nf, nt, L, n), lnps=1e-3 * amp * c(nf, n))


def compare(a, b, tol):
    for k in ("vrt", "tv", "lnps"):
        assert rel(a[k], b[k]) < tol, k
    assert rel_div(a, b) < tol
    if len(b["trc"]):
        assert rel(a["trc"], b["trc"]) < tol


def test_dfi_matches_oracle(oracle_mod):
    g, o, _ = pair(oracle_mod)
    g.dfi(3, t=0.0)
    o.dfi(3, 0.0)
    compare(g.get_state(), o.get_state(), 1e-9)
    g.advance(2)  # the step graph continues from the filtered state
    o.advance(2)
    compare(g.get_state(), o.get_state(), 1e-9)


def test_iau_matches_oracle_across_the_window(oracle_mod):
    g, o, _ = pair(oracle_mod)
    inc = increments(g, 3)
    fh = [0.0, 0.5, 1.0]
    for m in (g, o):
        m.set_iau(fh, 1.0, **inc)
    # t = -600 (before), 0 (first file), 600, 1200 (interior), 1800 (second
    # file), ..., 3600 (last file), 4200 (after)
    g.advance(9, t=-600.0)
    o.advance(9, t=-600.0)
    compare(g.get_state(), o.get_state(), 1e-9)


def test_iau_outside_the_window_changes_nothing():
    from gdpy import core, inputs

    ak, bk = inputs.hybrid_coords(20)
    st = inputs.smooth_random_state(42, 20, ntrac=1, seed=2)
    gs = []
    for with_iau in (False, True):
        g = core.Dycore(42, 128, 64, 20, ak, bk, ntrac=1, dt=600.0)
        g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=st["trc"])
        if with_iau:
            g.set_iau([5.0, 6.0], 1.0, **increments(g, 2))
        g.advance(4, t=0.0)
        gs.append(g.get_state())
    for k in ("vrt", "div", "tv", "trc", "lnps"):
        np.testing.assert_array_equal(gs[0][k], gs[1][k])


def test_iau_from_sigma_files(tmp_path):
    from gdpy import core, inputs, sigio

    T, L = 42, 20
    ak, bk = inputs.hybrid_coords(L)
    st = inputs.smooth_random_state(T, L, ntrac=1, seed=3)
    fg, anl = [], []
    rng = np.random.default_rng(1)
    for n in range(2):
        for kind, lst in (("fg", fg), ("anl", anl)):
            p = tmp_path / f"{kind}{n}.sig"
            h = sigio.hybrid_head(T, L, 1, 128, 64, ak, bk)
            f = {k: st[k] * (1 + 1e-3 * rng.standard_normal()) for k in ("vrt", "div", "tv", "trc", "lnps")}
            sigio.write(p, h, **f)
            lst.append(p)
    gs = []
    for via_files in (True, False):
        g = core.Dycore(T, 128, 64, L, ak, bk, ntrac=1, dt=600.0)
        g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=st["trc"])
        if via_files:
            g.set_iau_files([0.0, 1.0], fg, anl, delthrs=1.0)
        else:
            a = [sigio.read(p)[1] for p in anl]
            b = [sigio.read(p)[1] for p in fg]
            inc = {k: np.stack([x[k] - y[k] for x, y in zip(a, b)]) for k in ("vrt", "div", "tv", "trc", "lnps")}
            g.set_iau([0.0, 1.0], 1.0, **inc)
        g.advance(3, t=600.0)
        gs.append(g.get_state())
    for k in ("vrt", "div", "tv", "trc", "lnps"):
        np.testing.assert_array_equal(gs[0][k], gs[1][k])


def test_dfi_split_precision_follows_fp64(oracle_mod):
    g64, _, st = pair(oracle_mod)
    g32, _, _ = pair(oracle_mod, precision="tf32x3")
    for g in (g64, g32):
        g.dfi(3)
    a, b = g32.get_state(), g64.get_state()
    for k in ("vrt", "tv", "lnps"):
        assert rel(a[k], b[k]) < 1e-4, k
