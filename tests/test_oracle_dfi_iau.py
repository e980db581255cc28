"""Digital filter initialisation (src/run.f90:58-145, set_dfi_wts :567-588)
and the incremental analysis update (src/iau_module.f90) in the oracle, and
the library's filter weights (gd_dfi_weights, host only).  No GPU."""
import numpy as np
import pytest

from gdpy import core, inputs


def np_weights(n):
    """set_dfi_wts with its single-precision angles (acos(-1.) of a default-real literal)."""
    pif = np.float32(np.arccos(np.float32(-1.0)))
    w = np.ones(2 * n + 1)
    for k in range(2 * n + 1):
        sx = float(pif * np.float32(k - n) / np.float32(n))
        wx = float(pif * np.float32(k - n) / np.float32(n + 1))
        if k != n:
            w[k] = np.sin(wx) / wx * np.sin(sx) / sx
    return w / w.sum()


@pytest.mark.parametrize("n", [1, 3, 6, 12, 48])
def test_filter_weights(oracle_mod, n):
    w = core.dfi_weights(n)
    np.testing.assert_array_equal(w, oracle_mod.dfi_weights(n))
    np.testing.assert_allclose(w, np_weights(n), rtol=1e-15, atol=1e-18)
    assert abs(w.sum() - 1.0) < 1e-14
    np.testing.assert_allclose(w, w[::-1], rtol=1e-14, atol=1e-18)
    assert w.argmax() == n
    # the end weights vanish up to the single-precision pi of the angles
    assert abs(w[0]) < 1e-7


def rest(T=21, L=8, dt=600.0, **kw):
    import oracle_py

    ak, bk = inputs.hybrid_coords(L)
    st = inputs.hs_rest_state(T, L, seed=1, amp=0.0)
    o = oracle_py.Oracle(T, 64, 32, L, ak, bk, dt=dt, adiabatic=True, heldsuarez=False, **kw)
    return o, st


def test_filter_keeps_a_steady_state(oracle_mod):
    o, st = rest()
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    o.dfi(4)
    s = o.get_state()
    for k in ("tv", "lnps"):
        np.testing.assert_allclose(s[k], st[k], rtol=0, atol=1e-14 * np.abs(st[k]).max())
    assert not s["vrt"].any() and not s["div"].any()


def test_filter_damps_gravity_waves(oracle_mod):
    T, L = 21, 8
    deg, order = inputs.degree_order(T)
    rng = np.random.default_rng(3)
    pert = (rng.standard_normal(deg.size) + 1j * rng.standard_normal(deg.size)) * 1e-6
    pert[order == 0] = pert[order == 0].real
    pert[deg < 10] = 0
    runs = []
    for filt in (True, False):
        o, st = rest(T, L)
        o.set_state(st["vrt"], st["div"] + pert[None, :], st["tv"], st["lnps"])
        o.dfi(12) if filt else o.advance(12)
        runs.append(np.sqrt((np.abs(o.get_state()["div"]) ** 2).mean()))
    assert runs[0] < 0.3 * runs[1]


def test_iau_forcing_interpolates_in_time(oracle_mod):
    o, st = rest(ntrac=1)
    L, n = 8, o.nlm
    rng = np.random.default_rng(5)
    nf = 3
    inc = {k: rng.standard_normal(s) + 1j * rng.standard_normal(s) for k, s in
           (("vrt", (nf, L, n)), ("div", (nf, L, n)), ("tv", (nf, L, n)), ("trc", (nf, 1, L, n)), ("lnps", (nf, n)))}
    fh, delthrs = np.array([3.0, 4.5, 6.0]), 1.5
    o.set_iau(fh, delthrs, **inc)
    dt = delthrs * 3600

    def want(t):
        if t < fh[0] * 3600 or t > fh[-1] * 3600:
            return {k: 0 * v[0] for k, v in inc.items()}
        if t == fh[-1] * 3600:
            return {k: v[-1] / dt for k, v in inc.items()}
        if t == fh[0] * 3600:
            return {k: v[0] / dt for k, v in inc.items()}
        m = int(np.argmax(fh * 3600 > t))
        d = (fh[m] - t / 3600) / (fh[m] - fh[m - 1])
        return {k: ((1 - d) * v[m] + d * v[m - 1]) / dt for k, v in inc.items()}

    names = dict(vrt="dvrt", div="ddiv", tv="dtv", trc="dtrc", lnps="dlnps")
    for t in (0.0, 3 * 3600.0, 3.7 * 3600, 4.5 * 3600, 5.99 * 3600, 6 * 3600.0, 7 * 3600.0):
        f, w = o.getiauforcing(t), want(t)
        for k, kk in names.items():
            np.testing.assert_allclose(f[kk], w[k], rtol=1e-15, atol=1e-18, err_msg=f"{k} at {t}")


def test_iau_adds_the_increment_over_the_window(oracle_mod):
    # a uniform warming on a rest state drives no motion: the global-mean Tv
    # coefficient gains exactly the forcing of every step inside the window
    o, st = rest(dt=600.0)
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    L, n = 8, o.nlm
    inc = dict(vrt=np.zeros((2, L, n)), div=np.zeros((2, L, n)), tv=np.zeros((2, L, n), complex),
               lnps=np.zeros((2, n)))
    inc["tv"][:, :, 0] = 0.5 * np.sqrt(4 * np.pi)  # +0.5 K everywhere over delthrs
    o.set_iau([0.0, 1.0], 1.0, **inc)
    o.advance(9, t=-600.0)  # t = -600 (outside), 0 ... 3600 (7 steps inside), 4200 (outside)
    s = o.get_state()
    gain = (s["tv"][:, 0] - st["tv"][:, 0]).real / np.sqrt(4 * np.pi)
    np.testing.assert_allclose(gain, 7 * 600.0 / 3600.0 * 0.5, rtol=1e-12)
    assert np.abs(s["div"]).max() < 1e-18
