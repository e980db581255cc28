"""DCMIP-2012 on the GPU: gd_dcmip_ics and the simple-physics plugin
(src/phy_run_simple.f90, src/simple_physics_v5_1.f90) with the moist dry-mass
bookkeeping (dyn_run.f90:135-150, 605-634), against the FP64 oracle.

Tolerances (relative, max-norm over the field; divergence, two to three
orders of magnitude smaller than vorticity in these states, is measured
against the vorticity scale): initial state 1e-11 (both sides transform the
same analytic grid values); physics tendencies and three full steps 1e-9 in
FP64 (measured: 4e-11 and below; the increments are differences of O(300 K)
temperatures and O(10 m/s) winds, so state ulps show at ~1e-12 of them).
TF32x3 against FP64 after six steps of the moist baroclinic wave: vorticity
2e-4, divergence 1e-3 of the vorticity scale, Tv 2e-6, ln ps 1e-6, q 2e-5
(measured 5e-5, 2.4e-4, 5e-7, 1e-7, 2.6e-6; without the physics 6e-6, 1e-4,
2e-7, 6e-8, 2e-7).  The T42 tropical cyclone (radius 282 km against a
300 km grid) is not used there: its FP32-state error is 3e-4 in vorticity
after six steps even without physics.
"""
import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu

FVIRT = float(np.float32(461.5)) / float(np.float32(287.05)) - 1.0
KAPPA = float(np.float32(287.05)) / float(np.float32(1004.6))
GRAV = float(np.float32(9.80665))


def rel_div(a, b):
    """divergence error against the vorticity scale"""
    return float(np.abs(a["div"] - b["div"]).max() / np.abs(b["vrt"]).max())


def make(oracle_mod, dcmip, T=42, nlon=128, nlat=64, L=26, ntrac=1, dry=False, dt=600.0, precision="fp64", **extra):
    from gdpy import core, inputs

    ak, bk = inputs.hybrid_coords(L)
    kw = dict(ntrac=ntrac, dt=dt, heldsuarez=False, dry=dry, **extra)
    g = core.Dycore(T, nlon, nlat, L, ak, bk, precision=precision, dcmip=dcmip, **kw)
    o = oracle_mod.Oracle(T, nlon, nlat, L, ak, bk, dcmip=dcmip, **kw)
    return g, o, ak, bk


def oracle_ics(o, testcase, ak, bk, ntrac, dry):
    import dcmip_oracle as do

    st = do.ics(o, testcase, ak, bk, ntrac, dry, FVIRT, KAPPA, GRAV)
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=st["trc"], topo=st["topo"])
    return st


def moist_pair(oracle_mod, testcase, ntrac, boost=1.6, **kw):
    """Both models on the DCMIP state with humidity scaled by boost: the
    analytic states are subsaturated, the scaled one condenses at once."""
    g, o, ak, bk = make(oracle_mod, testcase, ntrac=ntrac, **kw)
    g.dcmip_ics(testcase)
    st = oracle_ics(o, testcase, ak, bk, ntrac, False)
    for m in (g, o):
        x = m.get_state()
        trc = x["trc"].copy()
        trc[0] *= boost
        m.set_state(x["vrt"], x["div"], x["tv"], x["lnps"], trc=trc, topo=st["topo"])
    return g, o


@pytest.mark.parametrize("testcase,ntrac,dry", [(51, 1, False), (42, 3, False), (41, 3, True)])
def test_initial_state_matches_oracle(oracle_mod, testcase, ntrac, dry):
    g, o, ak, bk = make(oracle_mod, testcase, ntrac=ntrac, dry=dry)
    g.dcmip_ics(testcase)
    st = oracle_ics(o, testcase, ak, bk, ntrac, dry)
    a = g.get_state()
    for k in ("vrt", "div", "tv", "lnps"):
        assert rel(a[k], st[k]) < 1e-11, k
    for n in range(ntrac):
        if np.abs(st["trc"][n]).max() > 0:
            assert rel(a["trc"][n], st["trc"][n]) < 1e-11, n
    # orography: phis of test 4 through the same gradient as gd_set_state
    g.getdyntend(1, inverse_only=True)
    o.getdyntend(1, inverse_only=True)
    assert rel(g.get_grid("dphisdx"), o.get_grid("dphisdx")) < 1e-10 or testcase // 10 == 5


@pytest.mark.parametrize("testcase,ntrac", [(51, 1), (42, 3), (43, 3)])
def test_simple_physics_tendencies_match_oracle(oracle_mod, testcase, ntrac):
    g, o = moist_pair(oracle_mod, testcase, ntrac)
    g.advance(2)  # spin the state off the analytic balance
    o.advance(2)
    g.getdyntend(3, inverse_only=True)
    o.getdyntend(3, inverse_only=True)
    a, b = g.getphytend(), o.getphytend()
    for k in ("dvrt", "ddiv", "dtv"):
        assert rel(a[k], b[k]) < 1e-9, k
    assert rel(a["dtrc"][0], b["dtrc"][0]) < 1e-9
    for n in range(1, ntrac):
        assert not a["dtrc"][n].any()
    assert not a["dlnps"].any()
    for name in ("precip", "pwat"):
        assert rel(g.get_grid(name), o.get_grid(name)) < 1e-9, name
    assert g.get_grid("precip").max() > 0  # it rains
    if testcase != 42:  # turbulent fluxes act on the winds
        assert np.abs(a["dvrt"]).max() > 0


@pytest.mark.parametrize("testcase,ntrac", [(51, 1), (43, 3)])
def test_moist_steps_match_oracle(oracle_mod, testcase, ntrac):
    g, o = moist_pair(oracle_mod, testcase, ntrac)
    g.advance(3)
    o.advance(3)
    a, b = g.get_state(), o.get_state()
    for k in ("vrt", "tv", "lnps"):
        assert rel(a[k], b[k]) < 1e-9, k
    assert rel_div(a, b) < 1e-9
    assert rel(a["trc"][0], b["trc"][0]) < 1e-9
    # dry mass from the moist bookkeeping on the first step
    assert g.diag()["pdryini"] == pytest.approx(o.diag()["pdryini"], rel=1e-12)
    assert rel(g.get_grid("apcp"), o.get_grid("apcp")) < 1e-9


def test_split_precision_step_follows_fp64(oracle_mod):
    g64, _ = moist_pair(oracle_mod, 43, 3)
    g32, _ = moist_pair(oracle_mod, 43, 3, precision="tf32x3")
    for g in (g64, g32):
        g.advance(6)
    a, b = g32.get_state(), g64.get_state()
    for k, tol in (("vrt", 2e-4), ("tv", 2e-6), ("lnps", 1e-6)):
        assert rel(a[k], b[k]) < tol, k
    assert rel_div(a, b) < 1e-3
    assert rel(a["trc"][0], b["trc"][0]) < 2e-5
    assert g32.get_grid("apcp").max() > 0
