"""GPU parity at the plain-FP64 configuration T126L64 (384x190 Gaussian
grid, 64 levels, 3 passive tracers, dt 600 s, Held-Suarez forcing):
seeded smooth random vorticity, divergence, temperature, ln(ps) and tracer
fields with spectral amplitudes ~ n^-2, against the FP64 CPU oracle.

Checked: the transform round trip (src/shtns.f90:171-231), every
getdyntend tendency (src/dyn_run.f90:33-305) and one full step
(src/run.f90:194-565).  Tolerances are max-norm relative errors; each test
prints the value it measured.
"""
import numpy as np
import pytest

from gdpy import core, inputs
from helpers import rel

pytestmark = pytest.mark.gpu

T, NLON, NLAT, L, NT, DT = 126, 384, 190, 64, 3, 600.0


@pytest.fixture(scope="module")
def both(oracle_mod):
    ak, bk = inputs.hybrid_coords(L)
    g = core.Dycore(T, NLON, NLAT, L, ak, bk, ntrac=NT, dt=DT)
    o = oracle_mod.Oracle(T, NLON, NLAT, L, ak, bk, ntrac=NT, dt=DT)
    st = inputs.smooth_random_state(T, L, ntrac=NT, seed=126)
    yield g, o, st
    g.close()


def set_both(g, o, st):
    for m in (g, o):
        m.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=st["trc"])


def test_round_trip_t126l64(both):
    g, o, st = both
    spec = np.concatenate([st["vrt"], st["tv"], st["trc"].reshape(-1, st["tv"].shape[1])])
    grid = g.spectogrd(spec)
    e_syn = rel(grid, o.spectogrd(spec))
    back = g.grdtospec(grid)
    e_rt = rel(back, spec)
    print(f"T126L64 synthesis vs oracle {e_syn:.2e}, round trip {e_rt:.2e}")
    assert e_syn < 1e-12 and e_rt < 1e-12


def test_getdyntend_t126l64(both):
    g, o, st = both
    set_both(g, o, st)
    a, b = g.getdyntend(1), o.getdyntend(1)
    errs = {k: rel(a[k], b[k]) for k in ("dvrt", "ddiv", "dtv", "dtrc", "dlnps")}
    print("T126L64 getdyntend", {k: f"{v:.2e}" for k, v in errs.items()})
    for k, e in errs.items():
        assert e < 1e-12, (k, e)
    # prs is the Phillips layer pressure ((p+^(k+1) - p-^(k+1)) / ((k+1)(p+ - p-)))^(1/k)
    # (src/pressure_data.f90:87-88): the difference of powers cancels in the
    # thin top layers, where 64 levels put it at ~2e-12 (measured 1.9e-12)
    for name, tol in (("ug", 1e-12), ("vg", 1e-12), ("tvg", 1e-12), ("dlnpsdt", 1e-12), ("dlnpdtg", 1e-12),
                      ("etadot", 1e-12), ("prs", 5e-12)):
        e = rel(g.get_grid(name), o.get_grid(name))
        assert e < tol, (name, e)


def test_one_step_t126l64(both):
    g, o, st = both
    set_both(g, o, st)
    g.advance(1)
    o.advance(1)
    a, b = g.get_state(), o.get_state()
    errs = {k: rel(a[k], b[k]) for k in ("vrt", "div", "tv", "lnps", "trc")}
    print("T126L64 one step", {k: f"{v:.2e}" for k, v in errs.items()})
    for k, e in errs.items():
        assert e < 1e-12, (k, e)
