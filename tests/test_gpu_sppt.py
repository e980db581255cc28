"""Stochastically perturbed physics (gd_set_sppt) against the CPU oracle.

The GPU step (FP64 path) with an attached pattern must follow the oracle's
step with the same single-precision pattern generator and the same SPPT
formula.  The patterns themselves agree to 2e-6 (their Gaussians differ in
the last ulp of log), so the perturbed states agree to the size of that
difference times the perturbation: tolerances below are stated per check.
"""
import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu

NORM = 2 * float(np.float32(np.pi))
PAT = (500e3, 1200.0, 21600.0, 0.5)  # lscale, dt, tau 6 h, amplitude 0.5


def make(oracle_mod, T=42, nlon=128, nlat=64, nlev=20, precision="fp64", seed=9, pj=20, sppt=True):
    from gdpy import core, inputs

    ak, bk = inputs.hybrid_coords(nlev)
    g = core.Dycore(T, nlon, nlat, nlev, ak, bk, dt=1200.0, precision=precision)
    o = oracle_mod.Oracle(T, nlon, nlat, nlev, ak, bk, dt=1200.0)
    st = inputs.hs_rest_state(T, nlev, seed=3, amp=1e-5)
    for m in (g, o):
        m.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    if sppt:
        gp = core.Pattern(*PAT, seed, pj, normalization=NORM)
        op = oracle_mod.PatternOracle(*PAT, seed, pj, NORM)
        gp.start()
        op.start()
        g.set_sppt(gp, 0.05, 0.10)
        o.set_sppt(op, 0.05, 0.10)
    return g, o


def test_sppt_grid_is_the_logit_of_the_synthesised_pattern(oracle_mod):
    g, o = make(oracle_mod)
    g.advance(1)
    grid = g.get_grid("sppt")[0]
    assert np.all(np.abs(grid) < 1)  # logit range
    # the pattern coefficients after one step, synthesised with the library's own transform
    pat = g._sppt.get()[0]
    full = np.zeros(g.nlm, np.complex128)
    T, pj = 42, 20
    i = k = 0
    for m in range(T + 1):
        for n in range(m, T + 1):
            if n <= pj:
                full[k] = pat[i]
                i += 1
            k += 1
    ref = 2 / (1 + np.exp(g.spectogrd(full[None])[0])) - 1
    np.testing.assert_allclose(grid, ref, rtol=0, atol=1e-13)


def test_sppt_step_matches_oracle(oracle_mod):
    g, o = make(oracle_mod)
    for n in (1, 2):
        g.advance(n)
        o.advance(n)
        a, b = g.get_state(), o.get_state()
        for k in ("vrt", "div", "tv", "lnps"):
            # pattern agreement 2e-6 x perturbation (0.5 of a physics tendency over a few steps)
            assert rel(a[k], b[k]) < 1e-9, (n, k, rel(a[k], b[k]))


def test_sppt_changes_the_trajectory(oracle_mod):
    g, _ = make(oracle_mod)
    h, _ = make(oracle_mod, sppt=False)
    g.advance(3)
    h.advance(3)
    a, b = g.get_state(), h.get_state()
    assert rel(a["vrt"], b["vrt"]) > 1e-6


@pytest.mark.parametrize("precision", ["fp32", "tf32x3"])
def test_sppt_in_fast_modes(oracle_mod, precision):
    g, o = make(oracle_mod, precision=precision)
    g.advance(4)  # eager first step, then the captured graph with the pattern inside
    o.advance(4)
    a, b = g.get_state(), o.get_state()
    tol = {"fp32": 2e-4, "tf32x3": 2e-4}[precision]
    for k in ("vrt", "tv", "lnps"):
        assert rel(a[k], b[k]) < tol, (k, rel(a[k], b[k]))


def test_sppt_rejects_a_pattern_finer_than_the_model(oracle_mod):
    from gdpy import core

    g, _ = make(oracle_mod, sppt=False)
    p = core.Pattern(*PAT, 1, 60, normalization=NORM)
    with pytest.raises(core.GdError):
        g.set_sppt(p)
