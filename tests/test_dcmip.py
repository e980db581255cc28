"""DCMIP-2012 analytic initial states: the library's host evaluation
(gd_dcmip_point, used by gd_dcmip_ics) against the numpy restatement of
src/dcmip_initial_conditions_test_4_v3.f90 and _test_5_v1.f90, and the
properties the test-case definitions state.  Host only: no GPU."""
import numpy as np
import pytest

import dcmip_oracle as do
from gdpy import core


def points(n, seed, near_tc=False):
    rng = np.random.default_rng(seed)
    if near_tc:
        lon = np.pi + rng.uniform(-0.15, 0.15, n)
        lat = np.deg2rad(10.0) + rng.uniform(-0.15, 0.15, n)
    else:
        lon = rng.uniform(0, 2 * np.pi, n)
        lat = np.arcsin(rng.uniform(-0.995, 0.995, n))
    p = rng.uniform(500.0, 101000.0, n)
    return lon, lat, p


@pytest.mark.parametrize("moist", [True, False])
def test_baroclinic_wave_points_match_restatement(moist):
    lon, lat, p = points(400, 1)
    lib = np.array([core.dcmip_point(42, a, b, c, moist) for a, b, c in zip(lon, lat, p)])
    ref = np.stack(do.test4(lon, lat, p, moist=moist), axis=1)
    for i, name in enumerate(["u", "v", "T", "phis", "ps", "q", "q1", "q2"]):
        np.testing.assert_allclose(lib[:, i], ref[:, i], rtol=1e-12, atol=1e-12 * np.abs(ref[:, i]).max() + 1e-300,
                                   err_msg=name)


@pytest.mark.parametrize("near", [True, False])
def test_tropical_cyclone_points_match_restatement(near):
    lon, lat, p = points(400, 2, near_tc=near)
    lib = np.array([core.dcmip_point(51, a, b, c) for a, b, c in zip(lon, lat, p)])
    ref = np.stack(do.test5(lon, lat, p), axis=1)
    for i, name in enumerate(["u", "v", "T", "phis", "ps", "q"]):
        np.testing.assert_allclose(lib[:, i], ref[:, i], rtol=1e-12, atol=1e-12 * np.abs(ref[:, i]).max() + 1e-300,
                                   err_msg=name)


def test_tropical_cyclone_structure():
    c = core.dcmip_point(51, np.pi, np.deg2rad(10.0), 95000.0)
    assert c[4] == pytest.approx(101500.0 - 1115.0)  # central pressure deficit
    assert abs(c[0]) < 1e-9 and abs(c[1]) < 1e-9  # calm at the centre
    far = core.dcmip_point(51, 0.0, 0.0, 95000.0)
    assert far[4] == pytest.approx(101500.0, abs=1e-6)
    # the strongest low-level wind lies some 100 km out, cyclonic (northern hemisphere)
    lons = np.pi + np.linspace(0.002, 0.1, 200)
    v = np.array([core.dcmip_point(51, x, np.deg2rad(10.0), 95000.0)[1] for x in lons])
    assert 15.0 < v.max() < 60.0 and v.argmax() > 3
    top = core.dcmip_point(51, np.pi + 0.02, np.deg2rad(10.0), 3000.0)
    assert top[0] == 0.0 and top[1] == 0.0 and top[5] == 1e-11  # above the tropopause


def test_baroclinic_wave_structure():
    lat = np.deg2rad(45.0)
    u = [core.dcmip_point(42, np.pi, lat, p)[0] for p in (25200.0, 50000.0, 90000.0)]
    assert u[0] == pytest.approx(4 * 35.0 * 0.25, rel=1e-12)  # jet core at eta0, 45N: 4 u0 sin^2 cos^2
    assert u[0] > u[1] > u[2]
    eq = core.dcmip_point(42, 1.0, 0.0, 100000.0)
    assert eq[5] == pytest.approx(0.021)  # humidity maximum at the surface equator
    dry = core.dcmip_point(41, 1.0, 0.0, 100000.0, moist=False)
    assert dry[5] == 0.0 and dry[2] > eq[2]  # dry: T is the virtual temperature itself


def test_bad_testcase_is_rejected():
    with pytest.raises(core.GdError):
        core.dcmip_point(31, 0.0, 0.0, 1e5)
