"""CPU tests of the error study's helpers (gdpy/error_study.py): the 1-ulp
perturbation that defines the FP64 floor and the per-field error norms."""
import numpy as np

from gdpy import error_study


def _state(rng, L=3, n=10, nt=2):
    c = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)
    st = dict(vrt=c(L, n), div=c(L, n), tv=300 + c(L, n), lnps=c(n), trc=c(nt, L, n))
    st["lnps"][0] = 11.5  # order-0 coefficients are real
    return st


def test_ulp_perturbation_moves_every_coefficient_by_one_ulp():
    rng = np.random.default_rng(0)
    st = _state(rng)
    p = error_study.ulp_perturbed(st)
    for k in ("vrt", "div", "tv", "lnps", "trc"):
        a, b = st[k], p[k]
        np.testing.assert_array_equal(b.real, np.nextafter(a.real, np.inf))
        nz = a.imag != 0
        np.testing.assert_array_equal(b.imag[nz], np.nextafter(a.imag[nz], np.inf))
        np.testing.assert_array_equal(b.imag[~nz], 0.0)  # real coefficients stay real
    assert p["lnps"].imag[0] == 0.0


def test_field_errors_norms():
    rng = np.random.default_rng(1)
    ref = _state(rng)
    x = {k: v.copy() for k, v in ref.items()}
    x["vrt"][1, 2] += 1e-3 * np.abs(ref["vrt"]).max()
    x["div"][0, 0] += 2.0
    e = error_study.field_errors(x, ref)
    assert abs(e["vrt"]["max_rel"] - 1e-3) < 1e-12
    assert e["tv"]["max_rel"] == 0.0 and e["lnps"]["l2_rel"] == 0.0
    np.testing.assert_allclose(e["div"]["max_rel"], 2.0 / np.abs(ref["div"]).max())
    np.testing.assert_allclose(e["div"]["max_rel_vrt_scale"], 2.0 / np.abs(ref["vrt"]).max())
    np.testing.assert_allclose(e["div"]["l2_rel"], 2.0 / np.linalg.norm(ref["div"]))
