"""GPU stochastic pattern generator (gd_pattern_*) against the CPU oracle.

Both restate src/patterngenerator.f90 in single precision with the same
Mersenne-twister stream.  The uniform stream and the polar method's
accept/reject decisions are identical; a differing decision would shift every
later value and show as an O(1) error.  The Gaussians agree to the last ulp
of the two log implementations, so noise and patterns are compared at 2e-6
relative (max-norm).  The variance spectra are host set-up in the same
single-precision order and must match exactly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NORM = 2 * float(np.float32(np.pi))


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def core():
    from gdpy import core as c

    return c


def pair(core, oracle_mod, jcap, seed, nfields=1, lscale=500e3, dt=900.0, tau=21600.0, stdev=0.8):
    g = core.Pattern(lscale, dt, tau, stdev, seed, jcap, normalization=NORM, nfields=nfields)
    o = oracle_mod.PatternOracle(lscale, dt, tau, stdev, seed, jcap, NORM, nfields)
    return g, o


def test_spectra_match_exactly(core, oracle_mod):
    g, o = pair(core, oracle_mod, 62, 5)
    vs, v1, phi = g.spectra()
    ovs, ov1, ophi = o.spectra()
    np.testing.assert_array_equal(vs, ovs)
    np.testing.assert_array_equal(v1, ov1)
    assert phi == ophi
    g.close()


@pytest.mark.parametrize("jcap", [21, 62])
def test_noise_stream_matches_oracle(core, oracle_mod, jcap):
    g, o = pair(core, oracle_mod, jcap, 1234)
    for _ in range(3):  # consecutive draws continue the same stream
        a, b = g.getnoise(), o.getnoise()
        assert rel(a, b) < 2e-6
    assert g.launch_count() > 0
    g.close()


def test_pattern_start_and_advance_match_oracle(core, oracle_mod):
    g, o = pair(core, oracle_mod, 62, 77, nfields=3)
    g.start()
    o.start()
    assert rel(g.get(), o.get()) < 2e-6
    for n in (1, 4, 20):
        g.advance(n)
        o.advance(n)
        assert rel(g.get(), o.get()) < 2e-6


def test_long_advance_crosses_draw_chunks(core, oracle_mod):
    # more steps than one draw buffer holds: the stream continues across chunks
    g, o = pair(core, oracle_mod, 62, 4242, nfields=3, dt=1800.0)
    g.start()
    o.start()
    g.advance(150)
    o.advance(150)
    assert rel(g.get(), o.get()) < 2e-6
    g.close()


def test_t574_pattern_matches_oracle(core, oracle_mod):
    g, o = pair(core, oracle_mod, 574, 31, lscale=250e3, dt=150.0, tau=21600.0)
    g.start()
    o.start()
    g.advance(3)
    o.advance(3)
    assert rel(g.get(), o.get()) < 2e-6
    g.close()


def test_set_get_round_trip(core):
    g = core.Pattern(500e3, 900.0, 21600.0, 0.5, 3, 21, nfields=2)
    x = (np.random.default_rng(0).standard_normal((2, g.nlm)) + 1j).astype(np.complex64).astype(np.complex128)
    g.set(x)
    np.testing.assert_array_equal(g.get(), x)
    g.close()


def test_bad_arguments_are_rejected(core):
    with pytest.raises(core.GdError):
        core.Pattern(500e3, 0.0, 21600.0, 0.5, 3, 21)
    with pytest.raises(core.GdError):
        core.Pattern(500e3, 900.0, 21600.0, 0.5, 3, 0)
