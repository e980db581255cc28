"""gd_ensemble_advance: members stepped together (each on its own stream and
step graph, overlapping on the GPU) give exactly the states of the same
members stepped one by one, with and without stochastic physics."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SMALL = [(2, 21, 64, 32, 8, 1, 1200.0), (1, 42, 128, 64, 20, 2, 900.0)]


@pytest.mark.parametrize("precision", ["fp64", "tf32x3"])
@pytest.mark.parametrize("sppt", [False, True])
def test_together_equals_one_by_one(precision, sppt):
    from gdpy import core, ensemble

    # the default tiles on both sides: autotuning may pick different levels
    # per warp for the two builds, which changes the last bits
    a = ensemble.build(precision, SMALL, sppt=sppt, seed0=5, autotune=False)
    b = ensemble.build(precision, SMALL, sppt=sppt, seed0=5, autotune=False)
    core.ensemble_advance(a, 4)
    for g in b:
        g.advance(4)
        g.sync()
    for x, y in zip(a, b):
        sx, sy = x.get_state(), y.get_state()
        for k in ("vrt", "div", "tv", "lnps", "trc"):
            np.testing.assert_array_equal(sx[k], sy[k])
    # members differ from each other (own seeds)
    assert not np.array_equal(a[0].get_state()["vrt"], a[1].get_state()["vrt"])
    for g in a + b:
        g.close()


def test_ensemble_rejects_bad_arguments():
    from gdpy import core

    with pytest.raises(core.GdError):
        core.ensemble_advance([], 1)
