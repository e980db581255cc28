"""The learned closure on the GPU: the network's forward pass and gradients
(gd_mlp, BF16 weights, FP32 accumulation; the products with the batch as
rows on the tensor cores) against the float64 numpy oracle with the same
BF16-rounded weights; tensor-core against SIMT training; training; the
closure inputs against the
library's transforms; a closure whose net is zero leaves the step bit for
bit unchanged; and what a trained closure gains over the plain coarse step.

Tolerances: forward 1e-5 and gradients 1e-4 of the largest entry (FP32
accumulation over at most a few hundred terms against float64); closure
inputs 1e-6 (float32 copies of the FP64 transforms).
"""
import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def net_and_data(nin=13, nh=32, nl=2, nout=7, n=300, seed=3):
    import mlp_oracle as mo
    from gdpy import core

    net = core.Mlp(nin, nh, nl, nout, seed=seed)
    rng = np.random.default_rng(seed)
    p = (rng.standard_normal(net.nparams) * 0.3).astype(np.float32)
    net.set_params(p)
    x = rng.standard_normal((n, nin)).astype(np.float32)
    t = rng.standard_normal((n, nout)).astype(np.float32)
    return net, p, x, t, mo.shapes(nin, nh, nl, nout)


def test_forward_matches_oracle():
    import mlp_oracle as mo

    net, p, x, _, shp = net_and_data()
    y = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    yo, _ = mo.forward(p, shp, x)
    assert rel(y, yo) < 1e-5
    np.testing.assert_array_equal(net.get_params(), p)


def test_closure_shape_forward_on_tensor_cores_matches_oracle():
    # the configured closure net (193 -> 256 x 3 -> 192): inference runs on the
    # tensor cores (TF32 hi + lo activations, weights exact in TF32)
    import mlp_oracle as mo
    from gdpy import core

    net = core.Mlp(193, 256, 3, 192, seed=11)
    rng = np.random.default_rng(11)
    shp = mo.shapes(193, 256, 3, 192)
    p = np.concatenate([np.concatenate([rng.standard_normal(fo * fi) * np.sqrt(2.0 / fi),
                                        rng.standard_normal(fo) * 0.1]) for fo, fi in shp]).astype(np.float32)
    net.set_params(p)
    x = rng.standard_normal((1000, 193)).astype(np.float32)
    y = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    yo, _ = mo.forward(p, shp, x)
    assert rel(y, yo) < 1e-5


def test_gradient_matches_oracle():
    import mlp_oracle as mo

    net, p, x, t, shp = net_and_data()
    loss, g = net.loss_grad(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda())
    lo, go = mo.loss_grad(p, shp, x, t)
    assert abs(loss - lo) <= 1e-5 * lo
    o = 0
    for fo, fi in shp:  # per layer: weights, then biases
        for sz in (fo * fi, fo):
            assert rel(g[o:o + sz], go[o:o + sz]) < 1e-4, (fo, fi, sz)
            o += sz


def test_closure_shape_gradient_matches_oracle():
    # the configured closure net (193 -> 256 x 3 -> 192): loss and every
    # layer's weight and bias gradients of the library's backward kernels
    # against the float64 oracle, on 512 columns
    import mlp_oracle as mo
    from gdpy import core

    nin, nh, nl, nout = 193, 256, 3, 192
    net = core.Mlp(nin, nh, nl, nout, seed=12)
    rng = np.random.default_rng(12)
    shp = mo.shapes(nin, nh, nl, nout)
    p = np.concatenate([np.concatenate([rng.standard_normal(fo * fi) * np.sqrt(2.0 / fi),
                                        rng.standard_normal(fo) * 0.1]) for fo, fi in shp]).astype(np.float32)
    net.set_params(p)
    x = rng.standard_normal((512, nin)).astype(np.float32)
    t = rng.standard_normal((512, nout)).astype(np.float32)
    loss, g = net.loss_grad(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda())
    lo, go = mo.loss_grad(p, shp, x, t)
    assert abs(loss - lo) <= 1e-5 * lo
    o = 0
    for fo, fi in shp:
        for sz in (fo * fi, fo):
            assert rel(g[o:o + sz], go[o:o + sz]) < 1e-4, (fo, fi, sz)
            o += sz
    assert o == net.nparams


def test_tensor_core_training_matches_simt_training(monkeypatch):
    # the configured closure net's loss and gradients with the training
    # products X W^T, dZ W and dZ^T A on the tensor cores (the default) and on
    # the SIMT kernels (GD_MLP_TRAIN_TC=0, read when a net is made): both
    # within FP32 accumulation of each other
    from gdpy import core

    nin, nh, nl, nout = 193, 256, 3, 192
    rng = np.random.default_rng(21)
    x = torch.from_numpy(rng.standard_normal((700, nin)).astype(np.float32)).cuda()
    t = torch.from_numpy(rng.standard_normal((700, nout)).astype(np.float32)).cuda()
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("GD_MLP_TRAIN_TC", flag)
        net = core.Mlp(nin, nh, nl, nout, seed=21)
        out.append(net.loss_grad(x, t))
    (l_tc, g_tc), (l_simt, g_simt) = out
    assert abs(l_tc - l_simt) <= 1e-5 * l_simt
    assert rel(g_tc, g_simt) < 1e-4
    assert not np.array_equal(g_tc, g_simt)  # two different product paths ran


def test_training_fits_a_smooth_map():
    from gdpy import core

    rng = np.random.default_rng(0)
    A = rng.standard_normal((10, 4)) / 3
    x = rng.standard_normal((4096, 10)).astype(np.float32)
    t = np.tanh(x @ A).astype(np.float32)
    net = core.Mlp(10, 64, 2, 4, seed=5)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    first = net.train_step(xd, td, 3e-3, want_loss=True)
    for _ in range(400):
        net.train_step(xd, td, 3e-3)
    last, _ = net.loss_grad(xd, td)
    assert last < 0.05 * first, (first, last)


def small_ctx(T=21, L=8, precision="fp64", dt=900.0):
    from gdpy import core, inputs

    nlon, nlat = {21: (64, 32), 42: (128, 64)}[T]
    ak, bk = inputs.hybrid_coords(L)
    return core.Dycore(T, nlon, nlat, L, ak, bk, ntrac=0, dt=dt, precision=precision)


def test_closure_features_match_transforms():
    from gdpy import inputs

    T, L = 21, 8
    g = small_ctx(T, L)
    st = inputs.smooth_random_state(T, L, ntrac=0, seed=4)
    g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    x = g.closure_features()
    u, v = g.getuv(st["vrt"], st["div"])
    tv = g.spectogrd(st["tv"])
    ps = np.exp(g.spectogrd(st["lnps"]))
    for k in range(L):
        assert rel(x[:, k], u[k].ravel()) < 1e-6
        assert rel(x[:, L + k], v[k].ravel()) < 1e-6
        assert rel(x[:, 2 * L + k], tv[k].ravel()) < 1e-6
    assert rel(x[:, 3 * L], ps[0].ravel()) < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "tf32x3"])
def test_zero_closure_changes_nothing(precision):
    from gdpy import core, inputs

    T, L = 21, 8
    st = inputs.hs_rest_state(T, L, seed=6)
    out = []
    for attach in (False, True):
        g = small_ctx(T, L, precision)
        g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
        if attach:
            net = core.Mlp(3 * L + 1, 16, 1, 3 * L)
            net.set_params(np.zeros(net.nparams, np.float32))
            net.set_norm(np.zeros(3 * L + 1), np.ones(3 * L + 1), np.zeros(3 * L), np.ones(3 * L))
            g.set_closure(net)
        g.advance(3)
        out.append(g.get_state())
    for k in ("vrt", "div", "tv", "lnps"):
        np.testing.assert_array_equal(out[0][k], out[1][k])


def test_closure_rejects_a_wrong_net():
    from gdpy import core

    g = small_ctx()
    net = core.Mlp(10, 8, 1, 5)
    with pytest.raises(core.GdError):
        g.set_closure(net)
    ok = core.Mlp(3 * 8 + 1, 8, 1, 3 * 8)
    with pytest.raises(core.GdError):  # no normalisation yet
        g.set_closure(ok)


def test_trained_closure_reduces_the_coarse_error():
    """T42L20 Held-Suarez truth, truncated to T21L20 every 6 h, and a coarse
    T21L20 model without the forcing: its 6-hour error is mostly the missing
    drag and relaxation, which a column's u, v, Tv and ps determine up to
    its latitude (the relaxation temperature depends on it and is not an
    input).  A net trained on 10 sample pairs must learn the part the column
    determines: the training loss falls below 0.7 of its start and the
    coarse model's 6-hour u and Tv errors on those pairs by more than 15 %
    with the net attached."""
    from gdpy import closure

    T_hi, T_lo, L = 42, 21, 20
    truth = closure.coarse_truth(T_hi, T_lo, L, 900.0, spin_days=2.0, days=2.5, every_h=6.0,
                                 precision="fp64", log=lambda *a: None)
    coarse = dict(heldsuarez=False)
    X, Y, E = closure.training_pairs(truth, T_lo, L, 1200.0, 6.0, "fp64", **coarse)
    net, losses = closure.train(X, Y, nhidden=64, nlayers=2, steps=1500, batch=2048, lr=2e-3,
                                log=lambda *a: None)
    assert losses[-1][1] < 0.7 * losses[0][1], losses
    _, _, E2 = closure.training_pairs(truth, T_lo, L, 1200.0, 6.0, "fp64", net=net, **coarse)
    for sl in (slice(0, L), slice(2 * L, 3 * L)):  # u and Tv
        before = np.sqrt((E[..., sl] ** 2).mean())
        after = np.sqrt((E2[..., sl] ** 2).mean())
        assert after < 0.85 * before, (sl, before, after)
