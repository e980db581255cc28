"""Learned per-column closure: a small network that corrects a coarse run's
tendencies, trained on coarse-grained high-resolution runs of this dycore.

The configuration: a coarse run (T62L64 in the full experiment) whose
columns' u, v, Tv (levels bottom to top) and ps go into a network nin = 3L+1
-> 256 (GELU) x 3 -> nout = 3L (du/dt, dv/dt, dTv/dt corrections), BF16
weights with FP32 accumulation.  The data come from the same dycore at a
higher truncation (T254L64), spectrally truncated to the coarse one every
`every_h` hours; the target of sample k is the coarse model's error after
`every_h` hours started from the coarse-grained truth of sample k,

    target_k = (truth_{k+1} - coarse_forecast_k) / (every_h h)   on the grid,

and the closure adds dt * net(columns) every step.  Alternatively
(target="tendency") the target is the truncation error of the tendencies
themselves, a deterministic function of the high-resolution state:

    target_k = trunc(tend_hi(truth_hi_k)) - tend_lo(trunc(truth_hi_k))   on the grid,

the dynamics (getdyntend, src/dyn_run.f90:33-305) plus the Held-Suarez
forcing (getphytend, src/phy_run_hs.f90:22-84) at each resolution, u and v
tendencies from the vorticity and divergence tendencies through getuv.  The
plain coarse step is the fallback (detach the net) and the yardstick:
`climate` compares zonal-mean u and T against the coarse-grained truth with
and without the net.

Run the experiment on a GPU with
    PYTHONPATH=gfs-dycore_gb300 python -m gdpy.closure --help
"""
import argparse
import json
import time

import numpy as np

from . import core, inputs

GRIDS = {21: (64, 32), 42: (128, 64), 62: (192, 94), 126: (384, 190), 254: (768, 384)}


def truncate(spec, T_hi, T_lo):
    """Spectral coefficients (m-major triangular, last axis) of truncation T_hi
    cut to T_lo: (m, n) kept for n <= T_lo."""
    idx = []
    off = 0
    for m in range(T_hi + 1):
        if m <= T_lo:
            idx.extend(range(off, off + (T_lo - m + 1)))
        off += T_hi - m + 1
    return np.asarray(spec)[..., np.asarray(idx)]


def _ctx(T, L, dt, precision, **kw):
    nlon, nlat = GRIDS[T]
    ak, bk = inputs.hybrid_coords(L)
    return core.Dycore(T, nlon, nlat, L, ak, bk, ntrac=0, dt=dt, precision=precision, **kw)


def full_tendency(g):
    """Spectral dynamics + Held-Suarez tendencies (dvrt, ddiv, dtv) of g's
    current state (getphytend reads the grids of the getdyntend pass)."""
    d = g.getdyntend(1)
    p = g.getphytend()
    return {k: d["d" + k] + p["d" + k] for k in ("vrt", "div", "tv")}


def coarse_truth(T_hi, T_lo, L, dt_hi, spin_days, days, every_h, seed=0, precision="tf32x3", log=print,
                 tendencies=False):
    """Held-Suarez run at T_hi from rest (seeded noise), sampled every `every_h`
    hours after `spin_days`, each sample truncated to T_lo.  With tendencies,
    each sample also carries the T_hi tendencies of its full state, truncated
    to T_lo (keys dvrt, ddiv, dtv)."""
    g = _ctx(T_hi, L, dt_hi, precision)
    st = inputs.hs_rest_state(T_hi, L, seed=seed)
    g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    per = int(round(every_h * 3600.0 / dt_hi))
    if abs(per * dt_hi - every_h * 3600.0) > 1e-6:
        raise ValueError("every_h must be a whole number of high-resolution steps")
    t0 = time.time()
    g.advance(int(round(spin_days * 86400.0 / dt_hi)))
    out = []
    nsamp = int(round(days * 24.0 / every_h)) + 1
    for k in range(nsamp):
        if k:
            g.advance(per)
        s = g.get_state()
        rec = {f: truncate(s[f], T_hi, T_lo) for f in ("vrt", "div", "tv", "lnps")}
        if tendencies:
            td = full_tendency(g)
            rec.update({"d" + f: truncate(td[f], T_hi, T_lo) for f in ("vrt", "div", "tv")})
        out.append(rec)
    log(f"truth T{T_hi}L{L}: {spin_days} + {days} days in {time.time() - t0:.1f} s, {len(out)} samples")
    return out


def features(g, state):
    g.set_state(state["vrt"], state["div"], state["tv"], state["lnps"])
    return g.closure_features()


def training_pairs(truth, T_lo, L, dt_lo, every_h, precision="tf32x3", net=None, col_frac=1.0, seed=0,
                   **coarse_kw):
    """(X, Y, E): closure inputs of every coarse sample k, the correction
    targets (truth_{k+1} - forecast_k) / every_h on the coarse grid and the
    errors themselves, stacked over samples [K-1, ncols, *].  With net
    attached, the forecasts include the closure (its remaining error).
    col_frac < 1 keeps that fraction of each sample's columns (drawn with
    seed).  coarse_kw configures the coarse model (default: the truth's
    forcing)."""
    g = _ctx(T_lo, L, dt_lo, precision, **coarse_kw)
    if net is not None:
        g.set_closure(net)
    per = int(round(every_h * 3600.0 / dt_lo))
    rng = np.random.default_rng(seed)
    X, Y, E = [], [], []
    for k in range(len(truth) - 1):
        x = features(g, truth[k])
        g.advance(per)
        f = g.closure_features()
        t = features(g, truth[k + 1])
        e = t[:, :3 * L] - f[:, :3 * L]
        if col_frac < 1.0:
            keep = rng.random(x.shape[0]) < col_frac
            x, e = x[keep], e[keep]
        X.append(x)
        E.append(e)
        Y.append(e / (every_h * 3600.0))
    return np.concatenate(X), np.concatenate(Y), np.concatenate(E)


def tendency_pairs(truth, T_lo, L, dt_lo, precision="tf32x3", col_frac=1.0, seed=0):
    """(X, Y): closure inputs of every coarse-grained sample and the targets
    trunc(tend_hi) - tend_lo(trunc state) on the coarse grid, columns [ncols,
    3L] (du/dt, dv/dt, dTv/dt at the levels bottom to top)."""
    g = _ctx(T_lo, L, dt_lo, precision)
    rng = np.random.default_rng(seed)
    X, Y = [], []
    for s in truth:
        x = features(g, s)
        lo = full_tendency(g)
        dvrt, ddiv, dtv = (s["d" + f] - lo[f] for f in ("vrt", "div", "tv"))
        du, dv = g.getuv(dvrt, ddiv)
        dt = g.spectogrd(dtv)
        y = np.concatenate([a.reshape(L, -1).T for a in (du, dv, dt)], axis=1)
        if col_frac < 1.0:
            keep = rng.random(x.shape[0]) < col_frac
            x, y = x[keep], y[keep]
        X.append(x)
        Y.append(y)
    return np.concatenate(X), np.concatenate(Y)


def train(X, Y, nhidden=256, nlayers=3, steps=3000, batch=4096, lr=1e-3, seed=1, device=0, log=print):
    """Fits an Mlp to columns X [n, nin] -> Y [n, nout] on the GPU with the
    library's kernels; inputs and outputs normalised per feature."""
    import torch

    X = X.reshape(-1, X.shape[-1]).astype(np.float32)
    Y = Y.reshape(-1, Y.shape[-1]).astype(np.float32)
    in_mu, in_sd = X.mean(0), X.std(0)
    in_sd = np.where(in_sd > 1e-6 * np.abs(in_mu).clip(1e-30) + 1e-12, in_sd, 1.0).astype(np.float32)
    out_mu, out_sd = Y.mean(0), Y.std(0)
    out_sd = np.where(out_sd > 0, out_sd, 1.0).astype(np.float32)
    dev = torch.device("cuda", device)
    xn = torch.from_numpy((X - in_mu) / in_sd).to(dev)
    yn = torch.from_numpy((Y - out_mu) / out_sd).to(dev)
    net = core.Mlp(X.shape[1], nhidden, nlayers, Y.shape[1], seed=seed, device=device)
    net.set_norm(in_mu, in_sd, out_mu, out_sd)
    rng = np.random.default_rng(seed)
    n = xn.shape[0]
    batch = min(batch, n)
    t0 = time.time()
    losses = []
    for s in range(steps):
        i = torch.from_numpy(rng.integers(0, n, batch)).to(dev)
        lr_s = lr * (0.1 ** (s / max(1, steps)))  # exponential decay to lr / 10
        want = s % 100 == 0 or s == steps - 1
        loss = net.train_step(xn.index_select(0, i).contiguous(), yn.index_select(0, i).contiguous(), lr_s, want)
        if want:
            losses.append((s, loss))
    net.sync()
    log(f"trained {net.nparams} parameters on {n} columns: {steps} steps in {time.time() - t0:.1f} s, "
        f"normalised loss {losses[0][1]:.4f} -> {losses[-1][1]:.4f}")
    return net, losses


def zonal_rmse(feat_a, feat_b, nlat, nlon, L):
    """RMSE over (latitude, level) of the zonal means of u and Tv."""
    a = feat_a.reshape(nlat, nlon, -1).mean(axis=1)
    b = feat_b.reshape(nlat, nlon, -1).mean(axis=1)
    du, dt = a[:, :L] - b[:, :L], a[:, 2 * L:3 * L] - b[:, 2 * L:3 * L]
    return float(np.sqrt((du ** 2).mean())), float(np.sqrt((dt ** 2).mean()))


def evaluate(truth, k0, T_lo, L, dt_lo, every_h, net, precision="tf32x3", **coarse_kw):
    """Coarse runs from coarse-grained truth sample k0 without and with the
    closure; zonal-mean u and T RMSE against the truth at each later sample."""
    nlon, nlat = GRIDS[T_lo]
    per = int(round(every_h * 3600.0 / dt_lo))
    res = {}
    for name, use in (("plain", None), ("closure", net)):
        g = _ctx(T_lo, L, dt_lo, precision, **coarse_kw)
        ref = _ctx(T_lo, L, dt_lo, precision)
        if use is not None:
            g.set_closure(use)
        s = truth[k0]
        g.set_state(s["vrt"], s["div"], s["tv"], s["lnps"])
        rows = []
        for k in range(k0 + 1, len(truth)):
            g.advance(per)
            rows.append(zonal_rmse(g.closure_features(), features(ref, truth[k]), nlat, nlon, L))
        res[name] = np.array(rows)
    return res


def climate(truth_eval, T_lo, L, dt_lo, every_h, net, precision="tf32x3", **coarse_kw):
    """Coarse runs over the evaluation window (from its first coarse-grained
    truth sample) without and with the closure.  Returns the RMSE over
    (latitude, level) of the time-mean zonal-mean u and T against the
    truth's, and the mean over the samples of the instantaneous zonal-mean
    RMSE."""
    nlon, nlat = GRIDS[T_lo]
    per = int(round(every_h * 3600.0 / dt_lo))
    ref = _ctx(T_lo, L, dt_lo, precision)

    def zm(feat):
        a = feat.reshape(nlat, nlon, -1).mean(axis=1)
        return a[:, :L], a[:, 2 * L:3 * L]

    tz = [zm(features(ref, s)) for s in truth_eval[1:]]
    t_u, t_t = np.mean([a for a, _ in tz], axis=0), np.mean([b for _, b in tz], axis=0)
    out = {}
    for name, use in (("plain", None), ("closure", net)):
        g = _ctx(T_lo, L, dt_lo, precision, **coarse_kw)
        if use is not None:
            g.set_closure(use)
        s = truth_eval[0]
        g.set_state(s["vrt"], s["div"], s["tv"], s["lnps"])
        zs, inst = [], []
        for k in range(1, len(truth_eval)):
            g.advance(per)
            z = zm(g.closure_features())
            zs.append(z)
            inst.append((np.sqrt(((z[0] - tz[k - 1][0]) ** 2).mean()), np.sqrt(((z[1] - tz[k - 1][1]) ** 2).mean())))
        m_u, m_t = np.mean([a for a, _ in zs], axis=0), np.mean([b for _, b in zs], axis=0)
        out[name] = {"mean_state_rmse_u": float(np.sqrt(((m_u - t_u) ** 2).mean())),
                     "mean_state_rmse_t": float(np.sqrt(((m_t - t_t) ** 2).mean())),
                     "instantaneous_rmse_u": float(np.mean([a for a, _ in inst])),
                     "instantaneous_rmse_t": float(np.mean([b for _, b in inst]))}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--t-hi", type=int, default=254)
    ap.add_argument("--t-lo", type=int, default=62)
    ap.add_argument("--nlev", type=int, default=64)
    ap.add_argument("--dt-hi", type=float, default=450.0)
    ap.add_argument("--dt-lo", type=float, default=1200.0)
    ap.add_argument("--spin-days", type=float, default=30.0)
    ap.add_argument("--train-days", type=float, default=160.0)
    ap.add_argument("--eval-days", type=float, default=60.0)
    ap.add_argument("--every-h", type=float, default=6.0)
    ap.add_argument("--col-frac", type=float, default=0.33, help="fraction of each sample's columns trained on")
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--precision", default="tf32x3")
    ap.add_argument("--target", default="error6h", choices=["error6h", "tendency"],
                    help="error6h: the coarse model's every_h-hour error; tendency: the truncation error of the "
                         "tendencies")
    ap.add_argument("--out", default=None, help="write the results (JSON) and the trained parameters (.npz) here")
    a = ap.parse_args(argv)
    L = a.nlev
    truth = coarse_truth(a.t_hi, a.t_lo, L, a.dt_hi, a.spin_days, a.train_days + a.eval_days, a.every_h,
                         precision=a.precision, tendencies=a.target == "tendency")
    ntrain = int(round(a.train_days * 24 / a.every_h))
    if a.target == "tendency":
        X, Y = tendency_pairs(truth[:ntrain + 1], a.t_lo, L, a.dt_lo, a.precision, col_frac=a.col_frac)
    else:
        X, Y, E = training_pairs(truth[:ntrain + 1], a.t_lo, L, a.dt_lo, a.every_h, a.precision,
                                 col_frac=a.col_frac)
    net, losses = train(X, Y, steps=a.steps, batch=a.batch, lr=a.lr)
    # the first evaluation week: 6-hour errors without and with the closure
    week = truth[ntrain:ntrain + int(round(7 * 24 / a.every_h)) + 1]
    _, _, e_plain = training_pairs(week, a.t_lo, L, a.dt_lo, a.every_h, a.precision)
    _, _, e_clos = training_pairs(week, a.t_lo, L, a.dt_lo, a.every_h, a.precision, net=net)
    rms = lambda e, sl: float(np.sqrt((e[..., sl] ** 2).mean()))
    held = {f: {"plain": rms(e_plain, sl), "closure": rms(e_clos, sl)}
            for f, sl in (("u", slice(0, L)), ("v", slice(L, 2 * L)), ("tv", slice(2 * L, 3 * L)))}
    clim = climate(truth[ntrain:], a.t_lo, L, a.dt_lo, a.every_h, net, a.precision)
    out = {
        "config": {k: getattr(a, k) for k in vars(a) if k != "out"},
        "train_columns": int(X.shape[0]),
        "loss": losses,
        "heldout_6h_error_rms": held,
        "eval_window": clim,
    }
    print(json.dumps({k: out[k] for k in ("train_columns", "heldout_6h_error_rms", "eval_window")}))
    if a.out:
        with open(a.out + ".json", "w") as f:
            json.dump(out, f, indent=1)
        np.savez(a.out + ".npz", params=net.get_params(), **dict(zip(("in_mu", "in_sd", "out_mu", "out_sd"),
                                                                      net._norm)))
    return out


if __name__ == "__main__":
    main()
