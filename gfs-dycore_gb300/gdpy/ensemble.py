"""Ensemble of mixed truncations with stochastically perturbed physics.

The batching workload: 16 members at T62L64 (192x94), 10 at T126L64
(384x190) and 6 at T254L64 (768x384), each with its own seeded initial noise
and its own AR(1) stochastic perturbation of the physics tendencies
(gd_set_sppt: amplitude 0.5, decorrelation 6 h, spectral pattern truncated at
n = 40), in split precision.  The members are advanced one by one
(gd_advance + sync per member) and together (gd_ensemble_advance: every
member's captured step graph on its own stream, overlapping on the GPU); the
rate is the sum over members of simulated time per wall time, member-days/day.
Each member's tile shapes are chosen by the autotuner (gd_autotune) at set-up
unless --no-autotune is given.

Usage (from the repository root):

    PYTHONPATH=gfs-dycore_gb300 python -m gdpy.ensemble --steps 10 --out ens.json
"""
import argparse
import json
import os
import time

import numpy as np

from . import core, inputs

MEMBERS = [  # (count, T, nlon, nlat, nlev, ntrac, dt)
    (16, 62, 192, 94, 64, 3, 1200.0),
    (10, 126, 384, 190, 64, 3, 600.0),
    (6, 254, 768, 384, 64, 3, 300.0),
]
PATTERN = dict(lscale=500e3, tau=6 * 3600.0, stdev=0.5, jcap=40)


def build(precision="tf32x3", members=MEMBERS, sppt=True, seed0=0, autotune=True):
    """The members, each with its state and pattern set; with autotune every
    member's tile shapes are chosen by gd_autotune on its own buffers (the
    best tiles differ between truncations)."""
    out = []
    i = 0
    for count, T, nlon, nlat, L, nt, dt in members:
        ak, bk = inputs.hybrid_coords(L)
        for _ in range(count):
            g = core.Dycore(T, nlon, nlat, L, ak, bk, ntrac=nt, dt=dt, precision=precision)
            st = inputs.smooth_random_state(T, L, ntrac=nt, seed=seed0 + i)
            g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=st["trc"])
            if sppt:
                p = core.Pattern(PATTERN["lscale"], dt, PATTERN["tau"], PATTERN["stdev"], 1000 + seed0 + i,
                                 min(PATTERN["jcap"], T))
                p.start()
                g.set_sppt(p)
            g.dt_s = dt
            g.tiles = g.autotune() if autotune else None
            out.append(g)
            i += 1
    return out


def measure(steps=10, warmup=3, precision="tf32x3", autotune=True):
    t0 = time.perf_counter()
    ms = build(precision, autotune=autotune)
    setup = time.perf_counter() - t0
    for g in ms:  # first step eager, second captures the graph
        g.advance(warmup)
    for g in ms:
        g.sync()
    sim = sum(g.dt_s for g in ms) * steps  # simulated seconds over all members
    t0 = time.perf_counter()
    for g in ms:
        g.advance(steps)
        g.sync()
    one_by_one = time.perf_counter() - t0
    t0 = time.perf_counter()
    core.ensemble_advance(ms, steps)
    together = time.perf_counter() - t0
    res = dict(workload="16xT62L64 + 10xT126L64 + 6xT254L64, SPPT 0.5 / 6 h / n<=40", precision=precision,
               members=len(ms), steps=steps,
               one_by_one=dict(seconds=one_by_one, member_days_per_day=sim / one_by_one),
               together=dict(seconds=together, member_days_per_day=sim / together),
               speedup=one_by_one / together, setup_seconds=setup,
               tiles={f"T{g.ntrunc}L{g.nlev}": g.tiles for g in ms} if autotune else None)
    finite = all(np.isfinite(g.get_state()["vrt"]).all() for g in ms)
    res["states_finite"] = bool(finite)
    for g in ms:
        g.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--precision", default="tf32x3", choices=["fp32", "tf32x3", "bf16x3", "fp64"])
    ap.add_argument("--out", default=None)
    ap.add_argument("--no-autotune", action="store_true", help="keep the default tile shapes")
    a = ap.parse_args()
    res = measure(a.steps, a.warmup, a.precision, autotune=not a.no_autotune)
    js = json.dumps(res)
    if a.out:
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        with open(a.out, "w") as f:
            f.write(js)
    print(js)


if __name__ == "__main__":
    main()
