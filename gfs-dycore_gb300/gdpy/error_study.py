"""Error of the fast precision modes against the plain FP64 GPU step.

Advances one FP64 context and one context per fast mode from the same
seeded initial state, in lockstep, and at each checkpoint compares the
spectral state field by field:

    max-norm relative error  max|x - x64| / max|x64|
    L2 relative error        ||x - x64||_2 / ||x64||_2

Usage (from the repository root):

    PYTHONPATH=gfs-dycore_gb300 python -m gdpy.error_study --workload T574L64 --hours 24 \
        --precisions tf32x3 fp32 --checkpoints 24 144 --out err.json
"""
import argparse
import json
import os
import sys
import time

import numpy as np

from . import core, inputs

WORKLOADS = {
    # name: (T, nlon, nlat, nlev, ntrac, dt)
    "T574L64": (574, 1152, 576, 64, 4, 150.0),
    "T126L64": (126, 384, 190, 64, 3, 600.0),
    "T42L20": (42, 128, 64, 20, 0, 1200.0),
}


def initial_state(name, T, nlat, L, nt, seed=0):
    if name == "T574L64":
        return inputs.balanced_jet_state(T, nlat, L, seed=seed, ntrac=nt)
    if name == "T126L64":
        return inputs.smooth_random_state(T, L, ntrac=nt, seed=seed)
    return inputs.hs_rest_state(T, L, seed=seed)


def field_errors(x, ref):
    out = {}
    for k in ("vrt", "div", "tv", "lnps", "trc"):
        if k not in ref or ref[k] is None or np.size(ref[k]) == 0:
            continue
        d = x[k] - ref[k]
        out[k] = dict(max_rel=float(np.abs(d).max() / max(np.abs(ref[k]).max(), 1e-300)),
                      l2_rel=float(np.linalg.norm(d) / max(np.linalg.norm(ref[k]), 1e-300)))
    return out


def run(workload, hours, precisions, checkpoints=None, seed=0, log=sys.stderr):
    T, nlon, nlat, L, nt, dt = WORKLOADS[workload]
    nsteps = int(round(hours * 3600.0 / dt))
    checkpoints = sorted(set(checkpoints or [])) or [nsteps]
    checkpoints = [c for c in checkpoints if 0 < c <= nsteps]
    if checkpoints[-1] != nsteps:
        checkpoints.append(nsteps)
    ak, bk = inputs.hybrid_coords(L)
    st = initial_state(workload, T, nlat, L, nt, seed)

    def ctx(prec):
        g = core.Dycore(T, nlon, nlat, L, ak, bk, ntrac=nt, dt=dt, precision=prec)
        g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=st.get("trc") if nt else None)
        return g

    ref = ctx("fp64")
    fast = {p: ctx(p) for p in precisions}
    res = dict(workload=workload, dt_s=dt, steps=nsteps, seed=seed, checkpoints=[])
    done = 0
    for c in checkpoints:
        t0 = time.time()
        ref.advance(c - done)
        for g in fast.values():
            g.advance(c - done)
        done = c
        s64 = ref.get_state()
        entry = dict(step=c, hours=c * dt / 3600.0, errors={})
        for p, g in fast.items():
            entry["errors"][p] = field_errors(g.get_state(), s64)
        res["checkpoints"].append(entry)
        print(json.dumps(entry), file=log, flush=True)
        print(f"  ({time.time() - t0:.1f} s)", file=log, flush=True)
    for g in list(fast.values()) + [ref]:
        g.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="T574L64", choices=list(WORKLOADS))
    ap.add_argument("--hours", type=float, default=24.0)
    ap.add_argument("--precisions", nargs="+", default=["tf32x3", "fp32"])
    ap.add_argument("--checkpoints", nargs="*", type=int, default=None, help="step numbers to compare at")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    res = run(a.workload, a.hours, a.precisions, a.checkpoints, a.seed)
    js = json.dumps(res)
    if a.out:
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        with open(a.out, "w") as f:
            f.write(js)
    print(js)


if __name__ == "__main__":
    main()
