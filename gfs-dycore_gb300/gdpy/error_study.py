"""Error of the fast precision modes against the plain FP64 GPU step.

Advances one FP64 context and one context per fast mode from the same
seeded initial state, in lockstep, and at each checkpoint compares the
spectral state field by field:

    max-norm relative error  max|x - x64| / max|x64|
    L2 relative error        ||x - x64||_2 / ||x64||_2

and the divergence error also against the vorticity scale,
max|div - div64| / max|vrt64| (the balanced flow's divergence is orders of
magnitude smaller than its vorticity, so its own max-norm magnifies any
error).

The pseudo-mode ``fp64_ulp`` is the floor: the FP64 step itself from the
initial state with every spectral coefficient moved by one unit in the last
place (numpy.nextafter towards +inf, real and imaginary parts).  No mode can
be expected to stay closer to the FP64 trajectory than the flow lets two FP64
trajectories 1 ulp apart stay.

Each mode's step is also timed (wall clock around its own advance, device
synchronised), so the table carries days/day against the FP64 step.

Usage (from the repository root):

    PYTHONPATH=gfs-dycore_gb300 python -m gdpy.error_study --workload T574L64 --hours 24 \
        --precisions fp64_ulp f64_tf32x3 tf32x3 bf16x3 fp32 --checkpoints 24 144 --out err.json
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
    "T62L64": (62, 192, 94, 64, 3, 1200.0),
}


def initial_state(name, T, nlat, L, nt, seed=0):
    if name in ("T574L64", "T62L64"):
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
    out["div"]["max_rel_vrt_scale"] = float(np.abs(x["div"] - ref["div"]).max() /
                                            max(np.abs(ref["vrt"]).max(), 1e-300))
    return out


def ulp_perturbed(st):
    """The state with every spectral coefficient one ulp larger (real and
    imaginary parts; zero imaginary parts of order 0 stay zero)."""
    out = dict(st)
    for k in ("vrt", "div", "tv", "lnps", "trc"):
        a = st.get(k)
        if a is None or np.size(a) == 0:
            continue
        re = np.nextafter(a.real, np.inf)
        im = np.where(a.imag != 0, np.nextafter(a.imag, np.inf), 0.0)
        out[k] = re + 1j * im
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
        x = ulp_perturbed(st) if prec == "fp64_ulp" else st
        g = core.Dycore(T, nlon, nlat, L, ak, bk, ntrac=nt, dt=dt, precision="fp64" if prec == "fp64_ulp" else prec)
        g.set_state(x["vrt"], x["div"], x["tv"], x["lnps"], trc=x.get("trc") if nt else None)
        return g

    ref = ctx("fp64")
    fast = {p: ctx(p) for p in precisions}
    wall = {p: 0.0 for p in ["fp64"] + list(fast)}
    timed_steps = 0
    res = dict(workload=workload, dt_s=dt, steps=nsteps, seed=seed, checkpoints=[])
    done = 0

    def adv(p, g, n):
        g.sync()
        t0 = time.perf_counter()
        g.advance(n)
        g.sync()
        # the first two steps run eagerly and capture the step graph: not timed
        if done >= 2:
            wall[p] += time.perf_counter() - t0

    for c in checkpoints:
        t0 = time.time()
        if done < 2 <= c:  # first two steps (eager + capture) apart from the timing
            for p, g in [("fp64", ref)] + list(fast.items()):
                g.advance(2 - done)
            done = 2
        adv("fp64", ref, c - done)
        for p, g in fast.items():
            adv(p, g, c - done)
        timed_steps += c - done
        done = c
        s64 = ref.get_state()
        entry = dict(step=c, hours=c * dt / 3600.0, errors={})
        for p, g in fast.items():
            entry["errors"][p] = field_errors(g.get_state(), s64)
        res["checkpoints"].append(entry)
        print(json.dumps(entry), file=log, flush=True)
        print(f"  ({time.time() - t0:.1f} s)", file=log, flush=True)
    if timed_steps:
        res["ms_per_step"] = {p: 1e3 * w / timed_steps for p, w in wall.items()}
        res["days_per_day"] = {p: dt / (ms * 1e-3) for p, ms in res["ms_per_step"].items() if ms > 0}
        res["speedup_vs_fp64"] = {p: res["ms_per_step"]["fp64"] / ms for p, ms in res["ms_per_step"].items()
                                  if ms > 0}
        print(json.dumps({k: res[k] for k in ("ms_per_step", "speedup_vs_fp64")}), file=log, flush=True)
    for g in list(fast.values()) + [ref]:
        g.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="T574L64", choices=list(WORKLOADS))
    ap.add_argument("--hours", type=float, default=24.0)
    ap.add_argument("--precisions", nargs="+", default=["fp64_ulp", "f64_tf32x3", "tf32x3", "fp32"],
                    help="modes compared with the FP64 step; fp64_ulp is the FP64 step from a 1-ulp perturbed state")
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
