#!/usr/bin/env python3
"""Benchmark of the GFS spectral dycore time step on GB300.

Metric: simulated days per wall-clock day at T574L64 (1152x576 Gaussian
grid, 64 levels, 7 prognostic 3-D fields = vrt, div, Tv + 4 tracers,
dt = 150 s), balanced-jet initial state, Held-Suarez forcing.  ``value`` is
the --precision step with the state resident in HBM.  ``precision_modes``
advances the plain FP64 GPU step and every fast mode --err-steps steps from
the same state and reports each mode's step time, its speed-up over FP64
and its relative error per spectral field against the FP64 state.

``e2e`` times the same step through the C ABI with the state copied in from
pinned host memory and out again every step, in the layout of the
reference's default build (single-precision reals: complex(4) spectral
arrays through gd_set_state_f / gd_advance / gd_get_state_f); the complex(8)
layout (gd_set_state / gd_get_state) is reported beside it.  ``configs`` adds the T42L20 and T126L64 configurations in
days/day (FP64 on the GPU, the FP64 CPU oracle on the host threads).
``--impl reference`` times full steps of the FP64 CPU restatement of the
reference algorithm (the reference's Fortran + SHTns build cannot be made
here) on the host cores.

Multi-GPU: replicas only (independent members, one per rank, no exchange);
``value`` is the aggregate member-days per day.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gfs-dycore_gb300"))

WORKLOADS = {
    # name: (T, nlon, nlat, nlev, ntrac, dt)
    "T574L64": (574, 1152, 576, 64, 4, 150.0),
    "T254L64": (254, 768, 384, 64, 3, 300.0),
    "T126L64": (126, 384, 190, 64, 3, 600.0),
    "T42L20": (42, 128, 64, 20, 0, 1200.0),
    # the T574 grid and transform lengths with a quarter of the levels: the
    # case for ncu captures, which must stay within a few GB of device memory
    "T574L16": (574, 1152, 576, 16, 1, 150.0),
}
METRIC = "simulated days/day at T574L64: mixed-precision vs FP64 GPU at stated error"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return dict(hbm=d["hbm_gbs"], bf16=d["bf16_tflops"], bf16s=d["bf16_tflops_sustained"], src="measured")
    return dict(hbm=6800.0, bf16=1900.0, bf16s=1700.0, src="fallback")


def make_state(name, seed):
    from gdpy import inputs

    T, nlon, nlat, L, nt, dt = WORKLOADS[name]
    if name in ("T574L64", "T574L16"):
        return inputs.balanced_jet_state(T, nlat, L, seed=seed, ntrac=nt)
    if name in ("T126L64", "T254L64"):
        return inputs.smooth_random_state(T, L, ntrac=nt, seed=seed)
    return inputs.hs_rest_state(T, L, seed=seed)


class Clocks:
    """nvidia-smi sampler for the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.device = device
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()
        self.f.flush()

    def summary(self):
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=["unavailable"], samples=0)
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return dict(sm_mhz=statistics.median(sm) if sm else None,
                    sm_max_mhz=float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                    reasons=reasons, samples=len(rows))


def work_counts(T, nlon, nlat, L, nt, rsize):
    """Algorithmic work of one step of this implementation, per phase.

    Legendre: 2*nlm*nlat flop per transformed complex column (a scalar
    transform; 4 flop per complex x real multiply-add over nlat/2 latitude
    pairs).  FFT/grid phases: bytes each row must move once.
    """
    nlm = (T + 1) * (T + 2) // 2
    ncolS = (5 + nt) * L + 1
    synth_cols = ncolS + (ncolS - 2 * L)
    anal_cols = ((4 + nt) * L + 1) + 2 * L
    cols = 3 * (synth_cols + anal_cols) + synth_cols + (3 * L + 1)
    scalar_flop = 2.0 * nlm * nlat
    ng = nlon * nlat
    cbytes = 2 * rsize
    c2r_rows = (7 + 3 * nt) * L + 3
    inv_rows = 5 * L + 3 + nt * L
    two_src = 2 * L + 0  # u, v read two Fourier columns
    c2r_bytes = 3 * (c2r_rows * ng * rsize + (c2r_rows + two_src) * (T + 1) * nlat * cbytes) + \
        (inv_rows * ng * rsize + (inv_rows + two_src) * (T + 1) * nlat * cbytes)
    r2c_rows = (4 + nt) * L + 1
    r2c_bytes = 3 * (r2c_rows * ng * rsize + (r2c_rows + 2 * L) * (T + 1) * nlat * cbytes) + \
        ((3 * L + 1) * ng * rsize + (3 * L + 1) * (T + 1) * nlat * cbytes)
    col_in = (7 + 3 * nt) * L + 3
    col_bytes = 3 * (col_in + r2c_rows) * ng * rsize + (5 * L + 3) * ng * rsize

    # Legendre GEMM launches: each reads (synthesis) or writes (analysis) its
    # real columns of the spectral array (nlm rows) and writes or reads them in
    # the Fourier array ((T+1) orders x nlat), and reads the table (hi and lo
    # copies in the split modes, nlm x nlat/2 each)
    def leg(ncomplex, tables):
        return 2 * ncomplex * (nlm + (T + 1) * nlat) * rsize + tables * nlm * (nlat // 2) * rsize

    ntab = 2 if rsize == 4 else 1
    legendre_launches = [ncolS, ncolS - 2 * L] * 4 + [(4 + nt) * L + 1, 2 * L] * 3 + [3 * L + 1]
    legendre_bytes = sum(leg(c, ntab) for c in legendre_launches)
    return dict(legendre_flop=cols * scalar_flop, legendre_cols=cols, c2r_bytes=c2r_bytes, r2c_bytes=r2c_bytes,
                col_bytes=col_bytes, scalar_flop=scalar_flop, legendre_bytes=legendre_bytes,
                legendre_launches=len(legendre_launches))


def gpu_arm(args):
    import torch

    from gdpy import core, inputs
    from gdpy.replicas import ReplicaGroup

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    grp = ReplicaGroup("nccl")  # replicas: one independent member per rank
    rank, world = grp.rank, grp.world
    name = args.workload
    T, nlon, nlat, L, nt, dt = WORKLOADS[name]
    ak, bk = inputs.hybrid_coords(L)
    st = make_state(name, seed=grp.member_seed())
    trc = st["trc"] if nt else None
    stream = torch.cuda.Stream()  # a capturable stream shared with the library

    def ctx(prec):
        g = core.Dycore(T, nlon, nlat, L, ak, bk, ntrac=nt, dt=dt, precision=prec, device=local)
        g.set_stream(stream.cuda_stream)
        g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=trc)
        return g

    def barrier():
        grp.barrier()
        torch.cuda.synchronize()

    def timed(g, steps, warmup):
        g.advance(warmup)
        barrier()
        n0 = g.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with Clocks(local) as ck:
            e0.record(stream)
            g.advance(steps)
            e1.record(stream)
            barrier()
        ms = grp.max_over_ranks(e0.elapsed_time(e1))
        return ms, g.launch_count() - n0, ck.summary()

    # fast-precision step (the headline), its tile shapes chosen by the library's autotuner on this context
    g = ctx(args.precision)
    tuned = None
    if not args.no_autotune:
        tuned = g.autotune()
        g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=trc)
    ms, launches, clocks = timed(g, args.steps, args.warmup)
    ms_step = ms / args.steps
    # simulated seconds per wall second == simulated days per day, summed over ranks
    value = grp.job_rate(dt * args.steps, ms * 1e-3)
    phases = g.profile_step()
    fast_state = g.get_state()
    steps_done = args.warmup + args.steps + 1

    # end to end through the C ABI with host buffers
    pinned = {}
    for k in ("vrt", "div", "tv", "lnps") + (("trc",) if nt else ()):
        t = torch.empty(st[k].shape + (2,), dtype=torch.float64, pin_memory=True)
        a = t.numpy().view(np.complex128).reshape(st[k].shape)
        a[...] = st[k]
        pinned[k] = a
    lib = core.load()
    import ctypes

    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    h2d = sum(a.nbytes for a in pinned.values())
    for _ in range(2):
        g.set_state(pinned["vrt"], pinned["div"], pinned["tv"], pinned["lnps"], trc=pinned.get("trc"))
        g.advance(1)
    barrier()
    e2e_steps = max(1, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        g._chk(lib.gd_set_state(g.h, P(pinned["vrt"]), P(pinned["div"]), P(pinned["tv"]),
                                P(pinned["trc"]) if nt else None, P(pinned["lnps"]), None))
        g.advance(1)
        g._chk(lib.gd_get_state(g.h, P(pinned["vrt"]), P(pinned["div"]), P(pinned["tv"]),
                                P(pinned["trc"]) if nt else None, P(pinned["lnps"])))
    barrier()
    e2e_ms = grp.max_over_ranks((time.perf_counter() - t0) * 1e3 / e2e_steps)
    e2e64 = dict(value=grp.job_rate(dt, e2e_ms * 1e-3), unit="simulated days/day",
                 h2d_bytes_per_step=h2d, d2h_bytes_per_step=h2d, ms_per_step=e2e_ms,
                 host_layout="complex(8) (gd_set_state / gd_get_state)")
    # the headline: the single-precision host entry points, the layout of the reference's default build
    # (kinds.f90: default_real = 1, r_kind = 4 -> complex(4) spectral arrays), half the bytes each way
    pin32 = {}
    for k in pinned:
        t = torch.empty(st[k].shape + (2,), dtype=torch.float32, pin_memory=True)
        a = t.numpy().view(np.complex64).reshape(st[k].shape)
        a[...] = st[k]
        pin32[k] = a
    h2d32 = sum(a.nbytes for a in pin32.values())
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        g._chk(lib.gd_set_state_f(g.h, P(pin32["vrt"]), P(pin32["div"]), P(pin32["tv"]),
                                  P(pin32["trc"]) if nt else None, P(pin32["lnps"]), None))
        g.advance(1)
        g._chk(lib.gd_get_state_f(g.h, P(pin32["vrt"]), P(pin32["div"]), P(pin32["tv"]),
                                  P(pin32["trc"]) if nt else None, P(pin32["lnps"])))
    barrier()
    e2e32_ms = grp.max_over_ranks((time.perf_counter() - t0) * 1e3 / e2e_steps)
    e2e = dict(value=grp.job_rate(dt, e2e32_ms * 1e-3), unit="simulated days/day",
               h2d_bytes_per_step=h2d32, d2h_bytes_per_step=h2d32, ms_per_step=e2e32_ms,
               host_layout="complex(4), the reference's default real kind (gd_set_state_f / gd_get_state_f)",
               double_precision_host=e2e64)

    # roofline of the dominant phase
    pk = peaks()
    rsize = 8 if args.precision.startswith("f") and args.precision != "fp32" else 4
    wc = work_counts(T, nlon, nlat, L, nt, rsize)
    dom = max(phases, key=phases.get)
    leg_ms = phases["legendre_synth"] + phases["legendre_anal"]
    if args.precision in ("tf32x3", "bf16x3", "f64_tf32x3", "f64_eddy") and \
            (dom in ("legendre_synth", "legendre_anal") or leg_ms >= max(phases.values())):
        if args.precision.startswith("f64"):  # the GEMM runs on FP32 staging copies of the FP64 operands
            wc = work_counts(T, nlon, nlat, L, nt, 4)
        # The split-precision Legendre GEMM issues 3 products per algorithmic one: 6 flop per
        # (coefficient, latitude pair) against ~4 bytes of array traffic per coefficient and column, an
        # intensity (~140 flop/B at T574 with the tables) below this GPU's tensor balance point: the HBM
        # roof is the lower one.
        nl = wc["legendre_launches"]
        achieved = wc["legendre_bytes"] / (leg_ms * 1e-3) / 1e9
        flops = wc["legendre_flop"] / (leg_ms * 1e-3) / 1e12
        roof = dict(kernel="k_tc_gemm_f (Legendre synthesis+analysis, orders m >= 1)", bound="hbm",
                    achieved=achieved, peak=pk["hbm"], unit="GB/s", frac=achieved / pk["hbm"], traffic=None,
                    peak_source=pk["src"], algorithmic_bytes_per_launch=wc["legendre_bytes"] / nl,
                    ms_per_launch=leg_ms / nl, algorithmic_tflops=flops, issued_tflops=3 * flops)
        # tensor rate: kind::tf32 is half the dense BF16 rate; the BF16 burst figure is measured
        tf32_peak = 0.5 * pk["bf16"]
        roof["tf32_peak_tflops"] = tf32_peak
        roof["tf32_peak_source"] = "0.5 x bf16_tflops (" + pk["src"] + "): dense TF32 is half the BF16 rate"
        roof["tensor_frac_of_tf32"] = 3 * flops / tf32_peak
        if args.precision == "tf32x3" and name == "T574L64":
            tr = profiled_gemm_traffic()
            if tr:
                roof["traffic"] = tr
                roof["traffic_unit"] = "bytes per launch (ncu, " + GEMM_PROFILE + ")"
    elif dom in ("legendre_synth", "legendre_anal") or leg_ms >= max(phases.values()):
        achieved = wc["legendre_flop"] / (leg_ms * 1e-3) / 1e12
        roof = dict(kernel="legendre GEMMs (synthesis+analysis)", bound="tensor", achieved=achieved,
                    peak=pk["bf16"], unit="TFLOP/s", frac=achieved / pk["bf16"], traffic=None,
                    peak_source=pk["src"] + " bf16 burst", note="SIMT FMA path; tensor peak shown for scale")
    else:
        key = {"fft_synth": "c2r_bytes", "fft_anal": "r2c_bytes", "columns": "col_bytes"}.get(dom)
        byt = wc[key] if key else None
        achieved = byt / (phases[dom] * 1e-3) / 1e9 if byt else None
        roof = dict(kernel=dom, bound="hbm", achieved=achieved, peak=pk["hbm"], unit="GB/s",
                    frac=(achieved / pk["hbm"]) if achieved else None, traffic=None, peak_source=pk["src"])
    g.close()

    # every precision mode against the plain FP64 step: the same seeded state advanced err_steps steps, each
    # mode timed over its own steps after the eager and capture steps, compared field by field
    modes = None
    if args.err_steps > 0:
        modes = precision_modes(ctx, st, args.err_steps, dt, stream, barrier, grp, args.precision)
    out = {
        "metric": METRIC, "value": value, "unit": "simulated days/day", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": DTYPES[args.precision],
        "data": "synthetic (seeded balanced jet, Held-Suarez forcing)",
        "config": {"workload": name, "ntrunc": T, "grid": f"{nlon}x{nlat}", "nlev": L, "ntrac": nt, "dt_s": dt,
                   "precision": args.precision, "parallelism": f"replicas x{world}", "autotune": tuned,
                   "l2": "inputs larger than L2 (resident state and grids are GBs)"},
        "precision_modes": modes, "e2e": e2e, "gpu_launches": int(launches), "roofline": roof,
        "phases_ms": phases, "clocks": clocks,
    }
    if modes:
        h = modes["modes"].get(args.precision)
        if h:
            out["fp64"] = dict(ms_per_step=modes["fp64_ms_per_step"], days_per_day=modes["fp64_days_per_day"],
                               speedup=modes["fp64_ms_per_step"] / ms_step, rel_err=h["rel_err"],
                               steps_compared=args.err_steps)
    if rank == 0:
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(name)
        if not args.no_configs:
            out["configs"] = config_rows(args.config_cpu)
        # the next rows beside the step: the stochastic pattern generator and the
        # DCMIP simple physics
        out["pattern_generator"] = pattern_generator_rate()
        if not args.no_dcmip:
            out["dcmip_simple_physics"] = dcmip_rate(args.precision if args.precision in SIMPLE_PREC else "tf32x3")
        if not args.no_closure:
            out["learned_closure"] = closure_rate("tf32x3")
        if not args.no_ensemble:
            # the batching workload: 32 mixed-truncation members with SPPT, stepped one by one and together
            from gdpy import ensemble

            out["ensemble"] = ensemble.measure(steps=10, warmup=3, precision="tf32x3")
        print(json.dumps(out))
    grp.close()


DTYPES = {"fp64": "f64", "fp32": "f32", "tf32x3": "f32+tf32x3", "bf16x3": "f32+bf16x3",
          "f64_tf32x3": "f64 (Legendre m>=1 tf32x3)", "f64_eddy": "f64 (eddy FFT f32, Legendre m>=1 tf32x3)"}
SIMPLE_PREC = ("fp64", "fp32", "tf32x3", "bf16x3")
COMPARE = ["f64_eddy", "f64_tf32x3", "tf32x3", "bf16x3", "fp32"]
GEMM_PROFILE = "profiles/tc_gemm_f_T574L64_tf32x3.md"


def profiled_gemm_traffic():
    """DRAM bytes per k_tc_gemm_f launch at T574L64 from the committed ncu
    summary (its 'Average over the four launches of a stage' line)."""
    import re

    path = os.path.join(ROOT, GEMM_PROFILE)
    if not os.path.exists(path):
        return None
    m = re.search(r"Average over the four launches of a stage: ([0-9.]+) GB per launch", open(path).read())
    return float(m.group(1)) * 1e9 if m else None


def precision_modes(ctx, st, nsteps, dt, stream, barrier, grp, headline):
    """FP64 and each fast mode from the same state, nsteps steps each; the
    first two steps (eager, then graph capture) are not timed."""
    import torch

    from gdpy.error_study import field_errors

    def run(prec):
        g = ctx(prec)
        g.advance(2)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.advance(nsteps - 2)
        e1.record(stream)
        barrier()
        ms = grp.max_over_ranks(e0.elapsed_time(e1)) / (nsteps - 2)
        x = g.get_state()
        g.close()
        return ms, x

    ms64, s64 = run("fp64")
    out = dict(steps=nsteps, hours=nsteps * dt / 3600.0, fp64_ms_per_step=ms64, fp64_days_per_day=dt / (ms64 * 1e-3),
               note="max-norm and L2 relative error per spectral field after the stated steps; div also against "
                    "the vorticity scale", modes={})
    for p in [headline] + [m for m in COMPARE if m != headline]:
        if p == "fp64":
            continue
        ms, x = run(p)
        e = field_errors(x, s64)
        out["modes"][p] = dict(ms_per_step=ms, days_per_day=dt / (ms * 1e-3), speedup_vs_fp64=ms64 / ms,
                               rel_err={k: v["max_rel"] for k, v in e.items()},
                               rel_err_l2={k: v["l2_rel"] for k, v in e.items()},
                               div_rel_err_vrt_scale=e["div"]["max_rel_vrt_scale"])
    return out


def config_rows(full_cpu=False):
    """The two smaller configurations in simulated days/day: the plain FP64
    step on the GPU over one simulated day (T42L20, dt 1200 s: 72 steps;
    T126L64 ntrac 3, dt 600 s: 144 steps) and the FP64 CPU oracle on all host
    threads, over a bounded sample (T42L20: one day; T126L64: 3 steps) or,
    with full_cpu, over the reference configurations' full runs (T42L20 10
    days, T126L64 one day)."""
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    from gdpy import core, inputs

    rows = {}
    for name, day_steps, cpu_sample, cpu_full in (("T42L20", 72, 72, 720), ("T126L64", 144, 3, 144)):
        T, nlon, nlat, L, nt, dt = WORKLOADS[name]
        ak, bk = inputs.hybrid_coords(L)
        st = make_state(name, seed=0)
        trc = st["trc"] if nt else None
        g = core.Dycore(T, nlon, nlat, L, ak, bk, ntrac=nt, dt=dt, precision="fp64")
        stream = torch.cuda.Stream()
        g.set_stream(stream.cuda_stream)
        g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=trc)
        g.advance(3)
        g.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.advance(day_steps)
        e1.record(stream)
        g.sync()
        gms = e0.elapsed_time(e1) / day_steps
        g.close()
        nth = os.cpu_count()
        o = oracle_py.Oracle(T, nlon, nlat, L, ak, bk, ntrac=nt, dt=dt, nthreads=nth)
        o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=trc)
        o.advance(1)
        n = cpu_full if full_cpu else cpu_sample
        t0 = time.perf_counter()
        o.advance(n)
        cs = (time.perf_counter() - t0) / n
        del o
        rows[name] = dict(gpu_fp64_days_per_day=dt / (gms * 1e-3), gpu_fp64_ms_per_step=gms,
                          gpu_steps=day_steps, cpu_days_per_day=dt / cs, cpu_s_per_step=cs, cpu_steps=n,
                          cpu_threads=nth, cpu_kind="port (FP64 oracle)",
                          gpu_over_cpu=(dt / (gms * 1e-3)) / (dt / cs))
    return rows


def dcmip_rate(precision, steps=10, warmup=3):
    """The DCMIP simple-physics plugin (src/phy_run_simple.f90 around
    src/simple_physics_v5_1.f90) in the full step: the moist baroclinic wave
    with surface fluxes and boundary-layer mixing (dcmip 43; DCMIP-2012 test 4
    initial state from gd_dcmip_ics; 3 tracers) at T574L64, dt 150 s.  The
    column kernel's roofline counts the algorithmic bytes of one launch: Tv,
    q, u, v read and their four increments written at every level, plus ps
    read, precipitation and precipitable water written and the accumulated
    precipitation read and written: (8 L + 5) nlat nlon words."""
    import torch

    from gdpy import core, inputs

    T, nlon, nlat, L, nt, dt = 574, 1152, 576, 64, 3, 150.0
    ak, bk = inputs.hybrid_coords(L)
    g = core.Dycore(T, nlon, nlat, L, ak, bk, ntrac=nt, dt=dt, precision=precision, heldsuarez=False, dry=False,
                    dcmip=43)
    stream = torch.cuda.Stream()
    g.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    g.dcmip_ics(43)
    ics_s = time.perf_counter() - t0
    # The analytic state is subsaturated everywhere; humidity x1.6 (as in the parity tests) makes the
    # large-scale condensation branch act from the first step, so the timed column kernel runs it.
    x = g.get_state()
    trc = x["trc"].copy()
    trc[0] *= 1.6
    g.set_state(x["vrt"], x["div"], x["tv"], x["lnps"], trc=trc, topo=g.get_topo())
    g.advance(warmup)
    g.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    g.advance(steps)
    e1.record(stream)
    g.sync()
    ms = e0.elapsed_time(e1) / steps
    ph = g.profile_step()
    rsize = 8 if precision == "fp64" else 4
    byt = (8 * L + 5) * nlat * nlon * rsize
    cms = ph["column_physics"]
    hbm = peaks()
    achieved = byt / (cms * 1e-3) / 1e9
    apcp = g.get_grid("apcp")
    g.close()
    return dict(workload="DCMIP-2012 4-3 moist baroclinic wave (humidity x1.6, condensing), simple physics, "
                         "T574L64 ntrac 3 dt 150 s",
                precision=precision, ms_per_step=ms, days_per_day=dt / (ms * 1e-3), initial_state_s=ics_s,
                phases_ms=ph, max_accumulated_precip_mm=float(apcp.max()),
                column_kernel=dict(kernel="k_simple_physics", bound="hbm", ms=cms, bytes=byt, achieved=achieved,
                                   peak=hbm["hbm"], unit="GB/s", frac=achieved / hbm["hbm"],
                                   peak_source=hbm["src"]))


def closure_rate(precision, steps=20, warmup=3, train_steps=50):
    """The learned per-column closure's configuration: a Held-Suarez T62L64
    step (dt 1200 s) with and without a closure net of the configured shape
    (193 -> 256 GELU x 3 -> 192, BF16 weights, FP32 accumulation; seeded
    weights and a unit normalisation: the cost does not depend on the values),
    and the training throughput of the library's forward + backward + Adam
    kernels on minibatches of 4096 columns.  Flops: 2 x 230 592 per column
    and inference, 6 x per column and training step."""
    import torch

    from gdpy import core, inputs

    T, nlon, nlat, L, dt = 62, 192, 94, 64, 1200.0
    ak, bk = inputs.hybrid_coords(L)
    st = inputs.hs_rest_state(T, L, seed=3)
    stream = torch.cuda.Stream()
    res = {}
    net = core.Mlp(3 * L + 1, 256, 3, 3 * L, seed=2)
    net.set_norm(np.zeros(3 * L + 1), np.ones(3 * L + 1), np.zeros(3 * L), np.full(3 * L, 1e-6))
    for name, use in (("plain", None), ("closure", net)):
        g = core.Dycore(T, nlon, nlat, L, ak, bk, ntrac=0, dt=dt, precision=precision)
        g.set_stream(stream.cuda_stream)
        g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
        if use is not None:
            g.set_closure(use)
        g.advance(warmup)
        g.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.advance(steps)
        e1.record(stream)
        g.sync()
        res[name] = e0.elapsed_time(e1) / steps
        if use is not None:
            g.set_closure(None)
        g.close()
    ncol = nlon * nlat
    x = torch.randn(4096, 3 * L + 1, device="cuda")
    t = torch.randn(4096, 3 * L, device="cuda")
    for _ in range(3):
        net.train_step(x, t, 1e-4)
    net.sync()
    t0 = time.perf_counter()
    for _ in range(train_steps):
        net.train_step(x, t, 1e-4)
    net.sync()
    tr = (time.perf_counter() - t0) / train_steps
    flop = 2.0 * net.nparams
    return dict(workload="Held-Suarez T62L64 dt 1200 s, closure net 193-256x3-192", precision=precision,
                ms_per_step_plain=res["plain"], ms_per_step_closure=res["closure"],
                closure_ms_per_step=res["closure"] - res["plain"],
                inference_tflops=flop * ncol / ((res["closure"] - res["plain"]) * 1e-3) / 1e12,
                train_ms_per_batch4096=tr * 1e3, train_columns_per_s=4096 / tr,
                train_tflops=3 * flop * 4096 / tr / 1e12)


def pattern_generator_rate(steps=40, cpu_steps=3):
    """The stochastic pattern generator (src/patterngenerator.f90) at T574:
    one AR(1) pattern (SPPT-like: 250 km, tau 6 h, dt 150 s), GPU steps per
    second through the C ABI, and the single-precision CPU oracle's on the
    same stream.  Each step draws 2 nlm = 331200 Gaussians from one
    Mersenne-twister stream, which bounds it (a sequential recurrence), not
    HBM."""
    import torch

    from gdpy import core

    jcap, args = 574, (250e3, 150.0, 21600.0, 0.8, 7)
    g = core.Pattern(*args, jcap)
    g.start()
    g.advance(2)
    g.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(torch.cuda.default_stream())
    g.advance(steps)
    e1.record(torch.cuda.default_stream())
    g.sync()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    g.close()
    out = dict(workload="T574 one pattern", ms_per_step=ms, steps_per_s=1e3 / ms,
               gaussians_per_s=2 * (jcap + 1) * (jcap + 2) / 2 * 1e3 / ms)
    try:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py

        o = oracle_py.PatternOracle(*args, jcap)
        o.start()
        t0 = time.perf_counter()
        o.advance(cpu_steps)
        out["cpu_port_ms_per_step"] = (time.perf_counter() - t0) * 1e3 / cpu_steps
    except Exception as e:  # the oracle is optional here
        out["cpu_port_ms_per_step"] = None
        out["cpu_note"] = str(e)[:120]
    return out


def cpu_baseline(name, nthreads=None, steps=1):
    """FP64 CPU restatement of the reference step (the oracle) on the host
    cores: full steps of the workload (all levels), timed one by one after
    the instance is built and its state set."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    from gdpy import inputs

    T, nlon, nlat, L, nt, dt = WORKLOADS[name]
    nthreads = nthreads or os.cpu_count()
    ak, bk = inputs.hybrid_coords(L)
    st = make_state(name, seed=0)
    o = oracle_py.Oracle(T, nlon, nlat, L, ak, bk, ntrac=nt, dt=dt, nthreads=nthreads)
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"], trc=st["trc"] if nt else None)
    secs = []
    for _ in range(steps):
        t0 = time.perf_counter()
        o.advance(1)
        secs.append(time.perf_counter() - t0)
    sec = statistics.median(secs)
    return dict(value=dt / sec, unit="simulated days/day", cores=nthreads, kind="port",
                sample=f"{steps} full step(s) of {name} (all {L} levels) on {nthreads} threads",
                seconds_per_step=sec, seconds=secs)


def reference_arm(args):
    """The CPU reference arm: the FP64 restatement of the reference step on
    the host cores, one instance, one warm-up step, then at least 3 (at most
    --steps) full steps timed one by one.  Each is a full step of the
    workload, so the line's steps are steps that ran."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    oracle_py.build()
    T, nlon, nlat, L, nt, dt = WORKLOADS[args.workload]
    n = max(3, min(args.steps, args.ref_steps))
    warm = 1
    cb = cpu_baseline(args.workload, steps=warm + n)
    secs = cb["seconds"][warm:]
    sec = statistics.median(secs)
    v = dt / sec
    cb.update(value=v, seconds_per_step=sec, seconds=secs,
              sample=f"{n} full steps of {args.workload} (all {L} levels) after {warm} warm-up step, "
                     f"one instance, {cb['cores']} threads")
    print(json.dumps({
        "metric": METRIC, "value": v, "unit": "simulated days/day", "n_gpus": 0, "steps": n,
        "warmup": warm, "steps_requested": args.steps, "warmup_requested": args.warmup,
        "ms_per_step": 1e3 * sec, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": "synthetic (seeded balanced jet, Held-Suarez forcing)",
        "config": {"workload": args.workload, "ntrunc": T, "grid": f"{nlon}x{nlat}", "nlev": L, "ntrac": nt,
                   "dt_s": dt, "precision": "fp64"},
        "cpu_baseline": cb,
        "e2e": {"value": v, "unit": "simulated days/day", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "FP64 C++ restatement of the reference algorithm (OpenMP over levels, per-level transforms as "
                "the reference calls SHTns); the reference's Fortran+SHTns build cannot be made on this image "
                "(no Fortran compiler, no SHTns/FFTW). Full steps are timed, so the arm runs at most "
                "--ref-steps of the requested steps.",
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gd", choices=["gd", "reference"])
    ap.add_argument("--precision", default="tf32x3", choices=list(DTYPES))
    ap.add_argument("--workload", default="T574L64", choices=list(WORKLOADS))
    ap.add_argument("--err-steps", type=int, default=24,
                    help="steps every precision mode and the FP64 step advance for the error comparison (0: none)")
    ap.add_argument("--ref-steps", type=int, default=3, help="full CPU steps the reference arm times (>= 3)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the T42L20 / T126L64 days/day rows")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the 32-member ensemble side measurement")
    ap.add_argument("--config-cpu", action="store_true",
                    help="time the CPU rows over the full runs (T42L20 10 days, T126L64 one day)")
    ap.add_argument("--no-dcmip", action="store_true", help="skip the DCMIP simple-physics side measurement")
    ap.add_argument("--no-closure", action="store_true", help="skip the learned-closure side measurement")
    ap.add_argument("--no-autotune", action="store_true",
                    help="step the headline context with the default tile shapes instead of the autotuner's")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gd":
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
