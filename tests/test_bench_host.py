"""The bench line's host-side inputs, on the CPU: the roofline's peaks come
from the committed peak measurements, its DRAM traffic from the committed ncu
summary of the GEMM, and the algorithmic bytes and flop from the workload's
shape alone."""
import json
import os

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_peaks_are_the_measured_ones():
    pk = bench.peaks()
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        m = json.load(open(path))
        assert pk["src"] == "measured"
        assert pk["hbm"] == m["hbm_gbs"] and pk["bf16"] == m["bf16_tflops"]
    else:
        assert pk["src"] == "fallback"


def test_gemm_traffic_comes_from_the_committed_profile():
    tr = bench.profiled_gemm_traffic()
    assert tr is not None, bench.GEMM_PROFILE
    # the summary's per-launch average, in bytes: GB-sized at T574L64
    assert 1e9 < tr < 1e10


def test_work_counts_of_the_headline_workload():
    T, nlon, nlat, L, nt, _ = bench.WORKLOADS["T574L64"]
    wc = bench.work_counts(T, nlon, nlat, L, nt, 4)
    nlm = (T + 1) * (T + 2) // 2
    assert wc["scalar_flop"] == 2.0 * nlm * nlat
    # 15 Legendre launches per step, each moving GBs of operands, tables and results
    assert wc["legendre_launches"] == 15
    per_launch = wc["legendre_bytes"] / wc["legendre_launches"]
    assert 1e9 < per_launch < 5e9
    # FP64 operands double the array bytes, the tables are kept once instead of as hi + lo
    w8 = bench.work_counts(T, nlon, nlat, L, nt, 8)
    assert w8["c2r_bytes"] > wc["c2r_bytes"] and w8["col_bytes"] == 2 * wc["col_bytes"]
    assert w8["legendre_flop"] == wc["legendre_flop"]
