"""Multi-rank host logic on CPU: two gloo ranks, replicas only.

The multi-GPU path runs one independent ensemble member per rank.  These
tests drive the same host code (``gdpy.replicas.ReplicaGroup``, used by
bench.py with NCCL) with the gloo backend on CPU at world size 2.  Each rank
advances its own seeded member with the CPU oracle (the GPU path is covered
by the GPU tests); the checks are the timing reduction (MAX over ranks),
the weak-scaling aggregate, per-rank seeding and the absence of any exchange
of model data.
"""
import json
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, outdir):
    for p in (ROOT, os.path.join(ROOT, "gfs-dycore_gb300"), os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import oracle_py
    from gdpy import inputs
    from gdpy.replicas import ReplicaGroup

    grp = ReplicaGroup("gloo")
    T, nlev = 21, 8
    ak, bk = inputs.hybrid_coords(nlev)
    o = oracle_py.Oracle(T, 64, 32, nlev, ak, bk, dt=1200.0)
    st = inputs.hs_rest_state(T, nlev, seed=grp.member_seed(100))
    o.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    grp.barrier()
    o.advance(2)
    grp.barrier()
    s = o.get_state()
    # a stand-in elapsed time that differs by rank: the reduction must pick the slowest
    elapsed = 1.0 + rank
    tmax = grp.max_over_ranks(elapsed)
    rate = grp.job_rate(2 * 1200.0 / 86400.0, tmax)  # simulated days per wall second, whole job
    res = dict(rank=rank, world=grp.world, backend=grp.backend, root=grp.is_root, seed=grp.member_seed(100),
               tmax=tmax, rate=rate, vrt_norm=float(np.abs(s["vrt"]).sum()))
    with open(os.path.join(outdir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)
    grp.close()


def test_two_gloo_ranks_replicas(oracle_mod, tmp_path):
    import torch.multiprocessing as mp

    oracle_mod.build()
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r = [json.load(open(tmp_path / f"rank{i}.json")) for i in range(2)]
    assert [x["world"] for x in r] == [2, 2]
    assert [x["backend"] for x in r] == ["gloo", "gloo"]
    assert [x["root"] for x in r] == [True, False]
    # the timed region ends with the slowest rank
    assert r[0]["tmax"] == r[1]["tmax"] == 2.0
    # weak scaling: both ranks advanced 2 steps of 1200 s in at most 2 s
    np.testing.assert_allclose(r[0]["rate"], 2 * (2 * 1200.0 / 86400.0) / 2.0, rtol=1e-15)
    # independent members: different seeds, different states
    assert r[0]["seed"] != r[1]["seed"]
    assert r[0]["vrt_norm"] != r[1]["vrt_norm"]


def test_single_process_group_is_trivial():
    from gdpy.replicas import ReplicaGroup

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        assert k not in os.environ or os.environ[k] in ("0", "1")
    g = ReplicaGroup("gloo")
    assert g.world == 1 and g.is_root and g.dist is None
    assert g.max_over_ranks(3.5) == 3.5
    assert g.job_rate(1.0, 0.5) == 2.0
    g.close()


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        workload, steps, warmup, cpu_levels = "T42L20", 1, 0, 4

    def boom(*a, **k):
        raise AssertionError("rank 1 must not run the reference arm")

    monkeypatch.setattr(bench, "cpu_baseline", boom)
    bench.reference_arm(A())
    assert capsys.readouterr().out == ""
