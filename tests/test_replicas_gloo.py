"""The multi-GPU path of bench.py is replicas only: every rank runs the whole workload,
the job's time is the slowest rank's, its throughput the units of all ranks over that
time, and under the reference arm only rank 0 works.  Checked with two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 * (rank + 1)  # rank 1 is the slow one
    out[rank] = (bench.max_over_ranks(ms, dist, "cpu"), bench.job_value(1000, world, 5, bench.max_over_ranks(ms, dist, "cpu")))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_value_with_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0] == res[1]
    ms, value = res[0]
    assert ms == 20.0                                  # the slower rank's time
    assert value == pytest.approx(2 * 1000 * 5 / 0.020)  # both ranks' units over it


def test_single_process_and_reference_arm_on_other_ranks(capsys):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5

    class Args:
        warmup, steps, points = 3, 1, bench.N_POINTS
    bench.run_reference(Args, world=2, rank=1)  # rank 1 of the reference arm does no work
    assert capsys.readouterr().out == ""


def test_reference_arm_line_on_rank_zero(capsys, monkeypatch):
    """Rank 0 of the reference arm prints one JSON line with the GPU arm's metric and unit,
    the CPU baseline it timed (RNNG's landmark pipeline restated in C, kind "port"), no
    host-device bytes, and the same edges as the brute-force restatement (a 4,000-point
    prefix of the descriptors stands in for the 100,000 of a bench run)."""
    import json
    import sys
    sys.path.insert(0, ROOT)
    import bench
    import oracle
    from rnng_gb300 import synth
    x = synth.descriptor(n=4000, d=bench.DIM)
    monkeypatch.setattr(bench, "workload", lambda n=bench.N_POINTS: (x, synth.EPS_K2))

    class Args:
        warmup, steps, points, workload = 3, 2, bench.N_POINTS, "k2"
    bench.run_reference(Args, world=1, rank=0)
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True and d["steps"] == 2 and d["warmup"] == 3 and d["value"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1
    assert "first 4000 points" in cb["sample"]
    u, _, _ = oracle.eps_graph_l2(x, synth.EPS_K2)
    assert f"{u.size} edges" in cb["sample"]
