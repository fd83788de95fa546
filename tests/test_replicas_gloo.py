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
