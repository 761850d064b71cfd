"""The N > 1 path of bench.py (replicas, one rank per GPU): each rank times
its own copy of the workload, the timed region is reduced with MAX over
ranks, and the job rate is all ranks' units over that time.  Run here as two
gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [12.5, 17.0][rank]                       # the second rank is slower
    worst = bench.max_over_ranks(ms, dist, torch.device("cpu"))
    dist.barrier()
    out[rank] = (worst, bench.whole_job_rate(world, 98304, worst * 1e-3))
    dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(world):
        worst, rate = res[r]
        assert worst == 17.0
        assert rate == pytest.approx(2 * 98304 / 17.0e-3)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.25, None, None) == 3.25
    assert bench.whole_job_rate(1, 1000, 0.5) == 2000.0
