"""The multi-GPU mode of the benchmark is replicas only (the element path has
no exchange step on one GPU's layout): every rank runs the same workload and
the job's rate is all ranks' DOF updates over the slowest rank's time.  The
rank bookkeeping and the max-over-ranks reduction run here as two gloo ranks
on the CPU."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    ms = bench.max_over_ranks(10.0 + 5.0 * r, dist, "cpu")
    out.put((r, w, local, ms, bench.whole_job_rate(1000, w, ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[:3] for x in res] == [(0, 2, 0), (1, 2, 1)]
    for _, _, _, ms, rate in res:
        assert ms == 15.0
        assert rate == pytest.approx(2 * 1000 / 15e-3)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(10, 1, 2.0) == pytest.approx(5000.0)
