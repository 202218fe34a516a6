"""bench.py's whole-job figures over ranks (replicas, weak scaling), on two gloo ranks on
the CPU: the step times are the maximum over ranks and the effective samples per step
the sum over ranks, so `value` is whole-job throughput."""

import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank 0: 10 ms per step (e2e 11 ms), tau 1; rank 1: 12 ms (e2e 15 ms), tau 2
    ms, ms_e2e, tau = (10.0, 11.0, 1.0) if rank == 0 else (12.0, 15.0, 2.0)
    q.put((rank, bench.whole_job(ms, ms_e2e, 100, tau, True)))
    dist.barrier()
    dist.destroy_process_group()


def test_whole_job_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    eff = 100 / 1.0 + 100 / 2.0  # effective samples per step, summed over ranks
    for r in (0, 1):
        ms, ms_e2e, value, e2e = res[r]
        assert ms == 12.0 and ms_e2e == 15.0
        assert value == pytest.approx(eff / 12e-3) and e2e == pytest.approx(eff / 15e-3)


def test_whole_job_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    ms, ms_e2e, value, e2e = bench.whole_job(20.0, 25.0, 16384, 1.0, False)
    assert (ms, ms_e2e) == (20.0, 25.0)
    assert value == pytest.approx(16384 / 20e-3) and e2e == pytest.approx(16384 / 25e-3)
