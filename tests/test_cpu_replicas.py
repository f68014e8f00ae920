"""The replica path of bench.py (torchrun, N > 1: one independent replica per GPU,
no data-path collective) on two gloo ranks on the CPU: the timed region is the
slowest rank's, the value counts every rank's iterations, and the reference arm
runs on rank 0 only."""
import os
import socket
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t_max = bench.max_over_ranks(10.0 + 5.0 * rank, world)
        rate = bench.replicas_rate(world, 10, t_max)
        args = types.SimpleNamespace(steps=2, warmup=1, workload="small", ref_budget=1.0)
        ref = bench.run_reference(args, rank, world) if rank != 0 else "skipped"
        dist.barrier()
        q.put((rank, t_max, rate, ref))
    finally:
        dist.destroy_process_group()


def test_replica_timing_and_reference_arm_on_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_max, rate, ref in out:
        assert t_max == 15.0                      # the slowest rank's time, on every rank
        assert abs(rate - 2 * 10 / 0.015) < 1e-9  # iterations of both replicas / that time
    assert out[1][3] is None                      # rank 1 does no reference work


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replicas_rate(1, 4, 2000.0) == 2.0
