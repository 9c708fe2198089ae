"""The multi-GPU form of bench.py is replicas only: every rank advances its own
volume and the job's time is the slowest rank's.  Two `gloo` ranks on the
CPU check that aggregation (max over ranks, whole-job frames/s) and that the
reference arm leaves ranks other than 0 idle."""
import importlib.util
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _worker(rank, world, port, out):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        b = _bench()
        seconds = b.max_over_ranks(1.0 + rank, world, "cpu")   # rank 1 is the slow one
        # the reference arm: only rank 0 works (args None would fail there)
        ref = b.run_reference(None, rank, world) if rank != 0 else None
        out.put((rank, seconds, b.job_rate(world, 30, seconds), ref))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank(built):
    mp = pytest.importorskip("torch.multiprocessing")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, seconds, rate, ref in res:
        assert seconds == 2.0                 # both ranks see the slowest rank's time
        assert rate == 2 * 30 / 2.0           # frames of all replicas over that time
        assert ref is None and rank in (0, 1)


def test_single_rank_needs_no_process_group():
    b = _bench()
    assert b.max_over_ranks(1.25, 1, "cpu") == 1.25
    assert b.job_rate(1, 30, 0.15) == pytest.approx(200.0)
