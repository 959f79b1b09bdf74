"""Multi-GPU path on the CPU (gloo, two ranks): replicas only.

bench.py --gpus N runs one process per GPU, each solving its own survey
(no data-path collective); the reported time is the slowest rank's and the
throughput counts every rank's solves.  These tests run the rank logic with
the gloo backend on 127.0.0.1."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        import bench
        t = bench.max_over_ranks(10.0 + rank, ws, device="cpu")
        seed = bench.rank_seed(1, rank)
        out.put((rank, t, seed))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_report_the_slowest_rank():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [11.0, 11.0]   # max over ranks on every rank
    assert len({r[2] for r in res}) == ws        # each replica its own survey


def test_single_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
