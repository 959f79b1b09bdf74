"""Multi-GPU path on the CPU (gloo, two ranks).

bench.py --gpus N runs one process per GPU.  A single survey runs as
independent replicas (each rank its own seeded survey, no data-path
collective); the batched workload is partitioned: every rank solves a
disjoint subset of the same models, balanced by observations, and the
reported time is the slowest rank's.  These tests run that rank logic with
the gloo backend on 127.0.0.1, solving a tiny batch with the oracle (the CPU
restatement of the solver) on each rank: every model is solved exactly once
and the gathered per-model results equal the single-rank solves."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _tiny_batch():
    """Six small lawnmower models of uneven size (the batched workload's
    generator, scaled down)."""
    from stitch_ba import survey
    return [m[0] for m in survey.batched_models(6, seed=3, cam_range=(6, 14), ppc_range=(40, 80))]


def _solve(p):
    import ba_oracle as O
    q = p.copy()
    r = O.bundle_adjust(q, 8, 1.0, n_threads=1)
    return r.iterations, r.final_cost, q.center.copy(), q.points.copy()


def _worker(rank, ws, port, out):
    import sys
    for d in (ROOT, os.path.join(ROOT, "aerial-3d-model_gb300"), os.path.join(ROOT, "oracle")):
        sys.path.insert(0, d)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        import bench
        t = bench.max_over_ranks(10.0 + rank, ws, device="cpu")
        seed = bench.rank_seed(1, rank)
        ps = _tiny_batch()
        part = bench.partition_models([p.n_obs for p in ps], ws)[rank]
        mine = {i: _solve(ps[i]) for i in part}
        gathered = [None] * ws
        dist.all_gather_object(gathered, mine)
        solves = sum(len(g) for g in gathered)
        total = bench.sum_over_ranks(float(len(part)), ws, device="cpu")
        out.put((rank, t, seed, part, gathered if rank == 0 else None, solves, total))
    finally:
        dist.destroy_process_group()


def test_two_ranks_partition_the_batch_and_report_the_slowest_rank():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in range(ws)), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [11.0, 11.0]   # max over ranks on every rank
    assert len({r[2] for r in res}) == ws        # single-survey replicas: a seed each
    ps = _tiny_batch()
    parts = [r[3] for r in res]
    # every model on exactly one rank
    assert sorted(i for p in parts for i in p) == list(range(len(ps)))
    assert all(r[5] == len(ps) and r[6] == len(ps) for r in res)
    # per-model results gathered on rank 0 equal the single-rank solves
    gathered = {}
    for g in res[0][4]:
        assert not set(g) & set(gathered)
        gathered.update(g)
    for i, p in enumerate(ps):
        it, cost, centre, points = _solve(p)
        git, gcost, gcentre, gpoints = gathered[i]
        assert git == it and gcost == cost
        assert np.array_equal(gcentre, centre) and np.array_equal(gpoints, points)


def test_partition_balances_observations():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    sizes = [100, 90, 80, 10, 10, 10, 5]
    parts = bench.partition_models(sizes, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(sizes)))
    loads = [sum(sizes[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(sizes[3:])  # greedy by size: within one small model
    assert bench.partition_models(sizes, 1) == [list(range(len(sizes)))]
    # more ranks than models: the extra ranks get nothing
    assert sum(1 for p in bench.partition_models([5, 4], 4) if p) == 2


def test_single_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.sum_over_ranks(3.5, 1) == 3.5


@pytest.mark.parametrize("ws", [1, 2, 8])
def test_rank_workload_of_the_batch_covers_every_model(ws):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    from stitch_ba import survey
    sizes = [m[0].n_obs for m in survey.batched_models(12, seed=5, cam_range=(6, 12),
                                                        ppc_range=(30, 50))]
    parts = bench.partition_models(sizes, ws)
    assert len(parts) == ws
    assert sorted(i for p in parts for i in p) == list(range(12))
