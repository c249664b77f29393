"""The multi-rank logic of bench.py on CPU (gloo, world size 2): every rank
evaluates its own QAOA terms (weak scaling, no data-path collective) and the
job time is the max over ranks."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench
    import qtorch_gb300 as qg
    from oracle import port as oport
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dgf = qg.random_regular_graph(20, 3, seed=5)
    pts = bench.angle_points(1000 + rank, 2)
    terms = bench.build_terms(dgf, pts[0])[:4]
    vals = []
    for q, m in terms:
        seq = qg.Plan(q, m, ordering="linegraph", symbolic=True).sequence()
        v, _ = oport.replay_value(q, m, seq)
        vals.append(v.real)
    t = bench.max_over_ranks([1.0 + rank, 5.0 - rank], world, "cpu")
    out.put((rank, t, vals, pts[0]))
    dist.destroy_process_group()


def test_two_ranks_weak_scaling_and_max_time():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, t0, v0, a0), (r1, t1, v1, a1) = res
    assert t0 == t1 == [2.0, 5.0]
    assert a0 != a1                      # each rank has its own parameter points
    assert all(abs(x) <= 1.0 + 1e-12 for x in v0 + v1)
