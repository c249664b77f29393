"""A plan from the ordering search runs bit-exact with the oracle's replay of
its recorded sequence (FP64) and within 1e-6 in the mixed form."""
import pytest

import qtorch_gb300 as qg
from oracle import port

pytestmark = pytest.mark.gpu


def test_searched_plan_replays_bit_exact(ctx):
    dgf = qg.random_regular_graph(50, 3, seed=3)
    q, m = qg.qaoa_term_text(dgf, 2, [0.3, 0.8, 0.6, 0.2], 16)
    plan = qg.Plan(q, m, ordering="search", seed=1, tries=25, ctx=ctx)
    v64 = plan.execute(qg.FP64)
    v_or, flops = port.replay_value(q, m, plan.sequence())
    assert flops == plan.flops
    assert v64 == v_or
    assert abs(plan.execute(qg.MIXED) - v64) <= 1e-6


def test_sharded_plans_on_one_rank_match_one_batch(ctx):
    """evaluate_plans_sharded on a one-rank group is the plain batch."""
    import os
    import socket

    import torch.distributed as dist

    from qtorch_gb300 import shard
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=0, world_size=1)
    try:
        dgf = qg.random_regular_graph(20, 3, seed=9)
        plans = [qg.Plan(*qg.qaoa_term_text(dgf, 1, [0.4, 1.2], e), ordering="linegraph", ctx=ctx)
                 for e in range(qg.qaoa_num_edges(dgf))]
        got = shard.evaluate_plans_sharded(plans, qg.FP64, ctx)
        b = qg.Batch(ctx)
        for p in plans:
            b.add(p)
        assert list(got) == list(b.execute(qg.FP64))
    finally:
        dist.destroy_process_group()
