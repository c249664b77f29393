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
