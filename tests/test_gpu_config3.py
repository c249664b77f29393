"""Config 3 at its stated size: MaxCut QAOA p=2 light-cone terms of a seeded
3-regular 50-vertex graph whose seeded stochastic ordering (the reference's
ParallelContract, src/ContractionTools.h:219-388, with a fixed seed) reaches a
qTorch rank-13 or rank-14 intermediate -- 2^26 or 2^28 complex elements, the
"rank 26-28" of dimension-2 legs.  Such plans exceed the grouped interpreter
and run step by step; their large complex64 steps, a rank 11-14 tensor met by
a gate-sized one, are bound by HBM bandwidth and take the streaming kernel
(or the tiled kernel).  FP64 must equal the oracle's replay of the same sequence bit for
bit; the mixed form must stay within 1e-6 of FP64, on values far from zero."""
import pytest

import qtorch_gb300 as qg
from oracle import port

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6
ANGLES = [0.3, 0.8, 0.6, 0.2]   # beta_1, beta_2, gamma_1, gamma_2


def term(edge):
    dgf = qg.random_regular_graph(50, 3, seed=3)
    return qg.qaoa_term_text(dgf, 2, ANGLES, edge)


def test_rank13_term_fp64_bit_exact_and_mixed_within_tolerance(ctx):
    q, m = term(16)
    plan = qg.Plan(q, m, ordering="stochastic", seed=11, ctx=ctx)
    assert plan.peak_rank == 13
    v64 = plan.execute(qg.FP64)
    st0 = ctx.stream_steps
    vmx = plan.execute(qg.MIXED)
    assert ctx.stream_steps >= st0 + 3, "the rank 11-13 steps did not take the streaming kernel"
    v_or, flops = port.replay_value(q, m, plan.sequence())
    assert flops == plan.flops
    assert v64 == v_or
    assert abs(v64) > 1e-3
    assert abs(vmx - v64) <= MIXED_TOL


@pytest.mark.parametrize("edge,seed", [(5, 533), (72, 542)])
def test_rank14_terms_mixed_within_tolerance(ctx, edge, seed):
    q, m = term(edge)
    plan = qg.Plan(q, m, ordering="stochastic", seed=seed, ctx=ctx)
    assert plan.peak_rank == 14
    v64 = plan.execute(qg.FP64)
    st0 = ctx.stream_steps
    vmx = plan.execute(qg.MIXED)
    assert ctx.stream_steps >= st0 + 2
    assert abs(v64) > 1e-3
    assert abs(vmx - v64) <= MIXED_TOL
    # a second run gives the same value (no state left behind by the first)
    assert plan.execute(qg.MIXED) == vmx
