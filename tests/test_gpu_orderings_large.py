"""Requests of the serving range on the GPU: plans from the size-greedy and
automatic orderings run bit-exact with the oracle's replay of their recorded
sequence (FP64); slicings of more than one chunk of slices add up to the
unsliced value; the server's work cap refuses what it must and serves the
rest."""
import pytest

import qtorch_gb300 as qg
from qtorch_gb300.circuits import qft_measure_text, qft_text, random_circuit_text
from oracle import port

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ordering", ["greedy", "auto"])
@pytest.mark.parametrize("circuit", ["rand", "qft"])
def test_plan_replays_bit_exact(ctx, ordering, circuit):
    q, m = ((random_circuit_text(10, 8, 3), "Z") if circuit == "rand" else (qft_text(7, 2), qft_measure_text(7)))
    plan = qg.Plan(q, m, ordering=ordering, seed=2, ctx=ctx)
    v64 = plan.execute(qg.FP64)
    v_or, flops = port.replay_value(q, m, plan.sequence())
    assert flops == plan.flops
    assert v64 == v_or
    assert abs(v64) > 1e-3
    assert abs(plan.execute(qg.MIXED) - v64) <= 1e-6


def test_greedy_plan_of_a_20_qubit_circuit(ctx):
    """A 20-qubit depth-8 random circuit (whose line graph the min-fill walk
    also handles) under the greedy order: FP64 against the mixed form."""
    plan = qg.Plan(random_circuit_text(20, 8, 7), "Z", ordering="greedy", ctx=ctx)
    v64 = plan.execute(qg.FP64)
    assert abs(plan.execute(qg.MIXED) - v64) <= 1e-6


@pytest.mark.parametrize("prec", [qg.FP64, qg.MIXED])
def test_slicing_in_chunks_adds_up(ctx, prec):
    plan = qg.Plan(qft_text(8, 2), qft_measure_text(8), ordering="linegraph", ctx=ctx)
    want = plan.execute(qg.FP64)
    assert abs(want) > 1e-3
    s = plan.slice(plan.workspace_bytes(prec) // 20, prec, 16)
    assert s.num_slices > 4096
    tol = 1e-12 if prec == qg.FP64 else 1e-6
    assert abs(s.execute(prec) - want) <= tol * max(1.0, abs(want))


def test_work_cap_refuses_and_serves_the_rest(ctx):
    big = qg.Plan(random_circuit_text(12, 10, 1), "Z", ordering="auto", ctx=ctx)
    dgf = qg.random_regular_graph(20, 3, seed=9)
    small = [qg.Plan(*qg.qaoa_term_text(dgf, 1, [0.4, 1.1], e), ordering="linegraph", ctx=ctx) for e in range(4)]
    srv = qg.Server(max_inflight=8, precision=qg.MIXED, ctx=ctx, max_macs=big.flops - 1)
    try:
        with pytest.raises(qg.Refused):
            srv.submit(big)
        tickets = [srv.submit(p) for p in small]
        srv.drain()
        got = [srv.poll(t) for t in tickets]
        assert srv.stats()["refused"] == 1
        for p, (v, _) in zip(small, got):
            assert abs(v - p.execute(qg.FP64)) <= 1e-6
        srv.set_max_macs(0)
        t = srv.submit(big)
        srv.drain()
        assert abs(srv.poll(t)[0] - big.execute(qg.FP64)) <= 1e-6
    finally:
        srv.close()


def test_rank_16_plans_are_rejected_before_any_launch(ctx):
    """A plan whose largest intermediate is rank 16 (2^32 elements) is beyond
    the step kernels' 32-bit tile, run and output counters: executing it fails
    with InvalidFunctionInput before any launch, and the server refuses it at
    submission; the context stays usable."""
    big = qg.Plan(random_circuit_text(22, 16, 21), "Z", ordering="auto", ctx=ctx)
    assert big.peak_rank == 16
    with pytest.raises(qg.InvalidFunctionInput):
        big.execute(qg.MIXED)
    assert "rank-16" in ctx.last_error
    srv = qg.Server(max_inflight=4, precision=qg.MIXED, ctx=ctx, max_macs=int(3e13))
    try:
        with pytest.raises(qg.Refused):
            srv.submit(big)
    finally:
        srv.close()
    small = qg.Plan(random_circuit_text(10, 8, 3), "Z", ordering="auto", ctx=ctx)
    assert abs(small.execute(qg.MIXED) - small.execute(qg.FP64)) <= 1e-6
