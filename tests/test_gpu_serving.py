"""Serving: continuous batching with memory admission.  Each request's result
is the same alone and in the mix (bit for bit in FP64, within 1e-6 in the
mixed form)."""
import time

import numpy as np
import pytest

import qtorch_gb300 as qg
from conftest import load_golden

pytestmark = pytest.mark.gpu


def request_mix(ctx):
    """QAOA terms at several points plus a few golden sample circuits."""
    plans = []
    dgf = qg.random_regular_graph(20, 3, seed=9)
    rng = np.random.default_rng(3)
    for e in range(0, qg.qaoa_num_edges(dgf), 3):
        bg = list(rng.uniform(0, np.pi, 2))
        q, m = qg.qaoa_term_text(dgf, 1, bg, e)
        plans.append(qg.Plan(q, m, ordering="linegraph", ctx=ctx))
    for case in load_golden("networks.json"):
        if case["gate_files"]:
            continue
        plans.append(qg.Plan(case["qasm"], case["measure"], ordering="sequence", sequence=case["sequence"], ctx=ctx))
    return plans


@pytest.mark.parametrize("prec", [qg.FP64, qg.MIXED])
def test_alone_equals_in_the_mix(ctx, prec):
    plans = request_mix(ctx)
    alone = [p.execute(prec) for p in plans]
    srv = qg.Server(max_inflight=8, precision=prec, ctx=ctx)
    try:
        tickets = []
        for i, p in enumerate(plans):
            tickets.append(srv.submit(p))
            if i % 4 == 0:
                time.sleep(0.001)    # arrivals while earlier requests run
        srv.drain()
        mixed = [srv.poll(t) for t in tickets]
        stats = srv.stats()
    finally:
        srv.close()
    assert all(m is not None for m in mixed)
    for a, (v, lat) in zip(alone, mixed):
        if prec == qg.FP64:
            assert v == a
        else:
            assert abs(v - a) <= 1e-6
        assert lat >= 0
    assert stats["completed"] == len(plans)
    assert 0 < stats["p50_s"] <= stats["p99_s"]


def test_admission_respects_memory_budget():
    c = qg.Context(0)
    try:
        plans = request_mix(c)[:6]
        need = max(p.workspace_bytes(qg.FP64) for p in plans) + 64 * 1024
        c.set_memory_budget(need * 3)
        srv = qg.Server(max_inflight=64, precision=qg.FP64, ctx=c)
        try:
            tickets = [srv.submit(p) for p in plans]
            srv.drain()
            assert all(srv.poll(t) is not None for t in tickets)
        finally:
            srv.close()
        # a request larger than the whole budget is refused at submission
        c.set_memory_budget(1024)
        srv = qg.Server(max_inflight=4, precision=qg.FP64, ctx=c)
        try:
            with pytest.raises(qg.OutOfMemory):
                srv.submit(plans[0])
        finally:
            srv.close()
    finally:
        c.close()


@pytest.mark.parametrize("prec", [qg.FP64, qg.MIXED])
def test_requests_above_the_budget_are_sliced(prec):
    """A request whose workspace exceeds the whole budget is split over cut
    wires (qt_plan_slice) so that one slice fits, runs alone slice by slice, and
    returns the unsliced value (FP64 to a few ulp, mixed within 1e-6); requests
    that fit are served as before."""
    from qtorch_gb300.circuits import random_circuit_text
    c = qg.Context(0)
    try:
        big = qg.Plan(random_circuit_text(12, 12, 5), "Z", ordering="linegraph", ctx=c)
        small = request_mix(c)[:4]
        want = big.execute(qg.FP64)
        budget = big.workspace_bytes(prec) // 8 + big.workspace_bytes(prec) // 64
        c.set_memory_budget(budget)
        srv = qg.Server(max_inflight=16, precision=prec, ctx=c)
        try:
            tickets = [srv.submit(big)] + [srv.submit(p) for p in small] + [srv.submit(big)]
            srv.drain()
            got = [srv.poll(t) for t in tickets]
            assert all(g is not None for g in got)
            vals = [g[0] for g in got]
            tol = 1e-12 if prec == qg.FP64 else 1e-6
            for v in (vals[0], vals[-1]):
                assert abs(v - want) <= tol * max(1.0, abs(want))
            for p, v in zip(small, vals[1:-1]):
                assert abs(v - p.execute(prec)) <= (0 if prec == qg.FP64 else 1e-6)
        finally:
            srv.close()
    finally:
        c.close()


def test_small_requests_pass_a_heavy_one():
    """A heavy request runs step by step on its own lane's stream; small
    requests submitted right after it are served on another lane meanwhile
    (the shared plan's owner context is not held by the heavy run), so they
    finish first, and their values are unchanged."""
    from qtorch_gb300.circuits import qft_text
    ctx = qg.Context(0)
    try:
        heavy = qg.Plan(qft_text(13, 4), "Z", ordering="linegraph", ctx=ctx)
        dgf = qg.random_regular_graph(20, 3, seed=9)
        small = [qg.Plan(*qg.qaoa_term_text(dgf, 1, [0.5, 1.2], e), ordering="linegraph", ctx=ctx)
                 for e in range(8)]
        alone = [p.execute(qg.MIXED) for p in small]
        heavy_alone = heavy.execute(qg.MIXED)
        srv = qg.Server(max_inflight=16, precision=qg.MIXED, ctx=ctx)
        try:
            for _ in range(2):   # the first pass warms the lanes' caches
                t_heavy = srv.submit(heavy)
                tickets = [srv.submit(p) for p in small]
                srv.drain()
                v_heavy, l_heavy = srv.poll(t_heavy)
                got = [srv.poll(t) for t in tickets]
            assert abs(v_heavy - heavy_alone) <= 1e-6
            for (v, lat), want in zip(got, alone):
                assert abs(v - want) <= 1e-6
                assert lat < l_heavy
        finally:
            srv.close()
    finally:
        ctx.close()


def test_light_requests_run_while_a_heavy_one_waits_for_memory():
    """A budget that holds one heavy request: the second waits for memory
    while the first runs.  Light requests submitted meanwhile are served on
    the light lane at once -- the dispatcher blocks only the heavy lanes until
    a wave ends -- so they finish long before the first heavy request."""
    import time

    from qtorch_gb300.circuits import random_circuit_text
    ctx = qg.Context(0)
    try:
        heavy = qg.Plan(random_circuit_text(14, 12, 6), "Z", ordering="auto", ctx=ctx)   # 4e8 MACs
        dgf = qg.random_regular_graph(20, 3, seed=9)
        small = [qg.Plan(*qg.qaoa_term_text(dgf, 1, [0.5, 1.2], e), ordering="linegraph", ctx=ctx)
                 for e in range(8)]
        alone = [p.execute(qg.FP64) for p in small]
        heavy_alone = heavy.execute(qg.FP64)
        # the server's footprint of an FP64 request: workspace + leaves + 4 KB
        fp = heavy.workspace_bytes(qg.FP64) + 16 * heavy.leaf_values().size + 4096
        ctx.set_memory_budget(int(fp * 1.5))
        srv = qg.Server(max_inflight=64, precision=qg.FP64, ctx=ctx)
        try:
            for _ in range(2):   # the first pass warms the lanes' caches
                t1, t2 = srv.submit(heavy), srv.submit(heavy)
                time.sleep(0.001)   # the second heavy request is waiting for memory by now
                tickets = [srv.submit(p) for p in small]
                srv.drain()
                v1, l1 = srv.poll(t1)
                v2, l2 = srv.poll(t2)
                got = [srv.poll(t) for t in tickets]
            assert v1 == heavy_alone and v2 == heavy_alone
            assert l2 > l1
            for (v, lat), want in zip(got, alone):
                assert v == want
                assert lat < 0.5 * l1, (lat, l1)
        finally:
            srv.close()
    finally:
        ctx.set_memory_budget(0)
        ctx.close()
