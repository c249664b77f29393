"""Launch policies and the autotuner of a batch's grouped launch.

A policy moves workspaces between shared memory and the global slab, turns the
staging of plan blocks and leaves on or off, caps the CTAs per SM and picks the
schedule.  None of that touches the arithmetic of an instance, so every policy
(and whatever the autotuner picks) must give bit-identical values."""
import numpy as np
import pytest

import qtorch_gb300 as qg

pytestmark = pytest.mark.gpu


def qaoa_batch(ctx, prec, points=8):
    """p=1 and p=2 MaxCut terms at a few (gamma, beta) points: workspaces from a
    few KB (p=1) to hundreds of KB (p=2); 81 terms a point, so more instances
    than CTAs (three per SM on 152 SMs) at eight points."""
    b = qg.Batch(ctx)
    plans = []
    for p, nodes, seed in [(1, 30, 3), (2, 24, 5)]:
        dgf = qg.random_regular_graph(nodes, 3, seed=seed)
        for k in range(points):
            bg = [0.2 + 0.1 * k] * p + [0.5 - 0.05 * k] * p
            for e in range(qg.qaoa_num_edges(dgf)):
                q, m = qg.qaoa_term_text(dgf, p, bg, e)
                pl = qg.Plan(q, m, ordering="linegraph", ctx=ctx)
                plans.append(pl)
                b.add(pl)
    b.prepare(prec)
    return b, plans


POLICIES = [
    dict(ws_smem_cap=0, stage_cap=0),                  # everything from global memory
    dict(ws_smem_cap=128 << 10),                       # large workspaces in shared memory, 1 CTA per SM
    dict(ws_smem_cap=8 << 10, stage_cap=24 << 10),
    dict(ctas_per_sm=1, static_schedule=1),
    dict(static_schedule=1),
    dict(kernel_ctas=2),                               # 128 registers a thread
    dict(kernel_ctas=4, ws_smem_cap=16 << 10),         # 64 registers a thread
    dict(kernel_ctas=3, stage_cap=0),
    dict(kernel_ctas=5, ws_smem_cap=0, stage_cap=0),   # 48 registers a thread
    dict(kernel_ctas=1),                               # 512 threads a CTA, one CTA per SM
]


@pytest.mark.parametrize("prec", [qg.MIXED, qg.FP64])
def test_policies_give_identical_values(ctx, prec):
    b, _ = qaoa_batch(ctx, prec)
    b.run()
    want = b.fetch()
    base = b.launch_info()
    assert base["n_grouped"] == len(b) and base["dynamic_schedule"] == 1
    assert base["kernel_ctas"] == 4   # default with more instances than two CTAs per SM hold
    assert base["grid"] == 4 * 152 and base["stage_bytes"] == 0
    for pol in POLICIES:
        b.set_launch_policy(**pol)
        info = b.launch_info()
        if pol.get("ws_smem_cap") == 0:
            assert info["ws_smem_bytes"] == 0 and info["ws_slab_bytes"] > 0 and info["n_staged"] == 0
        if pol.get("ws_smem_cap") == 128 << 10:
            assert info["n_ws_smem"] > base["n_ws_smem"]
        if pol.get("static_schedule"):
            assert info["dynamic_schedule"] == 0
        if pol.get("ctas_per_sm") == 1:
            assert info["grid"] <= base["grid"] // 2
        if "kernel_ctas" in pol:
            assert info["kernel_ctas"] == pol["kernel_ctas"]
        b.run()
        assert np.array_equal(b.fetch(), want), pol


def test_autotune_keeps_values_and_reports_policy(ctx):
    b, _ = qaoa_batch(ctx, qg.MIXED)
    b.use_graph(True)
    b.run()
    want = b.fetch()
    pol, us = b.autotune(reps=2)
    assert us > 0
    assert b.launch_policy == pol
    assert np.array_equal(b.fetch(), want)   # the autotuner leaves the current values
    b.run()                                  # graph captured under the chosen policy
    assert np.array_equal(b.fetch(), want)


def test_policy_that_does_not_fit_is_refused(ctx):
    # a p=2 term whose workspace exceeds the 227 KiB of shared memory a CTA may
    # have on sm_103 (the first found among 40-vertex graphs)
    b = qg.Batch(ctx)
    big = None
    for seed in range(100, 116):
        dgf = qg.random_regular_graph(40, 3, seed=seed)
        for e in range(qg.qaoa_num_edges(dgf)):
            pl = qg.Plan(*qg.qaoa_term_text(dgf, 2, [0.3, 0.2, 0.6, 0.4], e), ordering="linegraph", ctx=ctx)
            if pl.workspace_bytes(qg.MIXED) > 232448:
                big = pl
                break
        if big is not None:
            break
    assert big is not None
    b.add(big)
    b.prepare(qg.MIXED)
    assert b.launch_info()["n_grouped"] == 1
    b.run()
    want = b.fetch()
    before = b.launch_policy
    with pytest.raises(qg.QtError):
        b.set_launch_policy(ws_smem_cap=1 << 30, stage_cap=1 << 30)
    with pytest.raises(qg.QtError):
        b.set_launch_policy(kernel_ctas=7)   # no such variant
    assert b.launch_policy == before
    b.run()
    assert np.array_equal(b.fetch(), want)


def test_policy_set_before_prepare_applies(ctx):
    dgf = qg.random_regular_graph(20, 3, seed=9)
    b = qg.Batch(ctx)
    for e in range(qg.qaoa_num_edges(dgf)):
        b.add(qg.Plan(*qg.qaoa_term_text(dgf, 1, [0.4, 0.6], e), ordering="linegraph", ctx=ctx))
    b.set_launch_policy(ws_smem_cap=0, stage_cap=0)
    b.prepare(qg.MIXED)
    info = b.launch_info()
    assert info["ws_smem_bytes"] == 0 and info["stage_bytes"] == 0 and info["n_ws_smem"] == 0
    b.run()
    got = b.fetch()
    b.set_launch_policy()
    b.run()
    assert np.array_equal(b.fetch(), got)
