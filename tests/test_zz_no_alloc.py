"""qt_plan_execute_static, the entry point that allocates no device memory.

Some callers cannot call cudaMalloc: code that runs under a framework that owns
every byte of the device, or a latency-bound loop that must not pay
cudaMalloc's implicit synchronisation.  They hand over inputs and outputs in
device memory they already own, and the engine works in a statically reserved
device array.  This test calls that entry point through the C ABI, twice in a
row on the same static array, and checks it against qt_plan_execute: equal bit
for bit in FP64, within 1e-6 in the mixed form; across those calls neither the
context's allocator nor the device's free memory may change.  It lives in a
file of its own that pytest collects last."""
import ctypes

import numpy as np
import pytest

import qtorch_gb300 as qg
from conftest import load_golden

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


def static_call(lib, ctx, plan, prec, leaves, out):
    return lib.qt_plan_execute_static(ctx.handle, plan.handle, prec, ctypes.c_void_p(leaves.data_ptr()),
                                      ctypes.cast(ctypes.c_void_p(out.data_ptr()), ctypes.POINTER(ctypes.c_double)))


def plans_under_test(ctx):
    dgf = qg.random_regular_graph(20, 3, seed=12)
    out = []
    for p, bg in ((1, [0.7, 1.3]), (2, [0.2, 0.9, 1.1, 0.4])):
        for e in (0, 5):
            q, m = qg.qaoa_term_text(dgf, p, bg, e)
            out.append(qg.Plan(q, m, ordering="linegraph", ctx=ctx))
    case = load_golden("networks.json")[0]
    out.append(qg.Plan(case["qasm"], case["measure"], ordering="sequence", sequence=case["sequence"], ctx=ctx))
    return out


@pytest.mark.parametrize("prec", [qg.FP64, qg.MIXED], ids=["fp64", "mixed"])
def test_static_entry_point_matches_plan_execute(prec):
    import torch
    lib = qg._capi.load()
    lib.qt_plan_execute_static.restype = ctypes.c_int
    lib.qt_plan_execute_static.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.POINTER(ctypes.c_double)]
    ctx = qg.Context(0)
    try:
        for plan in plans_under_test(ctx):
            want = plan.execute(prec)
            leaves = plan.leaf_values()
            if prec == qg.MIXED:
                leaves = leaves.astype(np.complex64)
            d_leaves = torch.from_numpy(leaves).cuda()
            outs = [torch.full((2,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(2)]
            # the leaves are written on torch's stream: complete them before the context's stream reads them
            torch.cuda.synchronize()
            stats0 = ctx.memory_stats()
            # two calls in a row on the same static array; the device's free
            # memory is compared around the second (the first launch of a kernel
            # may let the driver grow its local-memory reservation)
            assert static_call(lib, ctx, plan, prec, d_leaves, outs[0]) == 0, ctx.last_error
            ctx.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            assert static_call(lib, ctx, plan, prec, d_leaves, outs[1]) == 0, ctx.last_error
            ctx.synchronize()
            assert torch.cuda.mem_get_info()[0] == free0  # no device memory allocated
            assert ctx.memory_stats() == stats0          # no block taken from or added to the allocator
            got = []
            for out in outs:
                v = out.cpu().numpy()
                got.append(complex(v[0], v[1]))
            for g in got:
                if prec == qg.FP64:
                    assert g == want
                else:
                    assert abs(g - want) <= MIXED_TOL
    finally:
        ctx.close()


def test_static_entry_point_rejects_oversized_plans():
    import torch
    lib = qg._capi.load()
    lib.qt_plan_execute_static.restype = ctypes.c_int
    lib.qt_plan_execute_static.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.POINTER(ctypes.c_double)]
    ctx = qg.Context(0)
    try:
        case = [c for c in load_golden("networks.json") if c["name"] == "4regRand20Node1-p1.qasm"][0]
        plan = qg.Plan(case["qasm"], case["measure"], ordering="sequence", sequence=case["sequence"], ctx=ctx)
        assert plan.workspace_bytes(qg.FP64) > 8 << 20
        d_leaves = torch.from_numpy(plan.leaf_values()).cuda()
        out = torch.zeros(2, dtype=torch.float64, device="cuda")
        rc = static_call(lib, ctx, plan, qg.FP64, d_leaves, out)
        assert rc == 9   # QT_ERR_OUT_OF_MEMORY
        assert "static scratch" in ctx.last_error
    finally:
        ctx.close()


def test_item_descriptors_match_lookup_path_bit_for_bit():
    """The mixed form's unscaled pass reads host-prepared per-item descriptors
    when a plan carries them; the static entry point's copy of the plan block
    has none, so it looks each item's step up.  Both must round the same
    products in the same order: equal bit for bit, over the 60 terms of a
    30-vertex p=1 objective (batched under two launch policies) and the p=2
    terms of a 20-vertex graph."""
    import torch
    lib = qg._capi.load()
    lib.qt_plan_execute_static.restype = ctypes.c_int
    lib.qt_plan_execute_static.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.POINTER(ctypes.c_double)]
    ctx = qg.Context(0)
    try:
        dgf = qg.random_regular_graph(30, 4, seed=1)
        plans = [qg.Plan(*qg.qaoa_term_text(dgf, 1, [0.3, 0.7], e), ordering="linegraph", ctx=ctx)
                 for e in range(60)]
        plans += plans_under_test(ctx)[:4]
        assert sum(p.item_descriptors > 0 for p in plans) >= 60
        lookup = []
        for plan in plans:
            d_leaves = torch.from_numpy(plan.leaf_values().astype(np.complex64)).cuda()
            out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            assert static_call(lib, ctx, plan, qg.MIXED, d_leaves, out) == 0, ctx.last_error
            ctx.synchronize()
            v = out.cpu().numpy()
            lookup.append(complex(v[0], v[1]))
        for plan, want in zip(plans, lookup):
            assert plan.execute(qg.MIXED) == want
        for ctas in (1, 2):
            batch = qg.Batch(ctx)
            for plan in plans:
                batch.add(plan)
            batch.prepare(qg.MIXED)
            batch.set_launch_policy(kernel_ctas=ctas)
            got = batch.execute(qg.MIXED)
            assert [complex(g) for g in got] == lookup
            batch._release()
    finally:
        ctx.close()
