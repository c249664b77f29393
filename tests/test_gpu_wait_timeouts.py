"""Failure detection without a fault, for the tcgen05 GEMM pipeline and the
grouped interpreter's staging (the streaming kernel's is in
test_gpu_stream.py): a test hook leaves a copy unissued -- a wait nothing
completes -- the bounded waits give up after a few thousand polls, the call
reports QT_ERR_CUDA, and with the hook off the same work on the same context
succeeds."""
import numpy as np
import pytest

import qtorch_gb300 as qg

pytestmark = pytest.mark.gpu


def gemm_step(rng):
    """rank 9 x rank 9 summed over 3 wires: M = N = 4096, K = 64 -- GEMM-shaped,
    both operands too large for the streaming kernel"""
    ra = rb = 9
    a = (rng.standard_normal(4 ** ra) + 1j * rng.standard_normal(4 ** ra)).astype(np.complex64)
    b = (rng.standard_normal(4 ** rb) + 1j * rng.standard_normal(4 ** rb)).astype(np.complex64)
    sa, sb = [0, 4, 7], [2, 5, 8]
    fa = [w for w in range(ra) if w not in sa]
    fb = [w for w in range(rb) if w not in sb]
    ffa = [1] * len(fa) + [0] * len(fb)
    return a, b, ffa, fa + fb, sa, sb


def test_gemm_wait_timeout_reports_an_error_and_the_context_recovers(ctx):
    lib = qg._capi.load()
    rng = np.random.default_rng(11)
    a, b, ffa, fi, sa, sb = gemm_step(rng)
    n0 = ctx.tensor_core_steps
    want = qg.contract_pair_c64(a, b, ffa, fi, sa, sb, ctx=ctx)
    assert ctx.tensor_core_steps == n0 + 1
    assert lib.qt_debug_gemm_fault(ctx.handle, 1, 4096) == 0
    try:
        with pytest.raises(qg.QtError) as info:
            qg.contract_pair_c64(a, b, ffa, fi, sa, sb, ctx=ctx)
        assert info.value.status == 10   # QT_ERR_CUDA
        assert "timed out" in str(info.value)
    finally:
        assert lib.qt_debug_gemm_fault(ctx.handle, 0, 0) == 0
    got = qg.contract_pair_c64(a, b, ffa, fi, sa, sb, ctx=ctx)
    assert np.array_equal(got, want)


def test_staging_wait_timeout_reports_an_error_and_the_context_recovers(ctx):
    lib = qg._capi.load()
    dgf = qg.random_regular_graph(20, 3, seed=9)
    plan = qg.Plan(*qg.qaoa_term_text(dgf, 1, [0.4, 1.1], 2), ordering="linegraph", ctx=ctx)
    want = plan.execute(qg.MIXED)
    assert lib.qt_debug_staging_fault(ctx.handle, 1, 4096) == 0
    try:
        with pytest.raises(qg.QtError) as info:
            plan.execute(qg.MIXED)
        assert info.value.status == 10
        assert "staging" in str(info.value)
    finally:
        assert lib.qt_debug_staging_fault(ctx.handle, 0, 0) == 0
    assert plan.execute(qg.MIXED) == want
