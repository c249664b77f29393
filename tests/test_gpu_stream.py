"""The streaming kernel (a small operand in shared memory, the large one read
once by TMA bulk copies) against a complex128 evaluation, and the per-tensor
power-of-two scaling of plans run step by step."""
import numpy as np
import pytest

import qtorch_gb300 as qg

pytestmark = pytest.mark.gpu


def random_maps(rng, ra, rb, nsum, shuffle_c):
    wa, wb = rng.permutation(ra), rng.permutation(rb)
    sum_a, sum_b = [int(x) for x in wa[:nsum]], [int(x) for x in wb[:nsum]]
    free = [(1, w) for w in range(ra) if w not in sum_a] + [(0, w) for w in range(rb) if w not in sum_b]
    if shuffle_c:
        free = [free[i] for i in rng.permutation(len(free))]
    return [f for f, _ in free], [w for _, w in free], sum_a, sum_b


def reference(a, b, ra, rb, ffa, fi, sa, sb):
    """C[c] = sum_k A[a(c,k)] B[b(c,k)] in complex128 with numpy (axis i of a
    reshaped tensor is wire rank-1-i: flat index sum_i idx_i 4^i)."""
    A = a.astype(np.complex128).reshape([4] * ra)
    B = b.astype(np.complex128).reshape([4] * rb)
    letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"
    la = [None] * ra
    lb = [None] * rb
    nxt = 0
    for x, y in zip(sa, sb):
        la[x] = lb[y] = letters[nxt]
        nxt += 1
    out = []
    for f, w in zip(ffa, fi):
        ch = letters[nxt]
        nxt += 1
        if f:
            la[w] = ch
        else:
            lb[w] = ch
        out.append(ch)
    spec = "".join(la[::-1]) + "," + "".join(lb[::-1]) + "->" + "".join(out[::-1])
    return np.einsum(spec, A, B).reshape(-1)


# steps with one small operand that keeps at most one free wire (C = A's free
# wires then B's: the pair kernel's shapes before); with C's digits in any
# other order every one of these goes to the streaming kernel
SHAPES = [(12, 3, 2), (3, 12, 2), (12, 4, 3), (4, 12, 3), (12, 1, 1), (1, 12, 1), (12, 2, 2), (12, 2, 1),
          (11, 5, 4), (10, 6, 5), (2, 12, 1)]


# wide shapes whose ContractNodes order takes the tiled or tensor-core kernel;
# with C's digits in another order they stream too -- among them small
# operands with 16 or 64 free indices (several passes over a tile) and outputs
# staged through shared memory
SHAPES_ANY_ORDER = [(12, 5, 2), (3, 12, 1), (12, 4, 1), (4, 12, 2), (5, 11, 2), (11, 6, 3)]
CASES = [(s, False) for s in SHAPES] + [(s, True) for s in SHAPES + SHAPES_ANY_ORDER]


@pytest.mark.parametrize("shape,shuffle_c", CASES,
                         ids=[f"{a}x{b}k{k}-{'any' if sh else 'cn'}" for (a, b, k), sh in CASES])
def test_streaming_contraction_matches_complex128(ctx, shape, shuffle_c):
    ra, rb, nsum = shape
    rng = np.random.default_rng(ra * 100 + rb * 10 + nsum + (7 if shuffle_c else 0))
    a = (rng.standard_normal(4 ** ra) + 1j * rng.standard_normal(4 ** ra)).astype(np.complex64)
    b = (rng.standard_normal(4 ** rb) + 1j * rng.standard_normal(4 ** rb)).astype(np.complex64)
    ffa, fi, sa, sb = random_maps(rng, ra, rb, nsum, shuffle_c)
    n0 = ctx.stream_steps
    got = qg.contract_pair_c64(a, b, ffa, fi, sa, sb, ctx=ctx)
    assert ctx.stream_steps == n0 + 1, "the step did not take the streaming kernel"
    want = reference(a, b, ra, rb, ffa, fi, sa, sb)
    err = np.max(np.abs(got - want))
    assert err <= 2e-6 * np.sqrt(4 ** nsum) * 8, err


@pytest.mark.parametrize("scale", [1e12, 1e-12])
def test_step_by_step_plans_scale_every_tensor(ctx, tmp_path, scale):
    """A 14-qubit circuit large enough to run step by step when alone, with an
    unnormalised gate of entries `scale` on five qubits: the value is
    scale^10 x O(1), 1e120 or 1e-120, far beyond FP32's range, yet every
    stored complex64 tensor stays near 1 (per-tensor power-of-two scaling)
    and the mixed value matches FP64 to FP32's relative accuracy."""
    from qtorch_gb300.circuits import random_circuit_text
    (tmp_path / "big.gate").write_text(f"{scale} 0 0 ({scale},0)")
    n = 14
    body = random_circuit_text(n, 12, 3).split("\n", 1)[1]
    qasm = f"{n}\ndef1 BIG big.gate\n" + "".join(f"H {q}\n" for q in range(n)) + \
        "".join(f"BIG {q}\n" for q in range(5)) + body
    plan = qg.Plan(qasm, "Z", ordering="linegraph", gate_dir=str(tmp_path), ctx=ctx)
    assert plan.flops > 1 << 24   # runs step by step when executed alone
    v64 = plan.execute(qg.FP64)
    assert 1e-3 < abs(v64) / scale ** 10 < 1e3
    vmx = plan.execute(qg.MIXED)
    assert abs(vmx - v64) <= 1e-5 * abs(v64)


def test_pipeline_wait_timeout_reports_an_error_and_the_context_recovers(ctx):
    """Failure detection without a fault: the test hook leaves every CTA's
    first tile unissued (a wait nothing completes), the bounded waits give up
    after a few thousand polls, the kernel drains the copies it did issue and
    raises its flag; the call returns QT_ERR_CUDA, and with the hook off the
    same contraction on the same context succeeds."""
    lib = qg._capi.load()
    ra, rb, nsum = 12, 3, 2
    rng = np.random.default_rng(5)
    a = (rng.standard_normal(4 ** ra) + 1j * rng.standard_normal(4 ** ra)).astype(np.complex64)
    b = (rng.standard_normal(4 ** rb) + 1j * rng.standard_normal(4 ** rb)).astype(np.complex64)
    ffa, fi, sa, sb = random_maps(rng, ra, rb, nsum, False)
    assert lib.qt_debug_stream_fault(ctx.handle, 1, 4096) == 0
    try:
        n0 = ctx.stream_steps
        with pytest.raises(qg.QtError) as info:
            qg.contract_pair_c64(a, b, ffa, fi, sa, sb, ctx=ctx)
        assert info.value.status == 10   # QT_ERR_CUDA
        assert "timed out" in str(info.value)
        assert ctx.stream_steps == n0 + 1
    finally:
        assert lib.qt_debug_stream_fault(ctx.handle, 0, 0) == 0
    got = qg.contract_pair_c64(a, b, ffa, fi, sa, sb, ctx=ctx)
    want = reference(a, b, ra, rb, ffa, fi, sa, sb)
    assert np.max(np.abs(got - want)) <= 2e-6 * 4 * 8
