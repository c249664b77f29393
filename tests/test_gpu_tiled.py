"""CTA-tiled steps and the dynamic instance schedule of the grouped interpreter.

p=2 QAOA light cones on 3-regular graphs have rank 5-9 intermediates whose
steps run CTA-wide as tiled products.  The FP64 form keeps the reference's
per-element summation order there too, so it stays bit-exact against the
oracle; the mixed form stays within the stated 1e-6."""
import numpy as np
import pytest

import qtorch_gb300 as qg
from oracle import port

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6
TILED = 1 << 7


def tiled_terms(dgf, p, point, want, max_peak=8):
    out = []
    for e in range(qg.qaoa_num_edges(dgf)):
        q, m = qg.qaoa_term_text(dgf, p, point, e)
        pl = qg.Plan(q, m, ordering="linegraph", symbolic=True)
        if pl.peak_rank <= max_peak and (pl.step_info(qg.FP64)[:, 6] & TILED).any():
            out.append((q, m))
        if len(out) == want:
            break
    return out


def test_tiled_steps_fp64_bit_exact_and_mixed_within_tolerance(ctx):
    dgf = qg.random_regular_graph(26, 3, seed=105)
    terms = tiled_terms(dgf, 2, [0.3, 0.9, 0.7, 0.2], 3)
    assert terms, "no term with a CTA-tiled step"
    for q, m in terms:
        plan = qg.Plan(q, m, ordering="linegraph", ctx=ctx)
        v_or, _ = port.replay_value(q, m, plan.sequence())
        assert plan.execute(qg.FP64) == v_or
        assert abs(plan.execute(qg.MIXED) - v_or) <= MIXED_TOL


def test_dynamic_schedule_keeps_instance_order(ctx):
    """More instances than CTAs: instances run longest first under the dynamic
    schedule, and every value still lands in its own slot."""
    dgf1 = qg.random_regular_graph(26, 3, seed=105)
    dgf2 = qg.random_regular_graph(20, 3, seed=7)
    plans = [qg.Plan(q, m, ordering="linegraph", ctx=ctx) for q, m in tiled_terms(dgf1, 2, [0.3, 0.9, 0.7, 0.2], 2)]
    for e in range(qg.qaoa_num_edges(dgf2)):
        q, m = qg.qaoa_term_text(dgf2, 1, [0.5, 1.3], e)
        plans.append(qg.Plan(q, m, ordering="linegraph", ctx=ctx))
    single = {id(p): p.execute(qg.FP64) for p in plans}
    rng = np.random.default_rng(3)
    order = [plans[i] for i in rng.integers(0, len(plans), 1500)]
    b = qg.Batch(ctx)
    for p in order:
        b.add(p)
    for prec in (qg.FP64, qg.MIXED):
        got = b.execute(prec)
        want = np.array([single[id(p)] for p in order])
        if prec == qg.FP64:
            assert np.array_equal(got, want)
        else:
            assert np.abs(got - want).max() <= MIXED_TOL



@pytest.mark.parametrize("ra,rb,ns", [(9, 9, 9), (9, 10, 9), (9, 9, 8)])
def test_long_reduction_steps(ctx, ra, rb, ns):
    """A sum of >= 4^8 terms into <= 16 outputs runs over the whole GPU: the
    FP64 form forms products in parallel and adds them in the reference's order
    (bit-exact), the complex64 form merges compensated partial sums."""
    rng = np.random.default_rng(ra + rb + ns)
    sa = list(rng.permutation(ra)[:ns])
    sb = list(rng.permutation(rb)[:ns])
    fa = [i for i in range(ra) if i not in sa]
    fb = [i for i in range(rb) if i not in sb]
    ffa, fi = [1] * len(fa) + [0] * len(fb), fa + fb
    a = rng.standard_normal(4 ** ra) + 1j * rng.standard_normal(4 ** ra)
    b = rng.standard_normal(4 ** rb) + 1j * rng.standard_normal(4 ** rb)
    want = port.contract_indices(a, b, ffa, fi, sa, sb)
    got = qg.contract_pair(a, b, ffa, fi, sa, sb, ctx=ctx)
    assert np.array_equal(got, want)
    a32, b32 = a.astype(np.complex64), b.astype(np.complex64)
    want32 = port.contract_indices(a32.astype(np.complex128), b32.astype(np.complex128), ffa, fi, sa, sb)
    got32 = qg.contract_pair_c64(a32, b32, ffa, fi, sa, sb, ctx=ctx)
    # compensated sums: the result is the exact sum of the complex64 products rounded once
    assert np.max(np.abs(got32 - want32)) <= 1e-6 * np.max(np.abs(want32)) + 1e-6


@pytest.mark.parametrize("ra,rb,ns", [(7, 7, 2), (8, 6, 3), (6, 8, 2), (7, 5, 1)])
def test_wide_pair_steps_run_tiled_over_the_gpu(ctx, ra, rb, ns):
    """Wide single contractions (the steps of plans run one at a time) use the
    whole-GPU tiled kernel: FP64 bit-exact, complex64 within rounding."""
    rng = np.random.default_rng(7 * ra + rb + ns)
    sa = list(rng.permutation(ra)[:ns])
    sb = list(rng.permutation(rb)[:ns])
    fa = [i for i in range(ra) if i not in sa]
    fb = [i for i in range(rb) if i not in sb]
    ffa, fi = [1] * len(fa) + [0] * len(fb), fa + fb
    a = rng.standard_normal(4 ** ra) + 1j * rng.standard_normal(4 ** ra)
    b = rng.standard_normal(4 ** rb) + 1j * rng.standard_normal(4 ** rb)
    assert np.array_equal(qg.contract_pair(a, b, ffa, fi, sa, sb, ctx=ctx), port.contract_indices(a, b, ffa, fi, sa, sb))
    a32, b32 = a.astype(np.complex64), b.astype(np.complex64)
    want = port.contract_indices(a32.astype(np.complex128), b32.astype(np.complex128), ffa, fi, sa, sb)
    got = qg.contract_pair_c64(a32, b32, ffa, fi, sa, sb, ctx=ctx)
    assert np.max(np.abs(got - want)) <= 2e-6 * np.sqrt(4 ** ns) * 4


@pytest.mark.parametrize("which", ["qft10", "qft12", "rand12", "rand16"])
def test_mid_size_plans_alone_run_step_by_step(ctx, which):
    """A plan above 2^24 complex MACs evaluated alone runs step by step over the
    whole GPU (tiled, tensor-core and compensated reduction kernels); FP64 stays
    bit-exact with the oracle's replay, mixed within 1e-6."""
    from qtorch_gb300.circuits import qft_measure_text, qft_text, random_circuit_text
    text = {"qft10": qft_text(10, 4), "qft12": qft_text(12, 5), "rand12": random_circuit_text(12, 10, 1),
            "rand16": random_circuit_text(16, 12, 10)}[which]
    # <Z> of a QFT'd basis state is 0 on every qubit; <X> of its last qubit is not
    meas = qft_measure_text(int(which[3:])) if which.startswith("qft") else "Z"
    plan = qg.Plan(text, meas, ordering="linegraph", ctx=ctx)
    assert plan.flops > 1 << 24
    v64 = plan.execute(qg.FP64)
    if which.startswith("qft"):
        assert abs(v64) > 1e-3
    if which in ("qft10", "rand12"):   # larger replays take too long on the host
        v_or, _ = port.replay_value(text, meas, plan.sequence())
        assert v64 == v_or
    assert abs(plan.execute(qg.MIXED) - v64) <= MIXED_TOL


@pytest.mark.parametrize("scale", [1e12, 1e-12])
def test_values_outside_the_unscaled_range_rerun_with_scaling(ctx, tmp_path, scale):
    """Mixed plans run first without power-of-two scaling and check every stored
    value against [2^-60, 2^60]; an unnormalised gate (entries 1e12 or 1e-12,
    superoperator entries 1e24 / 1e-24) pushes values out -- the value itself is
    5e71 / 5e-73, beyond FP32 -- the instance runs again with the scaling, and
    the result still matches FP64 to FP32 relative accuracy."""
    (tmp_path / "big.gate").write_text(f"{scale} 0 0 ({scale},0)")
    qasm = "3\ndef1 BIG big.gate\nH 0\nH 1\nCNOT 0 1\nBIG 0\nBIG 1\nRx 0.3 2\nCNOT 1 2\nBIG 2\nH 2\n"
    plan = qg.Plan(qasm, "0 T T", ordering="linegraph", gate_dir=str(tmp_path), ctx=ctx)
    v64 = plan.execute(qg.FP64)
    assert abs(v64) > 0
    b = qg.Batch(ctx)
    b.add(plan)
    vmx = b.execute(qg.MIXED)[0]
    assert np.isfinite(vmx)
    assert abs(vmx - v64) <= 1e-5 * abs(v64)


def test_tiny_entries_next_to_normal_ones(ctx, tmp_path):
    """A gate with entries 1 and 1e-12 (superoperator entries down to 1e-24,
    below 2^-60) next to O(1) ones: the unscaled pass flags those steps, finds
    their largest magnitudes normal and keeps its result, which must match FP64
    within the mixed tolerance.  An all-small tensor is the 1e-12 case above."""
    (tmp_path / "skew.gate").write_text("1 0 0 (1e-12,0)")
    qasm = "3\ndef1 SKEW skew.gate\nH 0\nH 1\nCNOT 0 1\nSKEW 0\nSKEW 1\nRx 0.3 2\nCNOT 1 2\nSKEW 2\nH 2\n"
    plan = qg.Plan(qasm, "0 T T", ordering="linegraph", gate_dir=str(tmp_path), ctx=ctx)
    v64 = plan.execute(qg.FP64)
    b = qg.Batch(ctx)
    b.add(plan)
    vmx = b.execute(qg.MIXED)[0]
    assert abs(vmx - v64) <= MIXED_TOL
