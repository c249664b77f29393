"""Parity of the CUDA path against the reference (golden fixtures) and the oracle.

FP64 form: bit-exact (the kernels sum every output element in the reference's
order with separately rounded multiplies and adds).  Mixed form: absolute error
<= 1e-6 against the FP64 result (the tolerance the target states)."""
import hashlib

import numpy as np
import pytest

import qtorch_gb300 as qg
from conftest import load_golden
from oracle import port, qaoa_terms
from test_oracle import pair_operands

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6
NETS = load_golden("networks.json")


def canon_digest(c):
    a = np.asarray(c, dtype=np.complex128).view(np.float64) + 0.0
    return hashlib.sha256(a.tobytes()).hexdigest()


def write_gate_files(tmp_path, case):
    for rel, text in case["gate_files"].items():
        p = tmp_path / rel
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_text(text)


@pytest.mark.parametrize("case", load_golden("pairs.json"), ids=lambda c: f"r{c['rank_a']}x{c['rank_b']}s{c['n_sum']}")
def test_contract_pair_bit_exact(ctx, case):
    a, b, ffa, fi, sa, sb = pair_operands(case["seed"], case["rank_a"], case["rank_b"], case["n_sum"])
    c = qg.contract_pair(a, b, ffa, fi, sa, sb, ctx=ctx)
    assert canon_digest(c) == case["sha256"]


def test_contract_pair_device_buffers(ctx):
    """The device-pointer entry point on caller-owned memory (torch tensors on the context stream)."""
    import torch
    case = load_golden("pairs.json")[15]
    a, b, ffa, fi, sa, sb = pair_operands(case["seed"], case["rank_a"], case["rank_b"], case["n_sum"])
    ta = torch.from_numpy(a).cuda()
    tb = torch.from_numpy(b).cuda()
    tc = torch.empty(4 ** len(fi), dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    qg.contract_pair_device(ta.data_ptr(), case["rank_a"], tb.data_ptr(), case["rank_b"], ffa, fi, sa, sb,
                            tc.data_ptr(), ctx=ctx)
    ctx.synchronize()
    assert canon_digest(tc.cpu().numpy()) == case["sha256"]


def test_contract_pair_arbitrary_free_order(ctx):
    """toNotSumOn in any order (B's wires first, interleaved) matches the oracle bit for bit."""
    rng = np.random.default_rng(5)
    a = rng.standard_normal(4 ** 3) + 1j * rng.standard_normal(4 ** 3)
    b = rng.standard_normal(4 ** 3) + 1j * rng.standard_normal(4 ** 3)
    ffa, fi, sa, sb = [0, 1, 0, 1], [2, 0, 0, 2], [1], [1]
    assert np.array_equal(qg.contract_pair(a, b, ffa, fi, sa, sb, ctx=ctx),
                          port.contract_indices(a, b, ffa, fi, sa, sb))


def test_contract_pair_rejects_bad_maps(ctx):
    with pytest.raises(qg.QtError):
        qg.contract_pair(np.ones(16), np.ones(16), [1, 1], [0, 0], [1], [1], ctx=ctx)


@pytest.mark.parametrize("case", NETS, ids=lambda c: c["name"] + ":" + c["measure"][:12])
def test_network_replay_bit_exact(ctx, case, tmp_path):
    """ContractGivenSequence on the GPU reproduces the reference's value bit for bit."""
    write_gate_files(tmp_path, case)
    n = qg.Network(case["qasm"], case["measure"], gate_dir=str(tmp_path), ctx=ctx)
    n.contract_sequence(case["sequence"])
    assert n.final_value == complex(*case["value"])
    assert n.flops == case["flops"]


@pytest.mark.parametrize("case", NETS[:8], ids=lambda c: c["name"] + ":" + c["measure"][:12])
@pytest.mark.parametrize("ordering", ["stochastic", "linegraph"])
def test_orderings_on_gpu_match_oracle(ctx, case, ordering, tmp_path):
    write_gate_files(tmp_path, case)
    n = qg.Network(case["qasm"], case["measure"], gate_dir=str(tmp_path), ctx=ctx)
    if ordering == "stochastic":
        n.contract_stochastic(31)
    else:
        n.contract_linegraph()
    v_oracle, _ = port.replay_value(case["qasm"], case["measure"], n.created_from(), gate_dir=str(tmp_path))
    assert n.final_value == v_oracle


@pytest.mark.parametrize("case", NETS, ids=lambda c: c["name"] + ":" + c["measure"][:12])
def test_plan_fp64_bit_exact_and_mixed_within_tolerance(ctx, case, tmp_path):
    write_gate_files(tmp_path, case)
    plan = qg.Plan(case["qasm"], case["measure"], ordering="sequence", sequence=case["sequence"],
                   gate_dir=str(tmp_path), ctx=ctx)
    ref = complex(*case["value"])
    assert plan.execute(qg.FP64) == ref
    assert abs(plan.execute(qg.MIXED) - ref) <= MIXED_TOL


def qaoa_batch(ctx, dgf, p, points, prec, graph=False):
    """All edge terms at every (beta, gamma) point, one batch; returns values and the term list."""
    n_edges = qg.qaoa_num_edges(dgf)
    terms = []
    b = qg.Batch(ctx)
    for bg in points:
        for e in range(n_edges):
            qasm, meas = qg.qaoa_term_text(dgf, p, bg, e)
            plan = qg.Plan(qasm, meas, ordering="linegraph", ctx=ctx)
            b.add(plan)
            terms.append((qasm, meas, plan))
    if graph:
        b.use_graph(True)
    return b.execute(prec), terms, b


def test_qaoa_p1_batch_fp64_matches_oracle_and_mixed_error(ctx):
    dgf = qg.random_regular_graph(30, 4, seed=1)
    rng = np.random.default_rng(0)
    points = [list(rng.uniform(0, np.pi, 2)) for _ in range(2)]
    v64, terms, _ = qaoa_batch(ctx, dgf, 1, points, qg.FP64)
    vmx, _, _ = qaoa_batch(ctx, dgf, 1, points, qg.MIXED)
    for k, (qasm, meas, plan) in enumerate(terms):
        v_or, _ = port.replay_value(qasm, meas, plan.sequence())
        assert v64[k] == v_or, k
    err = np.abs(vmx - v64)
    assert err.max() <= MIXED_TOL, err.max()


def test_qaoa_term_text_through_plan_matches_reference_generator(ctx):
    g = load_golden("qaoa.json")[0]
    for k in range(0, len(g["terms"]), 7):
        qasm = g["terms"][k]["qasm"]
        meas = qaoa_terms.term_measure(g["terms"][k]["qubits"])
        plan = qg.Plan(qasm, meas, ordering="linegraph", ctx=ctx)
        v_or, _ = port.replay_value(qasm, meas, plan.sequence())
        assert plan.execute(qg.FP64) == v_or


def test_batch_graph_replay_equals_direct(ctx):
    dgf = qg.random_regular_graph(20, 3, seed=4)
    pts = [[0.4, 1.1]]
    v1, _, _ = qaoa_batch(ctx, dgf, 1, pts, qg.FP64)
    v2, _, b = qaoa_batch(ctx, dgf, 1, pts, qg.FP64, graph=True)
    assert np.array_equal(v1, v2)
    b.run()
    assert np.array_equal(b.fetch(), v1)


def test_batch_set_leaves_changes_angles(ctx):
    dgf = qg.random_regular_graph(20, 3, seed=4)
    q1, m1 = qg.qaoa_term_text(dgf, 1, [0.4, 1.1], 0)
    q2, m2 = qg.qaoa_term_text(dgf, 1, [0.9, 0.2], 0)
    p1 = qg.Plan(q1, m1, ordering="linegraph", ctx=ctx)
    p2 = qg.Plan(q2, m2, ordering="linegraph", ctx=ctx)
    assert p1.sequence() == p2.sequence()   # same structure, other angles
    b = qg.Batch(ctx)
    b.add(p1)
    b.prepare(qg.FP64)
    b.run()
    first = b.fetch()[0]
    b.set_leaves(0, p2.leaf_values())
    b.upload()
    b.run()
    assert b.fetch()[0] == p2.execute(qg.FP64)
    assert first == p1.execute(qg.FP64)


def test_large_plan_runs_step_by_step(ctx):
    """A plan whose intermediates exceed the grouped limits runs with the whole-GPU kernel."""
    case = [c for c in NETS if c["name"] == "4regRand20Node1-p1.qasm"][0]
    plan = qg.Plan(case["qasm"], case["measure"], ordering="sequence", sequence=case["sequence"], ctx=ctx)
    assert plan.execute(qg.FP64) == complex(*case["value"])


def test_deadline_expires_with_an_error(ctx):
    case = NETS[0]
    n = qg.Network(case["qasm"], case["measure"], ctx=ctx)
    ctx.set_deadline(1e-9)
    try:
        with pytest.raises(qg.DeadlineExpired):
            n.contract_sequence(case["sequence"])
    finally:
        ctx.set_deadline(0)
    ctx.synchronize()


def test_memory_budget_is_enforced():
    c = qg.Context(0)
    try:
        c.set_memory_budget(1024)
        with pytest.raises(qg.OutOfMemory):
            qg.contract_pair(np.ones(4 ** 6), np.ones(4 ** 6), [1] * 5 + [0] * 5, list(range(1, 6)) + list(range(1, 6)),
                             [0], [0], ctx=c)
    finally:
        c.close()
