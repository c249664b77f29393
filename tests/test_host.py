"""Host-side logic of the product without a GPU: the C ABI library loads and
exports every declared symbol, and the symbolic network (ContractNodes
bookkeeping with no data), the orderings, the planner and the workload
generators agree with the reference's golden fixtures and the oracle."""
import os
import re

import numpy as np
import pytest

import qtorch_gb300 as qg
from conftest import REPO, load_golden
from oracle import port, qaoa_terms

NETS = load_golden("networks.json")


def declared_symbols():
    text = open(os.path.join(REPO, "include", "qtorch_gb300.h")).read()
    return sorted(set(re.findall(r"\b(qt_[a-z_0-9]+)\(", text)))


def test_library_exports_every_declared_symbol():
    lib = qg._capi.load()
    names = declared_symbols()
    assert len(names) > 60
    for n in names:
        assert hasattr(lib, n), n
    assert {s[0] for s in qg._capi.SIGNATURES} == set(names)


def test_no_device_is_an_error_not_a_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(qg.QtError):
        qg.Context(0)


def write_gate_files(tmp_path, case):
    for rel, text in case["gate_files"].items():
        p = tmp_path / rel
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_text(text)


@pytest.mark.parametrize("case", NETS, ids=lambda c: c["name"] + ":" + c["measure"][:12])
def test_symbolic_replay_records_the_same_sequence(case, tmp_path):
    write_gate_files(tmp_path, case)
    n = qg.Network(case["qasm"], case["measure"], gate_dir=str(tmp_path), symbolic=True)
    n.contract_sequence(case["sequence"])
    assert n.is_done
    assert [list(p) for p in n.created_from()] == case["sequence"]
    assert n.flops == case["flops"]


@pytest.mark.parametrize("case", NETS, ids=lambda c: c["name"] + ":" + c["measure"][:12])
@pytest.mark.parametrize("ordering", ["stochastic", "linegraph"])
def test_orderings_give_reference_values(case, ordering, tmp_path):
    """An ordering of this build, replayed by the oracle, reproduces the reference's value."""
    write_gate_files(tmp_path, case)
    n = qg.Network(case["qasm"], case["measure"], gate_dir=str(tmp_path), symbolic=True)
    if ordering == "stochastic":
        n.contract_stochastic(2024)
    else:
        n.contract_linegraph()
    assert n.is_done
    v, _ = port.replay_value(case["qasm"], case["measure"], n.created_from(), gate_dir=str(tmp_path))
    ref = complex(*case["value"])
    # a different ordering sums in a different order: agreement to rounding level
    assert abs(v - ref) <= 1e-12 * max(1.0, abs(ref))


def test_stochastic_ordering_is_reproducible():
    case = NETS[0]
    seqs = []
    for _ in range(2):
        n = qg.Network(case["qasm"], case["measure"], symbolic=True)
        n.contract_stochastic(99)
        seqs.append(n.created_from())
    assert seqs[0] == seqs[1]


@pytest.mark.parametrize("g", load_golden("linegraph.json"), ids=lambda g: g["name"])
def test_linegraph_order_is_a_permutation_of_wires(g):
    n = qg.Network(g["qasm"], g["measure"], symbolic=True)
    order = n.linegraph_order()
    n_wires = len({w[0] for node in g["nodes"] for w in node["wires"]})
    assert sorted(order) == list(range(1, n_wires + 1))


def test_linegraph_replay_matches_oracle_walk():
    """LGContract over a wire order: this build and the oracle's restatement record the same pairs."""
    case = NETS[0]
    n = qg.Network(case["qasm"], case["measure"], symbolic=True)
    order = n.linegraph_order()
    n.contract_wire_order(order)
    o = port.Net(case["qasm"], case["measure"])
    o.lg_contract(order)
    assert [tuple(p) for p in n.created_from()] == o.created_from()
    assert o.remaining_value == o.final_value


@pytest.mark.parametrize("g", load_golden("qaoa.json"), ids=lambda g: f"{g['dgf_name']}-p{g['p']}")
def test_qaoa_term_generator_matches_reference(g):
    assert qg.qaoa_num_edges(g["dgf"]) == len(g["terms"])
    for k, ref in enumerate(g["terms"]):
        qasm, meas = qg.qaoa_term_text(g["dgf"], g["p"], g["betas_gammas"], k)
        assert qasm == ref["qasm"]
        assert meas == qaoa_terms.term_measure(ref["qubits"])


@pytest.mark.parametrize("n,d,seed", [(30, 4, 1), (50, 3, 7), (20, 3, 3), (40, 3, 11)])
def test_random_regular_graph(n, d, seed):
    text = qg.random_regular_graph(n, d, seed)
    pairs, nq = qaoa_terms.read_dgf(text)
    deg = np.zeros(n, dtype=int)
    seen = set()
    for a, b in pairs:
        assert a != b and (min(a, b), max(a, b)) not in seen
        seen.add((min(a, b), max(a, b)))
        deg[a] += 1
        deg[b] += 1
    assert (deg == d).all() and len(pairs) == n * d // 2
    assert text == qg.random_regular_graph(n, d, seed)


def test_symbolic_plan_properties():
    g = load_golden("qaoa.json")[0]
    qasm, meas = qg.qaoa_term_text(g["dgf"], 1, [0.3, 0.7], 0)
    p = qg.Plan(qasm, meas, ordering="linegraph", symbolic=True)
    assert p.num_steps == p.num_leaves - 1
    seq = p.sequence()
    v, fl = port.replay_value(qasm, meas, seq)
    assert fl == p.flops
    # the leaves the plan binds are the reference's gate tables in node order
    leaves = p.leaf_values()
    net = port.Net(qasm, meas)
    ref = np.concatenate([net.node_values(i) for i in range(p.num_leaves)])
    assert np.array_equal(leaves, ref)
    assert p.workspace_bytes(qg.MIXED) <= p.workspace_bytes(qg.FP64)


def test_parse_errors_map_to_reference_exceptions():
    with pytest.raises(qg.InvalidFileFormat):
        qg.Network("2\nCNOT 0 0\n", "", symbolic=True)
    with pytest.raises(qg.InvalidFileFormat):
        qg.Network("2\nFOO 1\n", "", symbolic=True)
    with pytest.raises(qg.InvalidFileFormat):
        qg.Network("2\nH 7\n", "", symbolic=True)
    with pytest.raises(qg.InvalidFileFormat):
        qg.Network("two\nH 0\n", "", symbolic=True)
    with pytest.raises(qg.InvalidFile):
        qg.Network("1\ndef1 G /nonexistent/gate.gate\nG 0\n", "", symbolic=True)


def test_sequence_that_does_not_finish_is_contraction_failure():
    case = NETS[0]
    n = qg.Network(case["qasm"], case["measure"], symbolic=True)
    with pytest.raises(qg.ContractionFailure):
        n.contract_sequence(case["sequence"][:3])


def test_user_defined_sequence_of_wires():
    """ContractUserDefinedSequenceOfWires replays a recorded order (tests.cpp:772-853)."""
    case = NETS[0]
    n_orig = qg.Network(case["qasm"], case["measure"], symbolic=True).num_nodes
    # the file names original nodes: a merged node stands for its first parent
    to_orig, pairs = {}, []
    for new_id, (a, b) in enumerate(case["sequence"], start=n_orig):
        while a in to_orig:
            a = to_orig[a]
        while b in to_orig:
            b = to_orig[b]
        to_orig[new_id] = a
        pairs.append((a, b))
    text = "\n".join(f"{a} {b}" for a, b in pairs) + "\n"
    n = qg.Network(case["qasm"], case["measure"], symbolic=True)
    n.contract_user_sequence(text)
    assert n.is_done
    bad = qg.Network(case["qasm"], case["measure"], symbolic=True)
    with pytest.raises(qg.InvalidUserContractionSequence):
        bad.contract_user_sequence("0 1\n")


def test_reduce_circuit_then_contract():
    """ReduceCircuit (Network.h:1015-1118) folds gates; the reduced network still gives the value."""
    case = [c for c in NETS if c["name"] == "test_JW.qasm"][0]
    n = qg.Network(case["qasm"], case["measure"], symbolic=True)
    before = n.num_uncontracted
    n.reduce()
    assert n.num_uncontracted < before
    n.contract_stochastic(5)
    assert n.is_done


@pytest.mark.parametrize("case", load_golden("reduce.json"), ids=lambda c: c["name"])
def test_reduce_circuit_matches_reference(case):
    """ReduceCircuit makes the reference's contractions in the reference's order (Network.h:1015-1118)."""
    n = qg.Network(case["qasm"], case["measure"], symbolic=True)
    n.reduce()
    assert [list(p) for p in n.created_from()] == case["reduce_sequence"]
    assert [n.num_nodes, n.num_uncontracted] == case["reduced_nodes"]
    rest = case["sequence"][len(case["reduce_sequence"]):]
    n.contract_sequence(rest)
    assert n.is_done
    v, _ = port.replay_value(case["qasm"], case["measure"], case["sequence"])
    assert v == complex(*case["value"])


def test_interpreter_schedule_invariants():
    """Steps run level by level; inside a level the CTA-tiled products come
    last, and only steps that are products of two wide gathered matrices
    (>= 16 rows each side, >= 1024 outputs) are tiled."""
    dgf = qg.random_regular_graph(26, 3, seed=105)
    seen_tiled = 0
    for e in range(0, qg.qaoa_num_edges(dgf), 5):
        q, m = qg.qaoa_term_text(dgf, 2, [0.3, 0.9, 0.7, 0.2], e)
        plan = qg.Plan(q, m, ordering="linegraph", symbolic=True)
        for prec in (qg.FP64, qg.MIXED):
            si = plan.step_info(prec)
            assert len(si) == plan.num_steps
            assert np.all(np.diff(si[:, 0]) >= 0)
            for level in np.unique(si[:, 0]):
                tiled = (si[si[:, 0] == level, 6] & 128) != 0
                # a suffix of the level
                assert not np.any(tiled[:-1] & ~tiled[1:])
            for ra, rb, rc, ns, g, flags in si[:, 1:7]:
                if flags & 128:
                    fa, fb = ra - ns, rb - ns
                    assert fa >= 2 and fb >= 2 and ns >= 1 and g == 1
                    seen_tiled += 1
                elif prec == qg.FP64:
                    assert g == 1   # the FP64 form keeps one accumulator per output
    assert seen_tiled > 0


def test_linegraph_ordering_keeps_the_tree_shallow():
    """The line-graph order is picked for the lowest estimated GPU time among
    min-fill variants (shallow ties, seeded restarts, fill slack): every
    light-cone term of a 30-vertex 4-regular p=1 QAOA has at most 10 dependent
    levels (31 with classic min-fill) at peak rank 4."""
    dgf = qg.random_regular_graph(30, 4, seed=1)
    for e in range(qg.qaoa_num_edges(dgf)):
        q, m = qg.qaoa_term_text(dgf, 1, [0.3, 0.7], e)
        plan = qg.Plan(q, m, ordering="linegraph", symbolic=True)
        assert plan.peak_rank <= 4
        assert plan.step_info(qg.MIXED)[:, 0].max() + 1 <= 10
