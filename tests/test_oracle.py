"""The CPU oracle port against golden vectors generated by the unmodified reference.

Bit-exact: gate tensors (src/Node.h), single ContractIndices calls
(src/Network.h:876-971) and whole-network replays of recorded orderings
(ContractGivenSequence, src/ContractionTools.h:392-411).
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import load_golden
from oracle import port, qaoa_terms


def canon_digest(c):
    a = np.asarray(c, dtype=np.complex128).view(np.float64) + 0.0
    return hashlib.sha256(a.tobytes()).hexdigest()


def pair_operands(seed, ra, rb, ns):
    """Same generator as tests/golden/make_golden.py."""
    rng = np.random.default_rng(seed)
    sa = [int(x) for x in rng.permutation(ra)[:ns]]
    sb = [int(x) for x in rng.permutation(rb)[:ns]]
    fa = [i for i in range(ra) if i not in sa]
    fb = [i for i in range(rb) if i not in sb]
    a = rng.standard_normal(4 ** ra) + 1j * rng.standard_normal(4 ** ra)
    b = rng.standard_normal(4 ** rb) + 1j * rng.standard_normal(4 ** rb)
    return a, b, [1] * len(fa) + [0] * len(fb), fa + fb, sa, sb


def gate_case(g):
    name = g["name"]
    if name.startswith("ARB"):
        return None
    if ":" in name:
        kind, p = name.split(":")
        return port.gate_tensor(kind, float(p))
    return port.gate_tensor(name)


@pytest.mark.parametrize("g", load_golden("gates.json"), ids=lambda g: g["name"])
def test_gate_tensors_bit_exact(g):
    mine = gate_case(g)
    if mine is None:
        pytest.skip("arbitrary gate files are checked through network replays")
    ref = np.array([complex(a, b) for a, b in g["values"]])
    assert mine.size == ref.size == 4 ** g["rank"]
    assert np.array_equal(mine.view(np.float64), ref.view(np.float64))


@pytest.mark.parametrize("case", load_golden("pairs.json"), ids=lambda c: f"r{c['rank_a']}x{c['rank_b']}s{c['n_sum']}")
def test_contract_indices_bit_exact(case):
    a, b, ffa, fi, sa, sb = pair_operands(case["seed"], case["rank_a"], case["rank_b"], case["n_sum"])
    assert ffa == case["free_from_a"] and fi == case["free_idx"] and sa == case["sum_a"] and sb == case["sum_b"]
    c = port.contract_indices(a, b, ffa, fi, sa, sb)
    assert canon_digest(c) == case["sha256"]
    if "c" in case:
        ref = np.array([complex(x, y) for x, y in case["c"]])
        assert np.array_equal(c, ref)


def write_gate_files(tmp_path, case):
    for rel, text in case["gate_files"].items():
        p = tmp_path / rel
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_text(text)


@pytest.mark.parametrize("case", load_golden("networks.json"), ids=lambda c: c["name"] + ":" + c["measure"][:12])
def test_network_replay_bit_exact(case, tmp_path):
    write_gate_files(tmp_path, case)
    net = port.Net(case["qasm"], case["measure"], gate_dir=str(tmp_path))
    net.replay(case["sequence"])
    v = net.final_value
    assert v == complex(*case["value"])
    assert v == complex(*case["replay_value"])
    assert net.flops == case["flops"]
    assert [list(p) for p in net.created_from()] == case["sequence"]


@pytest.mark.parametrize("g", load_golden("qaoa.json"), ids=lambda g: f"{g['dgf_name']}-p{g['p']}")
def test_qaoa_term_text(g):
    terms = qaoa_terms.all_terms(g["dgf"], g["p"], g["betas_gammas"])
    assert len(terms) == len(g["terms"])
    for (edge, qasm, meas), ref in zip(terms, g["terms"]):
        assert list(edge) == ref["edge"]
        assert qasm == ref["qasm"]
        assert int(qasm.split("\n")[0]) == ref["qubits"]


@pytest.mark.parametrize("g", load_golden("linegraph.json"), ids=lambda g: g["name"])
def test_linegraph_wire_numbering(g):
    net = port.Net(g["qasm"], g["measure"])
    mine = net.lg_wire_ids()
    ref = [(n["node"], [w[0] for w in n["wires"]]) for n in g["nodes"]]
    assert mine[: len(ref)] == ref


def test_known_answers_from_reference_tests():
    """A few of the reference's own KATs (src/tests.cpp), through the oracle."""
    # Ry(0.1) measured in X / Z (tests.cpp:483-525)
    for meas, want in (("X", 0.0998334), ("Z", 0.995004), ("Y", 0.0)):
        net = port.Net("1\nRy 0.1 0\n", meas)
        net.contract(0, 1, 100)
        net.contract(2, 3, 100)
        assert abs(net.final_value.real - want) < 1e-5
    # Bell pair |00> -> P(00) = 0.5 (tests.cpp:1120-1135)
    net = port.Net("2\nH 0\nCNOT 0 1\n", "0 0")
    # nodes: 0,1 initial states, 2 H, 3 CNOT, 4,5 projectors; new nodes take ids 6, 7, ...
    seq = [(0, 2), (6, 3), (1, 7), (4, 8), (5, 9)]
    for a, b in seq:
        net.contract(a, b, 100)
    assert net.done and abs(net.final_value.real - 0.5) < 1e-12


def test_parse_errors():
    with pytest.raises(port.OracleError):
        port.Net("2\nCNOT 0 0\n", "")
    with pytest.raises(port.OracleError):
        port.Net("2\nFOO 1\n", "")
    with pytest.raises(port.OracleError):
        port.Net("2\nH 5\n", "")
