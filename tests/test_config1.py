"""Config 1: seeded 6-qubit depth-10 Rx + CZ circuits, <Z_0>, fixed-seed
stochastic ordering.  tests/golden/config1.json holds, per seed, the circuit,
the ordering this build records for it and the unmodified reference's value
and flop count for that ordering (ContractGivenSequence,
src/ContractionTools.h:392-411).  On the CPU: the generator and the ordering
are reproducible, and the oracle's replay equals the reference bit for bit."""
import pytest

import qtorch_gb300 as qg
from conftest import load_golden
from qtorch_gb300.circuits import config1_circuit_text
from oracle import port

CASES = load_golden("config1.json")


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"seed{c['seed']}")
def test_generator_and_ordering_are_reproducible(case):
    assert config1_circuit_text(case["seed"]) == case["qasm"]
    plan = qg.Plan(case["qasm"], case["measure"], ordering="stochastic", seed=case["seed"], symbolic=True)
    assert [list(p) for p in plan.sequence()] == case["sequence"]
    assert plan.flops == case["flops"]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"seed{c['seed']}")
def test_oracle_replay_equals_the_reference(case):
    v, flops = port.replay_value(case["qasm"], case["measure"], case["sequence"])
    assert flops == case["flops"]
    assert v == complex(*case["value"])
    assert abs(v) > 1e-3


def test_circuit_shape():
    lines = config1_circuit_text(7).splitlines()
    assert lines[0] == "6"
    gates = [ln.split() for ln in lines[1:]]
    assert sum(g[0] == "Rx" for g in gates) == 60
    cz = [g for g in gates if g[0] == "CZ"]
    assert len(cz) == 20
    for layer in range(10):
        a, b = cz[2 * layer], cz[2 * layer + 1]
        assert len({a[1], a[2], b[1], b[2]}) == 4   # two disjoint pairs
