"""Config 1 on the GPU: the FP64 form of each seeded 6-qubit circuit under its
recorded stochastic ordering equals the unmodified reference's value bit for
bit (tests/golden/config1.json); the mixed form is within 1e-6."""
import pytest

import qtorch_gb300 as qg
from conftest import load_golden

pytestmark = pytest.mark.gpu

CASES = load_golden("config1.json")


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"seed{c['seed']}")
def test_fp64_equals_the_reference(ctx, case):
    want = complex(*case["value"])
    for plan in (qg.Plan(case["qasm"], case["measure"], ordering="stochastic", seed=case["seed"], ctx=ctx),
                 qg.Plan(case["qasm"], case["measure"], ordering="sequence", sequence=case["sequence"], ctx=ctx)):
        assert plan.execute(qg.FP64) == want
        assert abs(plan.execute(qg.MIXED) - want) <= 1e-6


def test_network_path_equals_the_reference(ctx):
    """The reference-facing Network API (ContractNodes on device tensors) under
    the recorded sequence."""
    case = CASES[0]
    net = qg.Network(case["qasm"], case["measure"], ctx=ctx)
    net.contract_sequence(case["sequence"])
    assert net.final_value == complex(*case["value"])
