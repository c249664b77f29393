""".inp scripts (src/leviParser.hpp, the flow of src/main.cpp): parse, ReduceCircuit,
contract with the chosen method, write the result file."""
import pytest

import qtorch_gb300 as qg
from conftest import load_golden

CASE = [c for c in load_golden("networks.json") if c["name"] == "test_JW.qasm"][0]


def write_case(tmp_path, method, extra=""):
    (tmp_path / "c.qasm").write_text(CASE["qasm"])
    (tmp_path / "m.txt").write_text(CASE["measure"])
    inp = tmp_path / "run.inp"
    inp.write_text("# comment line\n>int threads 8\n>string qasm c.qasm\n>string measurement m.txt\n"
                   f">string contractmethod {method}\n>string outputpath out.txt\n{extra}")
    return str(inp)


@pytest.mark.parametrize("method", ["linegraph-qbb", "simple-stoch"])
def test_inp_flow_symbolic(tmp_path, monkeypatch, method):
    monkeypatch.chdir(tmp_path)
    inp = write_case(tmp_path, method, ">int seed 4\n")
    _, flops = qg.run_inp(inp, symbolic=True)
    assert flops > 0
    assert (tmp_path / "out.txt").read_text().startswith("Result of Contraction:")
    if method == "linegraph-qbb":
        text = (tmp_path / "output" / "qbb.out").read_text().split("\n")
        assert text[0] == " The optimal ordering is "
        assert sorted(int(x) for x in text[1].split()) == list(range(1, len(text[1].split()) + 1))


def test_inp_qbbonly_then_readqbbresonly(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    qg.run_inp(write_case(tmp_path, "linegraph-qbb", ">bool qbbonly true\n"), symbolic=True)
    order = (tmp_path / "output" / "qbb.out").read_text()
    _, f1 = qg.run_inp(write_case(tmp_path, "linegraph-qbb", ">bool readqbbresonly true\n"), symbolic=True)
    _, f2 = qg.run_inp(write_case(tmp_path, "linegraph-qbb"), symbolic=True)
    assert f1 == f2 > 0
    assert (tmp_path / "output" / "qbb.out").read_text() == order


def test_inp_bad_method(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    with pytest.raises(qg.InvalidContractionMethod):
        qg.run_inp(write_case(tmp_path, "cost-based"), symbolic=True)


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["linegraph-qbb", "simple-stoch"])
def test_inp_value_on_gpu(ctx, tmp_path, monkeypatch, method):
    monkeypatch.chdir(tmp_path)
    v, _ = qg.run_inp(write_case(tmp_path, method, ">int seed 4\n"), ctx=ctx)
    ref = complex(*CASE["value"])
    assert abs(v - ref) <= 1e-12
