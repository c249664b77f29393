"""The drop-in in C++ (no Python between the caller and the engine).

1. A C++ program compiled against include/qtorch/qtorch.hpp and linked to
   libqtorch_gb300.so runs the reference's sample circuits through
   ContractionTools and LineGraph: the given sequence reproduces the
   reference's value bit for bit, the seeded stochastic and line-graph
   orderings agree with it to the reference's own test tolerance (1e-5,
   src/tests.cpp), including its known answers -0.620705 for test_JW
   (tests.cpp:254-324) and 0.0035757 for the 20-node QAOA circuit
   (tests.cpp:425-472); a missing file throws the reference's InvalidFile.
2. The unmodified reference headers (staged in baseline/_ref/src) with the
   body of Network::ContractIndices replaced by a call to
   qt_contract_pair_host -- the binding INTEGRATION.md shows -- replay the
   recorded sequences and reproduce the reference's own values bit for bit.
"""
import os
import re
import shutil
import subprocess

import pytest

from conftest import REPO, load_golden

pytestmark = pytest.mark.gpu

CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
LIB = os.path.join(REPO, "qtorch_gb300", "_lib")
STAGED = os.path.join(REPO, "baseline", "_ref", "src")
LINK = [f"-L{LIB}", "-lqtorch_gb300", f"-L{CUDA}/lib64", "-lcudart", f"-Wl,-rpath,{LIB}", "-pthread"]


def cases(tmp_path):
    out = []
    for i, c in enumerate(load_golden("networks.json")):
        if c.get("gate_files"):
            continue
        q, m, s = tmp_path / f"c{i}.qasm", tmp_path / f"c{i}.meas", tmp_path / f"c{i}.seq"
        q.write_text(c["qasm"])
        m.write_text(c["measure"])
        s.write_text("\n".join(f"{a} {b}" for a, b in c["sequence"]) + "\n")
        out.append((c, str(q), str(m), str(s)))
    return out


def test_cpp_client_against_qtorch_hpp(tmp_path):
    exe = str(tmp_path / "client")
    r = subprocess.run(["g++", "-O2", "-std=c++17", f"-I{REPO}/include", f"-I{CUDA}/include", "-o", exe,
                        os.path.join(REPO, "tests", "cpp", "client.cpp")] + LINK, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cs = cases(tmp_path)
    args = [x for c in cs for x in c[1:]]
    r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=600, cwd=tmp_path)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("case ")]
    assert len(lines) == len(cs)
    for (c, *_), ln in zip(cs, lines):
        v = [float(x) for x in ln[2:8]]
        want = complex(*c["value"])
        assert complex(v[0], v[1]) == want, c["name"]                 # bit-exact replay
        assert abs(complex(v[2], v[3]) - want) <= 1e-5, c["name"]     # seeded stochastic
        assert abs(complex(v[4], v[5]) - want) <= 1e-5, c["name"]     # line graph
        assert int(ln[8]) == c["flops"]
        if c["name"] == "test_JW.qasm" and c["measure"].startswith("Z T T T"):
            assert abs(v[0] - -0.620705) <= 1e-5
        if c["name"] == "4regRand20Node1-p1.qasm":
            assert abs(v[0] - 0.0035757) <= 1e-5
    r = subprocess.run([exe, "missing"], capture_output=True, text=True, timeout=120)
    assert "exception Invalid Input or Output File Path" in r.stdout


# the reference's threaded MAC loop (src/Network.h:941-960) is replaced by the
# library call; the flop counter above it and the final-value rule below it stay
GPU_BODY = """        // GB300 engine: the contraction through the C ABI
        if (nodeA->GetTensorVals().size() == 0 || nodeB->GetTensorVals().size() == 0) {
            throw InvalidFunctionInput();
        }
        {
            static qt_ctx *qt_context = [] {
                qt_ctx *c = nullptr;
                if (qt_ctx_create(0, nullptr, &c) != QT_OK) throw ContractionFailure();
                return c;
            }();
            std::vector<uint8_t> ffa;
            std::vector<int32_t> fi, sa, sb;
            for (auto &f : toNotSumOn) { ffa.push_back(f.first ? 1 : 0); fi.push_back(f.second); }
            for (auto &s : toSumOn) { sa.push_back(s.first); sb.push_back(s.second); }
            if (qt_contract_pair_host(qt_context, reinterpret_cast<const double *>(nodeA->GetTensorVals().data()),
                                      nodeA->mRank, reinterpret_cast<const double *>(nodeB->GetTensorVals().data()),
                                      nodeB->mRank, (int) ffa.size(), ffa.data(), fi.data(), (int) sa.size(),
                                      sa.data(), sb.data(), reinterpret_cast<double *>(nodeC->GetTensorVals().data()))
                != QT_OK)
                throw ContractionFailure();
        }
"""


def patched_reference(dst):
    """Copy of the staged reference headers with the GPU body in ContractIndices."""
    shutil.copytree(STAGED, dst)
    path = os.path.join(dst, "Network.h")
    text = open(path).read()
    begin = text.index("//actually do the threading: using the lambda above")
    begin = text.rindex("\n", 0, begin) + 1
    end = text.index("if (toNotSumOn.size() == 0) {", begin)
    end = text.rindex("\n", 0, end) + 1
    text = text[:begin] + GPU_BODY + text[end:]
    text = re.sub(r'(#include "Exceptions.h")', r'\1\n#include "qtorch_gb300.h"', text, count=1)
    open(path, "w").write(text)


@pytest.mark.skipif(not os.path.isfile(os.path.join(STAGED, "Network.h")), reason="reference headers not staged")
def test_unmodified_reference_with_the_gpu_contract_indices(tmp_path):
    ref = str(tmp_path / "ref")
    patched_reference(ref)
    stub = tmp_path / "stub"
    stub.mkdir()
    (stub / "nlopt.hpp").write_text("")
    exe = str(tmp_path / "ref_gpu")
    r = subprocess.run(["g++", "-O2", "-std=c++11", "-w", f"-I{stub}", f"-I{ref}", f"-I{REPO}/include",
                        f"-I{CUDA}/include", "-o", exe, os.path.join(REPO, "oracle", "ref_harness.cpp")] + LINK,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    for c, q, m, s in cases(tmp_path):
        r = subprocess.run([exe, "seq", q, m, s], capture_output=True, text=True, timeout=300, cwd=tmp_path)
        assert r.returncode == 0, (c["name"], r.stdout[-500:], r.stderr[-500:])
        vals = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("value ")]
        flops = [int(ln.split()[1]) for ln in r.stdout.splitlines() if ln.startswith("flops ")]
        assert complex(float(vals[0][1]), float(vals[0][2])) == complex(*c["value"]), c["name"]
        assert flops[0] == c["flops"]
