"""Host-side check of the streaming kernel's tiling (no GPU): the C++ emulator
walks every tile of random steps exactly as the kernel's threads do, using the
library's own stream_plan, and checks every index against its buffer, that
each output is written exactly once, and the values against a direct
evaluation (tests/stream_emulator.cpp)."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.fixture(scope="module")
def emulator(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("emu") / "stream_emulator")
    lib = os.path.join(REPO, "qtorch_gb300", "_lib")
    cmd = ["g++", "-O2", "-std=c++17", f"-I{CUDA}/include", "-o", exe, os.path.join(REPO, "tests", "stream_emulator.cpp"),
           f"-L{lib}", "-lqtorch_gb300", f"-L{CUDA}/lib64", "-lcudart", f"-Wl,-rpath,{lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("seed", [1, 2])
def test_stream_tiling_covers_every_output_once(emulator, seed):
    r = subprocess.run([emulator, str(seed), "40"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    ok, checked, planned = r.stdout.split()
    assert ok == "ok" and int(checked) == int(planned) >= 20
