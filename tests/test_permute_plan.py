"""Host-side check of the tiled index permutation's tiling (no GPU): the C++
emulator (tests/permute_emulator.cpp) plans random permutations with the
library's permute_plan and walks every tile as the kernel's threads do,
checking bounds, alignment, single writes and every output element."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.fixture(scope="module")
def emulator(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("perm") / "permute_emulator")
    cmd = ["g++", "-O2", "-std=c++17", f"-I{CUDA}/include", "-o", exe, os.path.join(REPO, "tests", "permute_emulator.cpp"),
           os.path.join(REPO, "qtorch_gb300", "csrc", "permute_plan.cpp")]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_permute_tiling_covers_every_output_once(emulator, seed):
    r = subprocess.run([emulator, str(seed), "40"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok"), r.stdout
