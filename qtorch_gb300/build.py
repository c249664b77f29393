"""Build recipe of libqtorch_gb300.so (sm_103a only, no cmake).

The .cu translation units go through nvcc with one -gencode for sm_103a, the
host C++ through g++; everything links into qtorch_gb300/_lib/libqtorch_gb300.so.
Units compile in parallel and are skipped when their object is newer than the
sources, so a rebuild takes seconds.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libqtorch_gb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH
# -ffp-contract=off keeps the host-side gate tables rounded like the reference on every architecture
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-sign-compare",
             "-I" + os.path.join(CUDA, "include")]

CU_SOURCES = ["kernels.cu", "static_scratch.cu", "gemm_tc.cu", "stream.cu", "permute.cu"]
CXX_SOURCES = ["permute_plan.cpp", "core.cpp", "network.cpp", "orderings.cpp", "plan.cpp", "capi_host.cpp", "qaoa.cpp", "server.cpp", "slicing.cpp",
               "inp.cpp"]
HEADERS = ["engine.cuh", "kernels.h", "core.h", "plan.h", "gemm_tc.h", "scale.cuh", "stream.h", "permute.h", "dot2.cuh"]


def _deps():
    hs = [os.path.join(CSRC, h) for h in HEADERS]
    hs += [os.path.join(REPO, "include", "qtorch_gb300.h"), os.path.join(REPO, "include", "qtorch", "qtorch.hpp")]
    return max(os.path.getmtime(h) for h in hs)


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(path), _deps()):
        return obj, None
    if src.endswith(".cu"):
        cmd = [NVCC] + CU_FLAGS + ["-c", path, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = CU_SOURCES + CXX_SOURCES
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(_compile, srcs))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("build failed:\n" + "\n".join(errors))
    objs = [o for o, _ in results]
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC, "-shared", "-o", LIB] + objs + ARCH + ["-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
