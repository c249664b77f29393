"""The tcgen05 tensor-core path for GEMM-shaped steps (3xTF32 complex products,
FP32 accumulation in tensor memory) against a complex128 reference."""
import numpy as np
import pytest

import qtorch_gb300 as qg
from oracle import port

pytestmark = pytest.mark.gpu


def reference_step(a, b, ffa, fi, sa, sb):
    return port.contract_indices(a.astype(np.complex128), b.astype(np.complex128), ffa, fi, sa, sb)


# (7, 9, 3), (6, 10, 2) and (7, 10, 3) have more free indices on B: X holds A as
# (Re, Im) row pairs; (6, 10, 2) sums 16 terms, both halves in one k tile
@pytest.mark.parametrize("ra,rb,ns", [(9, 7, 3), (8, 8, 4), (10, 6, 2), (7, 9, 3), (6, 10, 2), (7, 10, 3)])
def test_gemm_step_matches_complex128(ctx, ra, rb, ns):
    rng = np.random.default_rng(ra * 100 + rb * 10 + ns)
    sa = list(rng.permutation(ra)[:ns])
    sb = list(rng.permutation(rb)[:ns])
    fa = [i for i in range(ra) if i not in sa]
    fb = [i for i in range(rb) if i not in sb]
    ffa, fi = [1] * len(fa) + [0] * len(fb), fa + fb
    a = (rng.standard_normal(4 ** ra) + 1j * rng.standard_normal(4 ** ra)).astype(np.complex64)
    b = (rng.standard_normal(4 ** rb) + 1j * rng.standard_normal(4 ** rb)).astype(np.complex64)
    got = qg.contract_pair_c64(a, b, ffa, fi, sa, sb, ctx=ctx)
    want = reference_step(a, b, ffa, fi, sa, sb)
    # each term carries ~2^-21 relative error; the sum has 4^ns terms of unit size
    scale = np.sqrt(4 ** ns)
    assert np.max(np.abs(got - want)) <= 2e-5 * scale


def random_circuit(n, depth, seed):
    rng = np.random.default_rng(seed)
    lines = [str(n)]
    for _ in range(depth):
        for q in range(n):
            lines.append(f"{rng.choice(['Rx', 'Ry', 'Rz'])} {rng.uniform(0, 6.28):.4f} {q}")
        perm = rng.permutation(n)
        for j in range(0, n // 4 * 2, 2):
            lines.append(f"CZ {perm[j]} {perm[j + 1]}")
    return "\n".join(lines) + "\n"


def test_large_circuit_mixed_with_tensor_cores_matches_fp64(ctx):
    """A 16-qubit depth-12 random circuit: its heaviest steps (>= 2^26 complex
    MACs each) are GEMMs; the mixed result stays within 1e-6 of the FP64 one."""
    q = random_circuit(16, 12, 1)
    plan = qg.Plan(q, "Z", ordering="linegraph", ctx=ctx)
    info = plan.step_info(qg.MIXED)
    assert any(4 ** (int(r[3]) + int(r[4])) >= 1 << 26 for r in info)
    v64 = plan.execute(qg.FP64)
    vmx = plan.execute(qg.MIXED)
    assert abs(vmx - v64) <= 1e-6
