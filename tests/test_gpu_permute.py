"""The tiled index permutation (qt_tensor_permute, permute.cu) against numpy,
bit for bit, and the permuted full contraction that the complex64 path takes
for the expectation value of a large network (Dot2 sums, within 1e-6 of the
complex128 value)."""
import numpy as np
import pytest

import qtorch_gb300 as qg

pytestmark = pytest.mark.gpu


def reference_permute(x, perm):
    """digit i of the result = digit perm[i] of x; numpy axis k is digit r-1-k"""
    r = len(perm)
    if r == 0:
        return x.copy()
    return x.reshape([4] * r).transpose([r - 1 - perm[r - 1 - k] for k in range(r)]).reshape(-1)


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("rank", [0, 1, 2, 3, 4, 5, 6, 7, 9, 11])
def test_permute_matches_numpy(ctx, dtype, rank):
    rng = np.random.default_rng(rank * 7 + (dtype == np.complex64))
    x = (rng.standard_normal(4 ** rank) + 1j * rng.standard_normal(4 ** rank)).astype(dtype)
    for trial in range(3):
        perm = list(rng.permutation(rank)) if trial else list(range(rank))[::-1]
        y = qg.permute(x, perm, ctx=ctx)
        assert y.dtype == x.dtype
        assert np.array_equal(y, reference_permute(x, perm)), (rank, perm)


def test_permute_round_trip_at_rank_13(ctx):
    """537 MB complex64: the permutation then its inverse gives x back bit for
    bit, and sampled entries sit where the index map puts them."""
    rng = np.random.default_rng(5)
    r = 13
    x = np.empty(4 ** r, dtype=np.complex64)
    x.real = rng.standard_normal(4 ** r, dtype=np.float32)
    x.imag = rng.standard_normal(4 ** r, dtype=np.float32)
    perm = [int(v) for v in rng.permutation(r)]
    inv = [0] * r
    for i, p in enumerate(perm):
        inv[p] = i
    y = qg.permute(x, perm, ctx=ctx)
    for idx in rng.integers(0, 4 ** r, 200):
        src = sum(((int(idx) >> (2 * i)) & 3) << (2 * perm[i]) for i in range(r))
        assert y[idx] == x[src]
    assert np.array_equal(qg.permute(y, inv, ctx=ctx), x)


def test_permute_rejects_a_non_permutation(ctx):
    x = np.zeros(4 ** 3, dtype=np.complex64)
    for bad in ([0, 0, 1], [0, 1, 3], [0, 1]):
        with pytest.raises(qg.QtError):
            qg.permute(x, bad, ctx=ctx)


@pytest.mark.parametrize("rank", [6, 10, 12])
def test_full_contraction_of_permuted_operands(ctx, rank):
    rng = np.random.default_rng(rank)
    a = (rng.standard_normal(4 ** rank) + 1j * rng.standard_normal(4 ** rank)).astype(np.complex64)
    b = (rng.standard_normal(4 ** rank) + 1j * rng.standard_normal(4 ** rank)).astype(np.complex64)
    sum_a = [int(v) for v in rng.permutation(rank)]
    sum_b = [int(v) for v in rng.permutation(rank)]
    got = qg.contract_pair_c64(a, b, [], [], sum_a, sum_b, ctx=ctx)[0]
    # pair j joins A wire sum_a[j] and B wire sum_b[j]: B in A's digit order
    perm = [0] * rank
    for j in range(rank):
        perm[sum_a[j]] = sum_b[j]
    b_in_a = reference_permute(b.astype(np.complex128), perm)
    want = np.dot(a.astype(np.complex128), b_in_a)
    scale = np.sum(np.abs(a.astype(np.complex128)) * np.abs(b_in_a))
    assert abs(got - want) <= 1e-6 * scale, (got, want)
