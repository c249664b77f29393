"""Index slicing (qt_plan_slice): a plan split over the values of a few cut
wires so that one slice's workspace fits a budget.  The value is the sum over
the slices (the network value is linear in every leaf), so it must equal the
unsliced value: to a few ulp in FP64 (the summation order differs) and within
the mixed tolerance in the mixed form."""
import numpy as np
import pytest

import qtorch_gb300 as qg
from qtorch_gb300.circuits import qft_text, random_circuit_text

CIRCUITS = {"rand12": lambda: random_circuit_text(12, 10, 1), "qft10": lambda: qft_text(10, 4),
            "rand12b": lambda: random_circuit_text(12, 12, 5)}


@pytest.mark.parametrize("name", sorted(CIRCUITS))
@pytest.mark.parametrize("div", [4, 16])
def test_slicing_meets_the_budget(name, div):
    p = qg.Plan(CIRCUITS[name](), "Z", ordering="linegraph", symbolic=True)
    ws = p.workspace_bytes(qg.FP64)
    s = p.slice(ws // div, qg.FP64, 8)
    assert 1 <= s.num_cuts <= 8
    assert s.workspace_bytes(qg.FP64) <= ws // div
    rows = qg._lib().qt_plan_step_info
    n = qg._lib().qt_plan_num_steps(qg._lib().qt_sliced_plan(s.handle))
    info = np.zeros((n, 8), dtype=np.int32)
    rows(qg._lib().qt_sliced_plan(s.handle), qg.FP64, info.ctypes.data_as(qg.ctypes.POINTER(qg.ctypes.c_int32)), n)
    # one rank-0 result per slice: the final-value rule sees the same shape of network
    assert int((info[:, 3] == 0).sum()) == 1
    # the slice's own leaves: the uncut ones whole, the cut ones one index smaller per cut
    sp = qg._lib().qt_sliced_plan(s.handle)
    assert qg._lib().qt_plan_num_leaves(sp) == p.num_leaves
    assert 0 < qg._lib().qt_plan_leaf_elems(sp) < p.leaf_values().size


def test_no_slicing_within_the_cut_limit_is_out_of_memory():
    p = qg.Plan(CIRCUITS["qft10"](), "Z", ordering="linegraph", symbolic=True)
    with pytest.raises(qg.OutOfMemory):
        p.slice(1024, qg.FP64, 2)


def test_a_plan_that_fits_is_not_cut():
    p = qg.Plan(random_circuit_text(10, 8, 3), "Z", ordering="linegraph", symbolic=True)
    s = p.slice(p.workspace_bytes(qg.MIXED), qg.MIXED, 8)
    assert s.num_cuts == 0 and s.num_slices == 1


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CIRCUITS))
@pytest.mark.parametrize("div", [4, 64])
def test_sliced_value_equals_unsliced(ctx, name, div):
    p = qg.Plan(CIRCUITS[name](), "Z", ordering="linegraph", ctx=ctx)
    v64 = p.execute(qg.FP64)
    if name.startswith("rand"):
        assert abs(v64) > 1e-4   # a value the slices have to add up to (<Z> of a QFT'd basis state is 0)
    for prec, tol in ((qg.FP64, 1e-12), (qg.MIXED, 1e-6)):
        try:
            s = p.slice(p.workspace_bytes(prec) // div, prec, 8)
        except qg.OutOfMemory:
            continue
        assert s.num_cuts >= 1
        v = s.execute(prec)
        assert abs(v - v64) <= tol * max(1.0, abs(v64)), (name, prec, s.num_cuts)
        assert s.execute(prec) == v   # the batch of slices is kept and replayed
        # other leaf values: the same slicing, every slice step by step
        assert abs(s.execute(prec, leaves=p.leaf_values()) - v) <= tol * max(1.0, abs(v64))
