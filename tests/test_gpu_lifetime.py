"""Object lifetimes across the C ABI: plans, batches, networks and servers keep
their context alive, so they may be freed after qt_ctx_destroy (the order a
garbage collector picks at interpreter exit)."""
import ctypes

import pytest

import qtorch_gb300 as qg

pytestmark = pytest.mark.gpu


def test_objects_outlive_their_context():
    lib = qg._capi.load()
    h = ctypes.c_void_p()
    assert lib.qt_ctx_create(0, None, ctypes.byref(h)) == 0
    ctx = h.value
    dgf = qg.random_regular_graph(20, 3, seed=4)
    q, m = qg.qaoa_term_text(dgf, 1, [0.4, 1.1], 0)
    plan = ctypes.c_void_p()
    assert lib.qt_plan_build(ctx, q.encode(), m.encode(), None, 1, 0, None, 0, ctypes.byref(plan)) == 0
    batch = ctypes.c_void_p()
    assert lib.qt_batch_create(ctx, ctypes.byref(batch)) == 0
    assert lib.qt_batch_add(batch, plan, None, None) == 0
    vals = (ctypes.c_double * 2)()
    assert lib.qt_batch_execute(batch, qg.MIXED, vals) == 0
    net = ctypes.c_void_p()
    assert lib.qt_network_create(ctx, q.encode(), m.encode(), None, ctypes.byref(net)) == 0
    # the owner lets go first; the objects still work and free cleanly afterwards
    assert lib.qt_ctx_destroy(ctx) == 0
    again = (ctypes.c_double * 2)()
    assert lib.qt_batch_execute(batch, qg.MIXED, again) == 0
    assert list(again) == list(vals)
    assert lib.qt_network_contract_linegraph(net) == 0
    assert lib.qt_batch_free(batch) == 0
    assert lib.qt_plan_free(plan) == 0
    assert lib.qt_network_free(net) == 0
