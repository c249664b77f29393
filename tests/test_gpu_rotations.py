"""Rotation leaves built on the device from angles (qt_batch_set_rotations_device).

Moving a batch of QAOA terms to a new (gamma, beta) point sends only the
angles; the interpreter rebuilds the Rx/Rz gate tensors before contracting
(same narrowing of the angle to float; FP32 trigonometry, so entries differ
from the host-built complex64 leaves by a few ulp).  The result must agree with
the host-built leaves to a few 1e-7 and with the FP64 form at the new point
within the mixed tolerance."""
import numpy as np
import pytest

import qtorch_gb300 as qg

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


def term_angles(qasm):
    out = []
    for line in qasm.split("\n"):
        t = line.split(" ")
        if t[0] in ("Rx", "Rz"):
            out.append(float(t[1]))
    return out


@pytest.mark.parametrize("p,nodes,degree", [(1, 30, 4), (2, 22, 3)])
def test_device_rotations_match_host_rotations(ctx, p, nodes, degree):
    dgf = qg.random_regular_graph(nodes, degree, seed=11)
    start = [0.3] * p + [0.7] * p
    moved = [0.9] * p + [0.25] * p
    n = qg.qaoa_num_edges(dgf)
    plans, new_terms = [], []
    for e in range(n):
        q, m = qg.qaoa_term_text(dgf, p, start, e)
        plans.append(qg.Plan(q, m, ordering="linegraph", ctx=ctx))
        new_terms.append(qg.qaoa_term_text(dgf, p, moved, e))
    angles = np.concatenate([term_angles(q) for q, _ in new_terms])
    b = qg.Batch(ctx)
    for pl in plans:
        b.add(pl)
    b.prepare(qg.MIXED)
    b.set_rotations_device(angles)
    b.run()
    dev = b.fetch()
    assert b.h2d_bytes == 8 * len(angles)
    b.set_rotations(angles)   # back to host-built leaves
    b.upload()
    b.run()
    host = b.fetch()
    assert np.abs(dev - host).max() <= 5e-7
    want = np.array([qg.Plan(q, m, ordering="linegraph", ctx=ctx).execute(qg.FP64) for q, m in new_terms])
    assert np.abs(dev - want).max() <= MIXED_TOL


def test_device_rotations_need_a_mixed_batch(ctx):
    dgf = qg.random_regular_graph(20, 3, seed=2)
    q, m = qg.qaoa_term_text(dgf, 1, [0.3, 0.7], 0)
    pl = qg.Plan(q, m, ordering="linegraph", ctx=ctx)
    b = qg.Batch(ctx)
    b.add(pl)
    b.prepare(qg.FP64)
    with pytest.raises(qg.QtError):
        b.set_rotations_device(np.array(term_angles(q)))


def test_evaluate_is_set_run_fetch(ctx):
    dgf = qg.random_regular_graph(30, 4, seed=11)
    plans, angles = [], []
    for e in range(qg.qaoa_num_edges(dgf)):
        q, m = qg.qaoa_term_text(dgf, 1, [0.3, 0.7], e)
        plans.append(qg.Plan(q, m, ordering="linegraph", ctx=ctx))
        angles += term_angles(qg.qaoa_term_text(dgf, 1, [1.2, 0.4], e)[0])
    b = qg.Batch(ctx)
    for pl in plans:
        b.add(pl)
    b.prepare(qg.MIXED)
    b.use_graph(True)
    one = b.evaluate(np.array(angles))
    b.set_rotations_device(np.array(angles))
    b.run()
    assert np.array_equal(one, b.fetch())
    assert np.array_equal(b.evaluate(), one)   # no angles: the current leaves again
    # later calls replay one captured graph (angles in, launch, values out)
    other = np.array(angles) * 0.5
    two = b.evaluate(other)
    b.set_rotations_device(other)
    b.run()
    assert np.array_equal(two, b.fetch())
    assert not np.array_equal(two, one)
    assert np.array_equal(b.evaluate(np.array(angles)), one)
