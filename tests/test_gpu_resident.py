"""Resident evaluation (qt_batch_use_resident): one CTA per instance stays on
the GPU and serves evaluate() calls posted in pinned host memory.  Its values
must equal the launched paths' bit for bit, it must leave when idle and come
back on the next call, and every other use of the batch must stop it first."""
import time

import numpy as np
import pytest

import qtorch_gb300 as qg

pytestmark = pytest.mark.gpu


def term_angles(qasm):
    return [float(line.split(" ")[1]) for line in qasm.split("\n") if line.split(" ")[0] in ("Rx", "Rz")]


def qaoa_terms(ctx, p, nodes, degree, seed, every=1):
    dgf = qg.random_regular_graph(nodes, degree, seed=seed)
    start = [0.3] * p + [0.7] * p
    plans, edges = [], range(0, qg.qaoa_num_edges(dgf), every)
    for e in edges:
        plans.append(qg.Plan(*qg.qaoa_term_text(dgf, p, start, e), ordering="linegraph", ctx=ctx))

    def angles(beta, gamma):
        out = []
        for e in edges:
            out += term_angles(qg.qaoa_term_text(dgf, p, [beta] * p + [gamma] * p, e)[0])
        return np.array(out)
    return plans, angles


def mixed_batch(ctx, plans):
    b = qg.Batch(ctx)
    for pl in plans:
        b.add(pl)
    b.prepare(qg.MIXED)
    b.use_graph(True)
    return b


@pytest.mark.parametrize("p,nodes,degree,every", [(1, 30, 4, 1), (2, 24, 3, 2)])
def test_resident_values_equal_launched_ones(ctx, p, nodes, degree, every):
    plans, angles = qaoa_terms(ctx, p, nodes, degree, seed=11, every=every)
    res = mixed_batch(ctx, plans)
    ref = mixed_batch(ctx, plans)
    res.use_resident(1.0)
    for k in range(6):
        a = angles(0.2 + 0.15 * k, 1.1 - 0.1 * k)
        got = res.evaluate(a)
        want = ref.evaluate(a)
        assert np.array_equal(got, want), k
    # the FP64 form at the last point, within the mixed tolerance
    want64 = np.array([qg.Plan(*qg.qaoa_term_text(qg.random_regular_graph(nodes, degree, seed=11), p,
                                                  [0.2 + 0.75] * p + [1.1 - 0.5] * p, e),
                               ordering="linegraph", ctx=ctx).execute(qg.FP64)
                       for e in range(0, qg.qaoa_num_edges(qg.random_regular_graph(nodes, degree, seed=11)), every)])
    assert np.abs(got - want64).max() <= 1e-6
    res.use_resident(0)


def test_resident_engine_leaves_when_idle_and_comes_back(ctx):
    plans, angles = qaoa_terms(ctx, 1, 20, 3, seed=4)
    b = mixed_batch(ctx, plans)
    ref = mixed_batch(ctx, plans)
    b.use_resident(0.005)   # leaves after 5 ms without a request
    for k in range(3):
        a = angles(0.4 + 0.1 * k, 0.9)
        assert np.array_equal(b.evaluate(a), ref.evaluate(a))
        time.sleep(0.05)
    assert b.resident_starts == 3
    b.use_resident(10.0)
    for k in range(20):   # back to back: one engine serves them all
        b.evaluate(angles(0.1 * k, 0.5))
    assert b.resident_starts == 4
    b.use_resident(0)


def test_other_uses_stop_the_engine(ctx):
    plans, angles = qaoa_terms(ctx, 1, 20, 3, seed=6)
    b = mixed_batch(ctx, plans)
    b.use_resident(2.0)
    a1, a2 = angles(0.3, 0.8), angles(0.9, 0.2)
    v1 = b.evaluate(a1)
    b.set_rotations_device(a2)   # stops the engine, then the launched path
    b.run()
    v2 = b.fetch()
    assert not np.array_equal(v1, v2)
    assert np.array_equal(b.evaluate(a1), v1)   # the engine starts again
    b.set_launch_policy(stage_cap=0)           # a policy change stops it too
    assert np.array_equal(b.evaluate(a2), v2)
    b._release()                                 # freed while it runs


def test_resident_needs_a_mixed_batch_with_one_cta_per_instance(ctx):
    plans, _ = qaoa_terms(ctx, 1, 20, 3, seed=8)
    b = qg.Batch(ctx)
    for pl in plans:
        b.add(pl)
    b.prepare(qg.FP64)
    with pytest.raises(qg.QtError):
        b.use_resident(1.0)
    big = qg.Batch(ctx)
    for _ in range(20):   # 30 terms x 20 > 2 CTAs per SM
        for pl in plans:
            big.add(pl)
    big.prepare(qg.MIXED)
    with pytest.raises(qg.QtError):
        big.use_resident(1.0)


def test_resident_engine_with_more_angles_than_threads(ctx):
    """Requests normally post each angle in a 64-bit word tagged with the
    request's number, polled one word per thread.  A plan with more rotations
    than a CTA has threads takes the other request path (the request word,
    then the angles); both must equal the launched path bit for bit."""
    rng = np.random.default_rng(21)
    lines = ["2"]
    for _ in range(150):
        lines += [f"Rx {rng.uniform(0, 6.28):.6f} 0", f"Rx {rng.uniform(0, 6.28):.6f} 1", "CZ 0 1"]
    qasm = "\n".join(lines) + "\n"
    long_plan = qg.Plan(qasm, "Z T", ordering="linegraph", ctx=ctx)
    assert long_plan.num_rotations == 300
    plans, angles = qaoa_terms(ctx, 1, 20, 3, seed=8)
    for group in ([long_plan], plans):
        res = mixed_batch(ctx, group)
        ref = mixed_batch(ctx, group)
        res.use_resident(1.0)
        for k in range(4):
            if group is plans:
                a = angles(0.3 + 0.2 * k, 0.8 - 0.1 * k)
            else:
                a = rng.uniform(0, 6.28, 300)
            got = res.evaluate(a)
            assert np.array_equal(got, ref.evaluate(a)), k
            assert np.all(np.isfinite(got))
        assert res.resident_starts == 1
        res.use_resident(0)
