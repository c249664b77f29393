"""The MaxCut QAOA driver around the engine: the whole-circuit writer and the
final-cut decoding of src/maxcut.cpp:29-140, the COBYLA objective of
src/maxcut.cpp:144-225.  Host checks run without a GPU; the decoding and the
objective run on the GPU against the oracle port under the same orderings."""
import numpy as np
import pytest

import qtorch_gb300 as qg
from conftest import load_golden
from oracle import maxcut_decode, port, qaoa_terms


@pytest.mark.parametrize("g", load_golden("qaoa.json")[:3], ids=lambda g: g["dgf_name"])
def test_whole_circuit_text_is_the_reference_writer(g):
    pairs, nq = qaoa_terms.read_dgf(g["dgf"])
    for p in (1, 2):
        bg = [0.3 + 0.1 * i for i in range(p)] + [0.7 - 0.1 * i for i in range(p)]
        assert qg.qaoa_circuit_text(g["dgf"], p, bg) == qaoa_terms.term_qasm(pairs, nq, p, bg)


def test_measurement_leaves_are_last_in_leaf_order():
    dgf = qg.random_regular_graph(8, 3, seed=2)
    text = qg.qaoa_circuit_text(dgf, 1, [0.4, 0.9])
    nq = int(text.split("\n", 1)[0])
    pl = qg.Plan(text, "T " * nq, ordering="linegraph", symbolic=True)
    tail = pl.leaf_values()[-4 * nq:].reshape(nq, 4)
    assert np.array_equal(tail, np.tile([1, 0, 0, 1], (nq, 1)))
    other = qg.Plan(text, "0 1 " + "T " * (nq - 2), ordering="linegraph", symbolic=True)
    assert other.sequence() == pl.sequence()   # the ordering does not depend on the measurement string


def test_oracle_decoding_first_marginal_is_one_half():
    """Flipping every bit maps a cut to itself, so P(first qubit reads 0) = 1/2."""
    dgf = qg.random_regular_graph(6, 3, seed=1)
    text = qg.qaoa_circuit_text(dgf, 1, [0.4, 0.9])
    nq = int(text.split("\n", 1)[0])
    seq = qg.Plan(text, "T " * nq, ordering="linegraph", symbolic=True).sequence()
    bits, cut, prob, probs = maxcut_decode.final_string(dgf, 1, [0.4, 0.9], seq)
    assert abs(probs[0] - 0.5) < 1e-12
    assert 0 < prob <= 1 and len(bits) == nq and 0 <= cut <= len(qaoa_terms.read_dgf(dgf)[0])


@pytest.mark.gpu
@pytest.mark.parametrize("n,p", [(8, 1), (10, 1), (8, 2)])
def test_final_string_fp64_matches_oracle(ctx, n, p):
    dgf = qg.random_regular_graph(n, 3, seed=n + p)
    bg = [0.35] * p + [0.8] * p
    bits, cut, prob, marg = qg.maxcut_final_string(dgf, p, bg, qg.FP64, ctx=ctx, marginals=True)
    text = qg.qaoa_circuit_text(dgf, p, bg)
    seq = qg.Plan(text, "T " * n, ordering="linegraph", symbolic=True).sequence()
    # the oracle's decoding (maxcut_decode.final_string), query by query, so
    # that an exact tie takes the bit the engine's coin gave at that position
    current, answer = 1.0, []
    for i in range(n):
        meas = " ".join(("1" if answer[j] else "0") if j < i else ("0" if j == i else "T") for j in range(n))
        v, _ = port.replay_value(text, meas, seq)
        assert v.real == marg[i], i          # bit-exact under the same ordering
        nxt = v.real / current
        if nxt > 0.5:
            current *= nxt
            answer.append(0)
        elif nxt < 0.5:
            current *= 1.0 - nxt
            answer.append(1)
        else:
            answer.append(bits[i])
            current *= 0.5
    pairs, _ = qaoa_terms.read_dgf(dgf)
    assert answer == bits and current == prob
    assert cut == sum(1 for a, b in pairs if answer[a] != answer[b])


@pytest.mark.gpu
def test_final_string_mixed_tracks_fp64(ctx):
    dgf = qg.random_regular_graph(10, 3, seed=4)
    bg = [0.3, 0.75]
    b64, c64, p64, m64 = qg.maxcut_final_string(dgf, 1, bg, qg.FP64, ctx=ctx, marginals=True)
    bmx, cmx, pmx, mmx = qg.maxcut_final_string(dgf, 1, bg, qg.MIXED, ctx=ctx, marginals=True)
    i = 0
    while i < len(b64) and b64[i] == bmx[i]:
        assert abs(m64[i] - mmx[i]) <= 1e-6
        i += 1
    assert abs(m64[i if i < len(b64) else -1] - mmx[i if i < len(b64) else -1]) <= 1e-6


@pytest.mark.gpu
def test_objective_and_cobyla_search(ctx):
    pytest.importorskip("scipy")
    dgf = qg.random_regular_graph(12, 3, seed=5)
    mc = qg.MaxCutQAOA(dgf, 1, ctx=ctx)
    start = [qg.maxcut.START_BETA, qg.maxcut.START_GAMMA]
    f0 = mc.objective(start)
    # the objective is the reference's sum over the light-cone terms (FP64 oracle)
    want = sum(0.5 * (1.0 - port.replay_value(q, m, qg.Plan(q, m, ordering="linegraph", seed=k + 1,
                                                             symbolic=True).sequence())[0].real)
               for k, (_, q, m) in enumerate(qaoa_terms.all_terms(dgf, 1, start)))
    assert abs(f0 - want) <= 1e-5
    x, f = mc.optimize(maxiter=40)
    assert f >= f0 - 1e-9 and f <= qg.qaoa_num_edges(dgf)
    assert abs(mc.objective(x) - f) <= 1e-9
    bits, cut, prob = mc.final_string(x)
    assert len(bits) == 12 and 0 < prob <= 1
    mc.close()
