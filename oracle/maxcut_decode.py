"""Restatement of qTorch's final-cut decoding — TEST INFRASTRUCTURE ONLY.

Follows maxcutGetFinalString (src/maxcut.cpp:29-140): the whole circuit
(outputInitialPlusStateToFile + applyU_CsThenU_Bs over every graph edge), then
qubit by qubit the probability that the qubit reads 0 given the bits chosen
so far -- measurement '1'/'0' on the decided qubits, '0' on the current one,
'T' on the rest -- contracted by the oracle port under a recorded ordering.
The likelier bit is kept and the running probability multiplied by its
probability; an exact tie takes the next bit of ``coin`` (the reference calls
rand()).
"""
from . import port
from . import qaoa_terms


def circuit_text(dgf_text, p, betas_gammas):
    pairs, nq = qaoa_terms.read_dgf(dgf_text)
    return qaoa_terms.term_qasm(pairs, nq, p, betas_gammas), pairs, nq


def final_string(dgf_text, p, betas_gammas, sequence, coin=lambda: 0):
    """(bits, cut edges, probability, per-qubit probabilities) under the node-id
    pair sequence ``sequence`` (the same for every measurement string)."""
    qasm, pairs, nq = circuit_text(dgf_text, p, betas_gammas)
    answer, current, probs = [], 1.0, []
    for i in range(nq):
        meas = " ".join(("1" if answer[j] else "0") if j < i else ("0" if j == i else "T") for j in range(nq))
        v, _ = port.replay_value(qasm, meas, sequence)
        nxt = v.real / current
        probs.append(v.real)
        if nxt > 0.5:
            current *= nxt
            answer.append(0)
        elif nxt < 0.5:
            current *= 1.0 - nxt
            answer.append(1)
        else:
            answer.append(coin() & 1)
            current *= 0.5
    cut = sum(1 for a, b in pairs if answer[a] != answer[b])
    return answer, cut, current, probs
