"""Orderings for requests of any size (no reference counterpart): the
size-greedy merge order and the automatic choice between it and the line
graph's min-fill walk.  Both are recorded as node-id sequences, so what they
produce replays through the sequence ordering and through the oracle."""
import time

import pytest

import qtorch_gb300 as qg
from qtorch_gb300.circuits import qft_measure_text, qft_text, random_circuit_text
from oracle import port


def small_cases():
    dgf = qg.random_regular_graph(20, 3, seed=9)
    q, m = qg.qaoa_term_text(dgf, 2, [0.3, 0.8, 0.6, 0.2], 4)
    return {"rand10x8": (random_circuit_text(10, 8, 3), "Z"), "qft7": (qft_text(7, 2), qft_measure_text(7)),
            "qaoa_p2": (q, m)}


@pytest.mark.parametrize("name", sorted(small_cases()))
@pytest.mark.parametrize("ordering", ["greedy", "auto"])
def test_recorded_sequence_replays(name, ordering):
    q, m = small_cases()[name]
    p = qg.Plan(q, m, ordering=ordering, seed=3, symbolic=True)
    again = qg.Plan(q, m, ordering="sequence", sequence=p.sequence(), symbolic=True)
    assert again.sequence() == p.sequence()
    assert (again.peak_rank, again.flops) == (p.peak_rank, p.flops)
    # the oracle contracts the same network in the recorded order to the value of
    # the line-graph ordering (both exact up to rounding in complex128)
    v, flops = port.replay_value(q, m, p.sequence())
    assert flops == p.flops
    lg = qg.Plan(q, m, ordering="linegraph", symbolic=True)
    w, _ = port.replay_value(q, m, lg.sequence())
    assert abs(v - w) <= 1e-12 * max(1.0, abs(w))


@pytest.mark.parametrize("name", sorted(small_cases()))
def test_greedy_is_deterministic_per_seed(name):
    q, m = small_cases()[name]
    a = qg.Plan(q, m, ordering="greedy", seed=5, symbolic=True)
    b = qg.Plan(q, m, ordering="greedy", seed=5, symbolic=True)
    assert a.sequence() == b.sequence()


@pytest.mark.parametrize("circuit", [(16, 12), (20, 8), (20, 14), (30, 8)])
def test_auto_keeps_the_smaller_intermediate(circuit):
    n, d = circuit
    q = random_circuit_text(n, d, 7)
    auto = qg.Plan(q, "Z", ordering="auto", symbolic=True)
    lg = qg.Plan(q, "Z", ordering="linegraph", symbolic=True)
    gr = qg.Plan(q, "Z", ordering="greedy", symbolic=True)
    assert auto.peak_rank <= lg.peak_rank
    assert auto.peak_rank <= gr.peak_rank + 1


@pytest.mark.parametrize("text", [
    lambda: random_circuit_text(20, 14, 7), lambda: random_circuit_text(24, 12, 7),
    lambda: random_circuit_text(30, 8, 7), lambda: qft_text(16, 3), lambda: qft_text(20, 3)])
def test_large_circuits_plan_in_well_under_a_second_each(text):
    """Planning of 20-30-qubit circuits: no host array is made for the
    intermediates of a symbolic network, so a plan takes milliseconds however
    large its tensors."""
    q = text()
    t = time.perf_counter()
    p = qg.Plan(q, "Z", ordering="auto", symbolic=True)
    assert time.perf_counter() - t < 3.0
    assert p.peak_rank >= 7


def test_beyond_the_engine_rank_limit_is_an_invalid_input():
    """An intermediate of more than 24 wires (4^24 elements) is beyond any
    device: planning stops with InvalidFunctionInput."""
    with pytest.raises(qg.InvalidFunctionInput):
        qg.Plan(random_circuit_text(30, 20, 7), "Z", ordering="auto", symbolic=True)


def test_slicing_beyond_one_chunk_of_slices():
    """More than 4096 slices (7+ cut wires) run in chunks; the slicing itself is
    host logic."""
    p = qg.Plan(qft_text(8, 2), qft_measure_text(8), ordering="linegraph", symbolic=True)
    s = p.slice(p.workspace_bytes(qg.MIXED) // 20, qg.MIXED, 16)
    assert s.num_cuts >= 7
    assert s.workspace_bytes(qg.MIXED) <= p.workspace_bytes(qg.MIXED) // 20


@pytest.mark.parametrize("case", [("rand26x12", 3.0e12), ("rand14x20", 2.0e11), ("qft16", 1.2e12)])
def test_greedy_search_keeps_heavy_circuits_cheap(case):
    """The automatic ordering runs 4096 seeded greedy walks (spread over host
    threads; the choice does not depend on their number): the serving mix's
    heavy circuits plan to far fewer complex MACs than with 32 walks (4.7e12,
    2.2e11 and 1.8e12), deterministically."""
    name, bound = case
    if name == "rand26x12":
        q, m = random_circuit_text(26, 12, 24), "Z"
    elif name == "rand14x20":
        q, m = random_circuit_text(14, 20, 14), "Z"
    else:
        q, m = qft_text(16, 7), qft_measure_text(16)
    a = qg.Plan(q, m, ordering="auto", symbolic=True)
    b = qg.Plan(q, m, ordering="auto", symbolic=True)
    assert a.sequence() == b.sequence()
    assert a.flops <= bound
    assert a.peak_rank <= 15
