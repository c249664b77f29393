"""preProcess-style ordering search (src/preprocess.h:28-52): seeded
stochastic tries scored by largest intermediate, then complex MACs."""
import pytest

import qtorch_gb300 as qg
from conftest import load_golden

ANGLES = [0.3, 0.8, 0.6, 0.2]


def terms():
    dgf = qg.random_regular_graph(50, 3, seed=3)
    return [qg.qaoa_term_text(dgf, 2, ANGLES, e) for e in (0, 16, 29, 40)]


@pytest.mark.parametrize("which", range(4))
def test_search_is_never_worse_than_its_first_try(which):
    q, m = terms()[which]
    best = qg.Plan(q, m, ordering="search", seed=11, tries=30, symbolic=True)
    first = qg.Plan(q, m, ordering="stochastic", seed=11, symbolic=True)
    assert (best.peak_rank, best.flops) <= (first.peak_rank, first.flops)
    assert 11 <= best.chosen_seed < 11 + 30
    # the chosen seed reproduces the recorded sequence
    again = qg.Plan(q, m, ordering="stochastic", seed=best.chosen_seed, symbolic=True)
    assert again.sequence() == best.sequence()
    assert (again.peak_rank, again.flops) == (best.peak_rank, best.flops)


def test_search_keeps_the_best_of_its_tries():
    q, m = terms()[1]
    best = qg.Plan(q, m, ordering="search", seed=1, tries=20, symbolic=True)
    scores = [(p.peak_rank, p.flops) for p in
              (qg.Plan(q, m, ordering="stochastic", seed=s, symbolic=True) for s in range(1, 21))]
    assert (best.peak_rank, best.flops) == min(scores)


def test_search_stops_at_the_first_try_under_the_mac_limit():
    """The reference stops at the first sequence fast enough; max_macs is that bound."""
    q, m = terms()[1]
    scores = [qg.Plan(q, m, ordering="stochastic", seed=s, symbolic=True).flops for s in range(1, 21)]
    limit = sorted(scores)[len(scores) // 2]
    first_ok = next(i for i, f in enumerate(scores) if f <= limit)
    p = qg.Plan(q, m, ordering="search", seed=1, tries=20, max_macs=limit, symbolic=True)
    assert p.chosen_seed <= 1 + first_ok   # no try after the first one under the limit


def test_search_rejects_zero_tries():
    case = load_golden("networks.json")[0]
    with pytest.raises(qg.QtError):
        qg.Plan(case["qasm"], case["measure"], ordering="search", tries=0, symbolic=True)
