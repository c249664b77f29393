"""Write the inputs the CPU reference arm of bench.py replays.

    python tests/golden/make_bench_inputs.py

bench_qaoa_p1_30node.json holds the benchmark's graph (the seeded random
4-regular 30-vertex graph, .dgf text) and, for every edge term, the line-graph
(min-fill) ordering this build's planner chooses for it, as node-id pairs of
the reference's GetAllNodes() (ContractGivenSequence, src/ContractionTools.h:
392-411).  The reference arm reads this file instead of running the planner, so
its process never loads this build's library; the engine arm checks that its
own plans still record these sequences.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

OUT = os.path.join(HERE, "bench_qaoa_p1_30node.json")
NODES, DEGREE, P, GRAPH_SEED = 30, 4, 1, 1


def build():
    import qtorch_gb300 as qg
    dgf = qg.random_regular_graph(NODES, DEGREE, seed=GRAPH_SEED)
    seqs = []
    for e in range(qg.qaoa_num_edges(dgf)):
        q, m = qg.qaoa_term_text(dgf, P, [0.4, 1.1], e)
        plan = qg.Plan(q, m, ordering="linegraph", symbolic=True)
        seqs.append([x for pair in plan.sequence() for x in pair])
    return {"workload": "MaxCut QAOA p=1, seeded random 4-regular graph, 30 nodes, line-graph (min-fill) ordering",
            "nodes": NODES, "degree": DEGREE, "p": P, "graph_seed": GRAPH_SEED, "dgf": dgf, "sequences": seqs}


if __name__ == "__main__":
    data = build()
    with open(OUT, "w") as f:
        json.dump(data, f, indent=0)
    print(OUT, len(data["sequences"]), "terms", file=sys.stderr)
