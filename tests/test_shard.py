"""Term sharding over ranks (qtorch_gb300.shard): longest-processing-time-first
partition by plan cost and the scalar gather, with two gloo ranks on CPU and a
fake evaluation (the partition and the exchange need no GPU)."""
import os
import socket

import numpy as np
import pytest

from qtorch_gb300 import shard


def test_lpt_partition_balances_and_covers_every_unit_once():
    rng = np.random.default_rng(3)
    costs = rng.pareto(1.5, 200) * 1e6 + 1e4
    for world in (1, 2, 3, 8):
        shares, loads = shard.lpt_partition(costs, world)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(costs)))
        assert np.allclose([costs[s].sum() for s in shares], loads)
        # Graham's bound for LPT: max load <= 4/3 OPT, OPT >= max(mean load, largest unit)
        opt_lb = max(costs.sum() / world, costs.max())
        assert loads.max() <= 4.0 / 3.0 * opt_lb + 1e-6


def test_lpt_puts_the_longest_units_first():
    # 10 -> rank 0, 8 -> rank 1, 3 -> rank 1 (8 < 10), 2 -> rank 0 (10 < 11), 1 -> rank 1 (11 < 12)
    shares, loads = shard.lpt_partition([1, 10, 3, 8, 2], 2)
    assert shares == [[1, 4], [0, 2, 3]]
    assert list(loads) == [12.0, 12.0]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, costs, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    from qtorch_gb300 import shard as sh
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seen = []

    def fake_evaluate(indices):
        seen.extend(indices)
        return [complex(i, -0.5 * i) for i in indices]

    vals = sh.evaluate_sharded(costs, fake_evaluate)
    out.put((rank, sorted(seen), vals.tolist()))
    dist.destroy_process_group()


@pytest.mark.parametrize("n_units", [7, 1])
def test_two_ranks_evaluate_their_shares_and_gather_every_value(n_units):
    import multiprocessing as mp
    costs = list(np.random.default_rng(n_units).uniform(1, 100, n_units))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    shares, _ = shard.lpt_partition(costs, 2)
    want = [complex(i, -0.5 * i) for i in range(n_units)]
    for rank, seen, vals in res:
        assert seen == shares[rank]        # each rank evaluated exactly its share
        assert vals == want                # and holds every unit's value in order
