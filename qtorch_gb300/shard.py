"""Independent terms over several GPUs: one process per GPU, no collective on
the data path.

QAOA edge terms, parameter points and requests are independent contractions.
The reference runs such units concurrently only as the two partitions of its
stochastic ordering (src/ContractionTools.h:359-368).  Here a list of units is
split over the ranks of a torch.distributed group longest-processing-time
first by plan cost -- each unit to the rank with the least work so far -- each
rank evaluates its share on its own GPU (one grouped launch), and the scalar
results are gathered back into the caller's order on every rank: the only
exchange is 16 bytes per unit.
"""
import numpy as np

# A grouped-interpreter level costs about as much as a few thousand complex
# MACs of one CTA (1.5 us per dependent level against ~2e9 MAC/s per CTA).
LEVEL_COST_MACS = 3000


def plan_cost(plan):
    """Estimated cost of one unit: its complex MACs plus a per-level latency term."""
    levels = int(plan.step_info()[:, 0].max()) + 1 if plan.num_steps else 0
    return float(plan.flops) + LEVEL_COST_MACS * levels


def lpt_partition(costs, world):
    """Longest processing time first: units in decreasing cost, each to the
    rank whose load is smallest (ties to the lowest rank).  Returns, per rank,
    the unit indices in increasing order; the largest load is at most 4/3 of
    the optimum plus nothing worse than one unit."""
    costs = np.asarray(costs, dtype=np.float64)
    loads = np.zeros(world)
    shares = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = int(np.argmin(loads))
        shares[r].append(i)
        loads[r] += costs[i]
    return [sorted(s) for s in shares], loads


def gather_values(local_indices, local_values, n_units, group=None):
    """All ranks' (index, complex value) pairs into one complex128 vector of n_units
    in the caller's order, on every rank (one all_gather of a padded tensor)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    counts = [0] * world
    dist.all_gather_object(counts, len(local_indices), group=group)
    width = max(max(counts), 1)
    buf = torch.zeros((width, 3), dtype=torch.float64)
    for j, (i, v) in enumerate(zip(local_indices, local_values)):
        buf[j, 0], buf[j, 1], buf[j, 2] = float(i), v.real, v.imag
    parts = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf, group=group)
    out = np.full(n_units, np.nan + 1j * np.nan, dtype=np.complex128)
    for r, part in enumerate(parts):
        for j in range(counts[r]):
            out[int(part[j, 0])] = complex(part[j, 1].item(), part[j, 2].item())
    return out


def evaluate_sharded(costs, evaluate, group=None):
    """Split units of the given costs over the group's ranks (LPT), call
    evaluate(indices) -> complex values on this rank's share, and return every
    unit's value on every rank."""
    import torch.distributed as dist
    world, rank = dist.get_world_size(group), dist.get_rank(group)
    shares, _ = lpt_partition(costs, world)
    mine = shares[rank]
    vals = list(evaluate(mine)) if mine else []
    return gather_values(mine, vals, len(costs), group)


def evaluate_plans_sharded(plans, precision, ctx, group=None):
    """The units are plans (each with its own leaves): this rank's share runs
    as one batch on ctx's device."""
    from . import Batch

    def run(indices):
        b = Batch(ctx)
        for i in indices:
            b.add(plans[i])
        vals = b.execute(precision)
        b._release()
        return vals
    return evaluate_sharded([plan_cost(p) for p in plans], run, group)
