"""Placement of independent work across ranks (one process per GPU).

The RK4 path has no exchange step between independent meshes, so several
GPUs run replicas or disjoint sets of ensemble members with no collective on
the data path; the only communication is the timing reduction (maximum over
ranks) and the final aggregation of counts.

`shard` assigns items (ensemble members, weighted by their cell counts) to
ranks by longest-processing-time-first greedy balancing, deterministically,
so every rank computes the same assignment without communicating.
"""


def shard(weights, world, rank):
    """Indices of the items rank `rank` of `world` owns; every item goes to exactly
    one rank and the per-rank weight sums are balanced (LPT greedy, ties by index)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world / rank")
    order = sorted(range(len(weights)), key=lambda i: (-weights[i], i))
    load = [0] * world
    owner = [0] * len(weights)
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += weights[i]
    return [i for i in range(len(weights)) if owner[i] == rank]


def reduce_over_ranks(value, op="max", device=None):
    """`value` reduced over the default process group (identity without one).
    Works on the gloo (CPU) and nccl (device tensor) backends."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op={"max": dist.ReduceOp.MAX, "sum": dist.ReduceOp.SUM}[op])
    return float(t.item())
