"""Multi-GPU: independent replicas, no collective on the data path.

The step does not shard (one grid's Jacobi sweeps would need a halo exchange per
sweep); batches of independent grids do. Grids are dealt to ranks by the
longest-processing-time-first rule on their cost (cells x sweeps), each rank steps
its own fs_batch, and ranks only meet at barriers around timed regions.
"""
from __future__ import annotations


def grid_cost(rows: int, cols: int, kd: int = 1, kp: int = 1) -> float:
    """Work of one step of a grid: interior cells x (3 diffusion + 2 pressure solves)."""
    return float((rows - 2) * (cols - 2)) * (3 * max(kd, 1) + 2 * max(kp, 1))


def partition_lpt(costs, world: int):
    """Deal items to `world` bins, largest first, each to the least-loaded bin (ties to
    the lowest rank). Returns a list of index lists, one per rank, each sorted."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    bins = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        bins[r].append(i)
        load[r] += costs[i]
    return [sorted(b) for b in bins]


def shard(shapes, world: int, rank: int, kd: int = 1, kp: int = 1):
    """Indices of the grids that `rank` steps."""
    costs = [grid_cost(r, c, kd, kp) for r, c in shapes]
    return partition_lpt(costs, world)[rank]
