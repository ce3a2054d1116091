"""Replica partitioning across ranks (CPU; the world_size-2 path runs as gloo ranks)."""
import os
import socket

import numpy as np
import pytest


def _pkg():
    import __graft_entry__

    __graft_entry__.load_package()
    from fluid2d_gb300 import replicas, workloads

    return replicas, workloads


def test_lpt_covers_every_grid_once_and_balances():
    replicas, workloads = _pkg()

    sizes = workloads.batch_sizes(256, seed=4)
    shapes = [(n + 2, n + 2) for n in sizes]
    for world in (1, 2, 3, 4, 8):
        parts = [replicas.shard(shapes, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(shapes)))
        loads = [sum(replicas.grid_cost(*shapes[i]) for i in p) for p in parts]
        assert max(loads) <= min(loads) + max(replicas.grid_cost(*s) for s in shapes)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, shapes, q):
    import torch.distributed as dist

    import oracle

    R, W = _pkg()

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = R.shard(shapes, world, rank)
    # each rank steps its own grids (the oracle stands in for the GPU here) and the
    # per-grid density mass is gathered on every rank
    out = {}
    for i in mine:
        r, c = shapes[i]
        d, u, v, ds, us, vs = W.random_state(r, c, 100 + i, vmax=0.02)
        d1, _, _ = oracle.gpu_solve(d, ds, 1e-3, u, v, us, vs, 1e-3, 0.1, kd=4, kp=4, nsteps=2)
        out[i] = float(d1.sum(dtype=np.float64))
    gathered = [None] * world
    dist.all_gather_object(gathered, (mine, out))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, gathered))


def test_two_gloo_ranks_step_disjoint_shards():
    import torch.multiprocessing as mp

    shapes = [(10, 10), (34, 20), (18, 18), (50, 50), (7, 9), (26, 34)]
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, shapes, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import oracle

    _, W = _pkg()
    for _, gathered in results:
        seen = sorted(i for mine, _ in gathered for i in mine)
        assert seen == list(range(len(shapes)))
        masses = {i: m for _, out in gathered for i, m in out.items()}
        for i, (r, c) in enumerate(shapes):
            d, u, v, ds, us, vs = W.random_state(r, c, 100 + i, vmax=0.02)
            d1, _, _ = oracle.gpu_solve(d, ds, 1e-3, u, v, us, vs, 1e-3, 0.1, kd=4, kp=4, nsteps=2)
            assert masses[i] == float(d1.sum(dtype=np.float64))
