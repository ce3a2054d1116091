"""Batched stepping of uneven grids vs independent single-grid handles and the oracle."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

SHAPES = [(34, 34), (66, 40), (130, 130), (5, 5), (200, 90), (3, 3), (258, 258), (17, 120)]


def _inputs(wl, shapes):
    return [wl.random_state(r, c, 1000 + k, vmax=0.03) for k, (r, c) in enumerate(shapes)]


# 240 small grids, about 60 per lane: a lane's diffusion pass covers ~180 fields, more
# than one launch's parameters carry (kMaxWideFields = 168), so it is split into two
# launches; its pressure passes (~60 fields) are one launch each
MANY = [(3 + (7 * k) % 29, 3 + (13 * k) % 37) for k in range(240)]


def _check_batch(fluid, wl, shapes, sweeps, tile_rows):
    kd, kp, steps = 30, 30, 4
    diff, visc, dt = 1e-3, 1e-3, 0.05
    ins = _inputs(wl, shapes)
    with fluid.Batch(shapes, diffuse_iterations=kd, pressure_iterations=kp, sweeps_per_pass=sweeps,
                     tile_rows=tile_rows, device=0) as b:
        for k, (d, u, v, ds, us, vs) in enumerate(ins):
            b.upload(k, d, u, v)
            b.upload_sources(k, ds, us, vs)
        b.step(diff, visc, dt, nsteps=steps)
        got = [b.download(k) for k in range(len(shapes))]
        st = b.stats()
        assert st["steps"] == steps and st["launches_per_step"] > 0
    for k, (d, u, v, ds, us, vs) in enumerate(ins):
        want = oracle.gpu_solve(d, ds, diff, u, v, us, vs, visc, dt, kd=kd, kp=kp, nsteps=steps)
        for g, o in zip(got[k], want):
            assert oracle.rel_linf(g, o) <= 1e-5, (k, shapes[k])
        with fluid.Solver(*shapes[k], diffuse_iterations=kd, pressure_iterations=kp, sweeps_per_pass=sweeps,
                          tile_rows=tile_rows, device=0) as s:
            s.upload(d, u, v)
            s.upload_sources(ds, us, vs)
            s.step(diff, visc, dt, nsteps=steps)
            single = s.download()
        for g, o in zip(got[k], single):
            assert oracle.rel_linf(g, o) <= 1e-6, (k, shapes[k])


@pytest.mark.parametrize("sweeps,tile_rows", [(8, 64), (5, 128), (30, 128)])
def test_batch_matches_single_handles_and_oracle(fluid, wl, sweeps, tile_rows):
    _check_batch(fluid, wl, SHAPES, sweeps, tile_rows)


@pytest.mark.parametrize("sweeps,tile_rows", [(8, 64), (5, 128)])
def test_batch_of_many_grids_matches_single_handles_and_oracle(fluid, wl, sweeps, tile_rows):
    _check_batch(fluid, wl, MANY, sweeps, tile_rows)
    with fluid.Batch(MANY, diffuse_iterations=30, pressure_iterations=30, sweeps_per_pass=sweeps,
                     tile_rows=tile_rows, device=0) as b:
        b.step(1e-3, 1e-3, 0.05)
        st = b.stats()
        # one launch per pass plus five advection / gradient launches in each of 4 lanes,
        # and more where diffusion passes were split
        assert st["launches_per_step"] > 4 * (st["passes_per_step"] + 5)


def test_batch_graph_equals_eager(fluid, wl):
    ins = _inputs(wl, SHAPES[:4])
    outs = []
    for use_graph in (0, 1):
        with fluid.Batch(SHAPES[:4], diffuse_iterations=10, pressure_iterations=10, use_graph=use_graph,
                         device=0) as b:
            for k, (d, u, v, ds, us, vs) in enumerate(ins):
                b.upload(k, d, u, v)
                b.upload_sources(k, ds, us, vs)
            b.step(1e-3, 1e-3, 0.05, nsteps=3)
            outs.append([b.download(k) for k in range(4)])
    for ga, gb in zip(*outs):
        for a, c in zip(ga, gb):
            assert oracle.rel_linf(a, c) <= 1e-6


def test_batch_argument_errors(fluid):
    with pytest.raises(fluid.FluidError):
        fluid.Batch([(2, 10)], device=0)
    with pytest.raises(fluid.FluidError):
        fluid.Batch([(10, 10)], warm_start=1, device=0)
    with fluid.Batch([(10, 10), (12, 12)], device=0) as b:
        with pytest.raises(ValueError):
            b.upload(0, *(np.zeros((12, 12), np.float32),) * 3)
