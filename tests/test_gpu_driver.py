"""Device-resident simulation driver: the reference's simulation::add_*_source and
simulation::update (src/simulation.cpp:44-64) on the handle's source grids, checked
against the oracle's restatement of the same driver around the GPU-semantics step."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _check(got, want):
    for g_, o in zip(got, want):
        assert oracle.rel_linf(g_, o) <= TOL


def test_add_sources_then_update(fluid, wl):
    n = 34
    d, u, v, _, _, _ = wl.random_state(n, n, 3, vmax=0.3)
    events = [(0, 0, 10, 12, 0.075, 0.0), (0, 1, 10, 12, 0.05, -0.02), (0, 0, 10, 12, 0.075, 0.0),
              (0, 1, 20, 5, -0.03, 0.04), (0, 0, 0, 7, 1.0, 0.0)]  # a boundary cell: the step ignores it
    with fluid.Solver(n, n, device=0) as s:
        s.upload(d, u, v)
        for _, kind, i, j, a, b in events:
            if kind == 0:
                s.add_density_source(i, j, a)
            else:
                s.add_velocity_source(i, j, a, b)
        s.update(1e-4, 1e-4, 0.1)
        want = oracle.simulation_run(d, u, v, events, 1, 1e-4, 1e-4, 0.1)
        _check(s.download(), want)
        # the sources were cleared: further updates run without them
        for _ in range(3):
            s.update(1e-4, 1e-4, 0.1)
        want = oracle.simulation_run(*want, [], 3, 1e-4, 1e-4, 0.1)
        _check(s.download(), want)


def test_scripted_drag_matches_the_driver_oracle(fluid, wl):
    n, steps = 66, 30
    d = np.zeros((n, n), np.float32)
    u = np.zeros_like(d)
    v = np.zeros_like(d)
    events = wl.drag_script(n, n, steps, seed=5)
    with fluid.Solver(n, n, device=0) as s:
        s.upload(d, u, v)
        s.run_script(events, steps, 1e-3, 1e-3, 0.05)
        got = s.download()
    want = oracle.simulation_run(d, u, v, events, steps, 1e-3, 1e-3, 0.05)
    _check(got, want)
    assert np.abs(got[0]).max() > 0


def test_script_in_two_calls_equals_one(fluid, wl):
    n = 34
    events = wl.drag_script(n, n, 10, seed=2)
    first = [e for e in events if e[0] < 4]
    second = [(e[0] - 4,) + tuple(e[1:]) for e in events if e[0] >= 4]
    z = np.zeros((n, n), np.float32)
    outs = []
    for parts in ([(events, 10)], [(first, 4), (second, 6)]):
        with fluid.Solver(n, n, device=0) as s:
            s.upload(z, z, z)
            for ev, k in parts:
                s.run_script(ev, k, 1e-3, 1e-3, 0.05)
            outs.append(s.download())
    # equal up to the order of the density splat's FP32 atomic additions (the reference
    # splats with atomics too, fluid_solver_gpu.cu:131-162)
    for a, b in zip(*outs):
        assert oracle.rel_linf(a, b) <= 1e-6


def test_script_rejects_bad_events(fluid):
    with fluid.Solver(34, 34, device=0) as s:
        for bad, steps in (([(1, 0, 5, 5, 1.0, 0.0), (0, 0, 5, 5, 1.0, 0.0)], 2),  # unsorted
                           ([(2, 0, 5, 5, 1.0, 0.0)], 2),                           # step out of range
                           ([(0, 0, 34, 5, 1.0, 0.0)], 1),                          # cell out of the grid
                           ([(0, 7, 5, 5, 1.0, 0.0)], 1)):                          # unknown kind
            with pytest.raises(fluid.FluidError) as e:
                s.run_script(bad, steps, 1e-3, 1e-3, 0.05)
            assert e.value.code == fluid.FS_ERR_ARG
        with pytest.raises(fluid.FluidError):
            s.add_density_source(-1, 3, 1.0)
