"""fs_solve_host on grids of at least 2^20 cells overlaps its host<->device copies with
the step: density and its source go up first and density diffuses while the velocity
grids are still uploading; the new density comes down while the velocity is projected.
The fields must be those of the device path (upload, step, download): velocity bit for
bit, density up to the order of the splat's FP32 atomic additions."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

CONFIGS = {
    "fixed": {},
    "warm": {"warm_start": 1},
    "residual": {"pressure_tolerance": 0.1, "pressure_max_iterations": 60000},
}
RATES = (1e-4, 2e-4, 0.1)


def _fields(wl, rows, cols, seed):
    d, u, v, ds, us, vs = wl.random_state(rows, cols, seed, vmax=0.3)
    return (d, u, v), (ds * 0.01, us * 0.01, vs * 0.01)


def _device_path(fluid, rows, cols, cfg, state, sources, steps):
    with fluid.Solver(rows, cols, device=0, **cfg) as s:
        s.upload(*state)
        s.upload_sources(*sources)
        for _ in range(steps):
            s.step(*RATES)
        return s.download()


def _same(got, want):
    assert oracle.rel_linf(got[0], want[0]) <= 1e-6
    assert np.array_equal(got[1], want[1]) and np.array_equal(got[2], want[2])


@pytest.mark.parametrize("rows,cols", [(1024, 1024), (1030, 1101)])
@pytest.mark.parametrize("name", list(CONFIGS))
@pytest.mark.parametrize("pinned", [False, True])
def test_overlapped_host_steps_equal_the_device_path(fluid, wl, rows, cols, name, pinned):
    cfg = CONFIGS[name]
    state, sources = _fields(wl, rows, cols, rows + cols)
    steps = 3
    want = _device_path(fluid, rows, cols, cfg, state, sources, steps)
    pins = []
    if pinned:
        pins = [fluid.PinnedArray(rows, cols) for _ in range(6)]
        for p, a in zip(pins, state + sources):
            p.array[...] = a
        d, u, v, ds, us, vs = (p.array for p in pins)
    else:
        d, u, v = (a.copy() for a in state)
        ds, us, vs = sources
    try:
        with fluid.Solver(rows, cols, device=0, **cfg) as s:
            for _ in range(steps):
                s.solve(d, ds, RATES[0], u, v, us, vs, RATES[1], RATES[2])
            st = s.stats()
            got = (d.copy(), u.copy(), v.copy())
    finally:
        for p in pins:
            p.free()
    _same(got, want)
    assert st["steps"] == steps and st["kernel_launches"] >= steps * st["launches_per_step"]


def test_host_and_device_steps_interleave(fluid, wl):
    """A host step, a device step on the sources it left, another host step: the same
    as three device steps."""
    rows = cols = 1024
    state, sources = _fields(wl, rows, cols, 7)
    want = _device_path(fluid, rows, cols, {}, state, sources, 3)
    d, u, v = (a.copy() for a in state)
    with fluid.Solver(rows, cols, device=0) as s:
        s.solve(d, sources[0], RATES[0], u, v, sources[1], sources[2], RATES[1], RATES[2])
        s.step(*RATES)
        d, u, v = s.download()
        s.solve(d, sources[0], RATES[0], u, v, sources[1], sources[2], RATES[1], RATES[2])
    _same((d, u, v), want)


def test_overlapped_host_step_matches_the_oracle(fluid, wl):
    """One host step on a 1024 x 1024 grid against the oracle's GPU-semantics step."""
    rows = cols = 1024
    state, sources = _fields(wl, rows, cols, 11)
    d, u, v = (a.copy() for a in state)
    with fluid.Solver(rows, cols, device=0, diffuse_iterations=20, pressure_iterations=20) as s:
        s.solve(d, sources[0], RATES[0], u, v, sources[1], sources[2], RATES[1], RATES[2])
    want = oracle.gpu_solve(*state[:1], sources[0], RATES[0], state[1], state[2], sources[1], sources[2], RATES[1],
                            RATES[2], kd=20, kp=20)
    for g, o in zip((d, u, v), want):
        assert oracle.rel_linf(g, o) <= 1e-5
