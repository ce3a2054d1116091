"""Bounded waits on the GPU (GPU required).

The residual-driven pressure solve is one cooperative launch whose CTAs meet at a
grid-wide barrier after every pass. Each wait there is bounded: after a poll limit the
CTA flags an error and every later barrier returns at once, so the kernel always ends.
Here the limit is set to one poll, which makes the waits run out on purpose (every CTA
is co-resident, so nothing is left waiting), and the test checks that the host sees
FS_ERR_TIMEOUT and that the same handle then steps like the oracle with the default
limit restored. No GPU fault is involved: the kernel returns normally with an error
status.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
TOL = 1e-5


def test_grid_barrier_timeout_is_reported_and_the_handle_recovers(fluid, wl):
    w = wl.small_sources(128, seed=17)  # 130 x 130: 6 tiles, so 6 CTAs meet at each barrier
    tol = 2e-2
    with fluid.Solver(w.rows, w.cols, pressure_tolerance=tol, pressure_max_iterations=20000, sweeps_per_pass=8,
                      device=0) as s:
        s.upload(*w.state())
        s.upload_sources(*w.sources())
        s.set_barrier_poll_limit(1)
        with pytest.raises(fluid.FluidError) as e:
            s.step(w.diffusion, w.viscosity, w.dt)
        assert e.value.code == fluid.FS_ERR_TIMEOUT
        # the same handle, default limit: a full step from the original state
        s.set_barrier_poll_limit(0)
        s.upload(*w.state())
        s.step(w.diffusion, w.viscosity, w.dt)
        d, u, v = s.download()
        st = s.stats()
    k1, k2 = st["pressure_iterations_last"]
    assert k1 > 0 and k2 > 0 and max(st["pressure_residual_last"]) <= tol
    od, ou, ov = w.state()
    od, ou, ov = oracle.gpu_solve_ex(od, w.ds, w.diffusion, ou, ov, w.us, w.vs, w.viscosity, w.dt, 15, k1, k2)
    for g, o in ((d, od), (u, ou), (v, ov)):
        assert oracle.rel_linf(g, o) <= TOL
