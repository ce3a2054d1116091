"""The autotuner picks a valid tiling, caches it, and the tuned solver keeps parity."""
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_autotune_picks_caches_and_keeps_parity(fluid, wl, tmp_path):
    w = wl.small_sources(96, seed=21, kd=20, kp=20)
    cache = tmp_path / "tune.txt"
    kw = dict(diffuse_iterations=20, pressure_iterations=20, device=0)
    t1 = fluid.autotune(w.rows, w.cols, w.diffusion, w.viscosity, w.dt, steps=2, cache_path=cache, **kw)
    assert t1["tile_rows"] in (64, 128) and 4 <= t1["sweeps_per_pass"] <= 16 and t1["ms_per_step"] > 0
    lines = cache.read_text().strip().splitlines()
    assert len(lines) == 1 and lines[0].split()[1:3] == [str(t1["tile_rows"]), str(t1["sweeps_per_pass"])]
    t2 = fluid.autotune(w.rows, w.cols, w.diffusion, w.viscosity, w.dt, steps=2, cache_path=cache, **kw)
    assert (t2["tile_rows"], t2["sweeps_per_pass"]) == (t1["tile_rows"], t1["sweeps_per_pass"])
    assert len(cache.read_text().strip().splitlines()) == 1  # served from the cache
    d, u, v = w.state()
    with fluid.Solver(w.rows, w.cols, tile_rows=t1["tile_rows"], sweeps_per_pass=t1["sweeps_per_pass"], **kw) as s:
        for _ in range(3):
            s.solve(d, w.ds, w.diffusion, u, v, w.us, w.vs, w.viscosity, w.dt)
    want = oracle.gpu_solve(*w.state()[:1], w.ds, w.diffusion, *w.state()[1:], w.us, w.vs, w.viscosity, w.dt,
                            kd=20, kp=20, nsteps=3)
    for g, o in zip((d, u, v), want):
        assert oracle.rel_linf(g, o) <= 1e-5
