"""The autotuner picks a valid tiling, caches it, and the tuned solver keeps parity."""
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_autotune_picks_caches_and_keeps_parity(fluid, wl, tmp_path):
    w = wl.small_sources(96, seed=21, kd=20, kp=20)
    cache = tmp_path / "tune.txt"
    kw = dict(diffuse_iterations=20, pressure_iterations=20, device=0)
    t1 = fluid.autotune(w.rows, w.cols, w.diffusion, w.viscosity, w.dt, steps=2, cache_path=cache, **kw)
    assert t1["tile_rows"] in (64, 128) and 2 <= t1["sweeps_per_pass"] <= 16 and t1["ms_per_step"] > 0
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


def test_batch_autotune_picks_caches_and_keeps_parity(fluid, wl, tmp_path):
    shapes = [(34, 34), (66, 40), (130, 130), (5, 5), (17, 120)]
    ins = [wl.random_state(r, c, 300 + k, vmax=0.03) for k, (r, c) in enumerate(shapes)]
    cache = tmp_path / "tune_batch.txt"
    kw = dict(diffuse_iterations=20, pressure_iterations=30, device=0)
    t1 = fluid.autotune_batch(shapes, 1e-3, 1e-3, 0.05, steps=1, cache_path=cache, **kw)
    # depths 2..16 and 15, 10, 8 (30 pressure sweeps in two, three or four passes)
    assert t1["tile_rows"] in (64, 128) and 2 <= t1["sweeps_per_pass"] <= 16 and t1["ms_per_step"] > 0
    lines = cache.read_text().strip().splitlines()
    assert len(lines) == 1 and lines[0].split()[1:3] == [str(t1["tile_rows"]), str(t1["sweeps_per_pass"])]
    t2 = fluid.autotune_batch(shapes, 1e-3, 1e-3, 0.05, steps=1, cache_path=cache, **kw)
    assert (t2["tile_rows"], t2["sweeps_per_pass"]) == (t1["tile_rows"], t1["sweeps_per_pass"])
    assert len(cache.read_text().strip().splitlines()) == 1  # served from the cache
    with fluid.Batch(shapes, tile_rows=t1["tile_rows"], sweeps_per_pass=t1["sweeps_per_pass"], **kw) as b:
        for k, (d, u, v, ds, us, vs) in enumerate(ins):
            b.upload(k, d, u, v)
            b.upload_sources(k, ds, us, vs)
        b.step(1e-3, 1e-3, 0.05, nsteps=2)
        got = [b.download(k) for k in range(len(shapes))]
    for k, (d, u, v, ds, us, vs) in enumerate(ins):
        want = oracle.gpu_solve(d, ds, 1e-3, u, v, us, vs, 1e-3, 0.05, kd=20, kp=30, nsteps=2)
        for g, o in zip(got[k], want):
            assert oracle.rel_linf(g, o) <= 1e-5, shapes[k]


def test_default_depth_rule(fluid):
    """sweeps_per_pass = 0: depth 8 on large grids and residual-target solves; the fewest
    passes on launch-bound small grids; an explicit depth is kept."""
    def depth(n, **kw):
        with fluid.Solver(n, n, device=0, **kw) as s:
            return s.stats()["sweeps_per_pass"]

    assert depth(130) == 20                                  # 15/20 sweeps: one pass per solve
    assert depth(130, diffuse_iterations=40, pressure_iterations=40) == 20  # two passes of 20
    assert depth(2050) == 8
    assert depth(130, pressure_tolerance=1e-3, pressure_max_iterations=100) == 8
    assert depth(130, sweeps_per_pass=5) == 5
