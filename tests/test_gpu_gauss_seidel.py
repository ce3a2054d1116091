"""The Gauss-Seidel method (FS_METHOD_GAUSS_SEIDEL): the reference's host solver
fluid_solver_cpu (src/fluid_solver_cpu.cpp:6-215) reproduced on the GPU, bit for bit.

Checked against the golden fixtures written by the compiled reference itself, and against
the oracle's restatement of the host solver (pinned bit for bit to the compiled host
solver) on seeded workloads: sizes from 3 to the largest one-CTA grid (234 on a GB300),
the tiled form above it (235, 301, the reference app's 800 and the benchmark's 2050),
iteration counts other than the reference's 20/20, and both splat paths."""
import pathlib

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
CASES = sorted(p.name[len("ref_cpu_"):-4] for p in GOLDEN.glob("ref_cpu_*.npz"))


def _gs(fluid, n, **kw):
    return fluid.FluidSolverGaussSeidel(n, device=0, **kw)


@pytest.mark.parametrize("case", CASES)
def test_bit_exact_vs_compiled_reference_fixture(fluid, case):
    z = np.load(GOLDEN / f"ref_cpu_{case}.npz")
    diff, visc, dt = (float(x) for x in z["params"])
    d, u, v = z["d"].copy(), z["u"].copy(), z["v"].copy()
    with _gs(fluid, d.shape[0]) as s:
        for _ in range(int(z["steps"])):
            s.solve(d, z["ds"], diff, u, v, z["us"], z["vs"], visc, dt)
    for got, key in ((d, "out_d"), (u, "out_u"), (v, "out_v")):
        np.testing.assert_array_equal(got, z[key])


def test_reference_cpu_workload_100_steps(fluid, wl):
    """130 x 130 (interior 128), seeded density blobs and velocity impulses, dt 0.1,
    diffusion = viscosity = 1e-4, 20/20 sweeps, 100 steps: every step bit-identical."""
    w = wl.small_sources(128, seed=11)
    d, u, v = w.d.copy(), w.u.copy(), w.v.copy()
    od, ou, ov = w.d.copy(), w.u.copy(), w.v.copy()
    with _gs(fluid, w.rows) as s:
        for step in range(100):
            s.solve(d, w.ds, w.diffusion, u, v, w.us, w.vs, w.viscosity, w.dt)
            od, ou, ov = oracle.cpu_solve(od, w.ds, w.diffusion, ou, ov, w.us, w.vs, w.viscosity, w.dt)
            for g_, o in ((d, od), (u, ou), (v, ov)):
                assert np.array_equal(g_, o), f"step {step}"
    assert np.abs(d).max() > 0


@pytest.mark.parametrize("n,kd,kp", [(3, 20, 20), (4, 20, 20), (17, 1, 1), (40, 0, 3), (64, 7, 33), (66, 20, 0)])
def test_sizes_and_iteration_counts(fluid, wl, n, kd, kp):
    d, u, v, ds, us, vs = wl.random_state(n, n, n + kd, vmax=0.5)
    args = (0.05, 0.02, 0.1)
    with _gs(fluid, n, diffuse_iterations=kd, pressure_iterations=kp) as s:
        s.upload(d, u, v)
        s.upload_sources(ds, us, vs)
        s.step(args[0], args[1], args[2], 3)
        gd, gu, gv = s.download()
    od, ou, ov = oracle.cpu_solve(d, ds, args[0], u, v, us, vs, args[1], args[2], kd=kd, kp=kp, nsteps=3)
    for g_, o in ((gd, od), (gu, ou), (gv, ov)):
        np.testing.assert_array_equal(g_, o)


ONE_CTA_MAX = 234  # the largest grid whose field fits one GB300 SM's shared memory


def _vs_oracle(fluid, n, d, u, v, ds, us, vs, diff, visc, dt, steps, kd=20, kp=20):
    with _gs(fluid, n, diffuse_iterations=kd, pressure_iterations=kp) as s:
        s.upload(d, u, v)
        s.upload_sources(ds, us, vs)
        s.step(diff, visc, dt, steps)
        got = s.download()
    want = oracle.cpu_solve(d, ds, diff, u, v, us, vs, visc, dt, kd=kd, kp=kp, nsteps=steps)
    for g_, o in zip(got, want):
        np.testing.assert_array_equal(g_, o)


@pytest.mark.parametrize("n", [ONE_CTA_MAX, ONE_CTA_MAX + 1])
def test_either_side_of_the_one_cta_limit(fluid, wl, n):
    w = wl.small_sources(n - 2, seed=5)
    _vs_oracle(fluid, n, w.d, w.u, w.v, w.ds, w.us, w.vs, w.diffusion, w.viscosity, w.dt, 4)


@pytest.mark.parametrize("n,kd,kp,vmax", [(301, 20, 20, 0.5), (301, 7, 33, 0.5), (257, 0, 5, 0.5), (300, 20, 20, 2.0)])
def test_tiled_sizes_counts_and_splat_paths(fluid, wl, n, kd, kp, vmax):
    """vmax 2.0 moves sources ~60 cells: the in-order splat; 0.5 the gathering one."""
    d, u, v, ds, us, vs = wl.random_state(n, n, n + kd, vmax=vmax)
    _vs_oracle(fluid, n, d, u, v, ds, us, vs, 0.05, 0.02, 0.1, 3, kd, kp)


def test_reference_app_size(fluid, wl):
    """800 x 800, the reference app's grid (src/app.cpp:30-31), vortex field, 20/20, 5 steps."""
    w = wl.vortex_field(798, seed=6, kd=20, kp=20, vortices=24, rmin=8, rmax=30)
    _vs_oracle(fluid, w.rows, w.d, w.u, w.v, w.ds, w.us, w.vs, w.diffusion, w.viscosity, w.dt, 5)


def test_benchmark_size(fluid, wl):
    """2050 x 2050, the benchmark's vortex field at the host solver's 20/20, 2 steps."""
    w = wl.vortex_field(2048, seed=2, kd=20, kp=20)
    _vs_oracle(fluid, w.rows, w.d, w.u, w.v, w.ds, w.us, w.vs, w.diffusion, w.viscosity, w.dt, 2)


def test_tiled_barrier_timeout(fluid, wl):
    """A tiled solve whose grid-barrier waits run out after one poll reports
    FS_ERR_TIMEOUT; with the default bound restored the same handle steps exactly."""
    n = 301
    d, u, v, ds, us, vs = wl.random_state(n, n, 3, vmax=0.5)
    with _gs(fluid, n) as s:
        s.upload(d, u, v)
        s.upload_sources(ds, us, vs)
        s.set_barrier_poll_limit(1)
        with pytest.raises(fluid.FluidError) as e:
            s.step(0.05, 0.02, 0.1)
        assert e.value.code == fluid.FS_ERR_TIMEOUT
        s.set_barrier_poll_limit(0)
        s.upload(d, u, v)
        s.step(0.05, 0.02, 0.1)
        got = s.download()
    want = oracle.cpu_solve(d, ds, 0.05, u, v, us, vs, 0.02, 0.1, nsteps=1)
    for g_, o in zip(got, want):
        np.testing.assert_array_equal(g_, o)


def test_rejections(fluid):
    n = fluid.gauss_seidel_max_size()
    bad = [dict(rows=n + 1, cols=n + 1), dict(rows=34, cols=40), dict(rows=34, cols=34, warm_start=1),
           dict(rows=34, cols=34, pressure_tolerance=1e-3, pressure_max_iterations=100)]
    for kw in bad:
        rows, cols = kw.pop("rows"), kw.pop("cols")
        with pytest.raises(fluid.FluidError) as e:
            fluid.Solver(rows, cols, method=fluid.FS_METHOD_GAUSS_SEIDEL, device=0, **kw)
        assert e.value.code == fluid.FS_ERR_ARG
    with _gs(fluid, 34) as s:
        with pytest.raises(fluid.FluidError) as e:
            s.stage(0, 1e-4, 0.1)
        assert e.value.code == fluid.FS_ERR_STATE
