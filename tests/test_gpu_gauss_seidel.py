"""The Gauss-Seidel method (FS_METHOD_GAUSS_SEIDEL): the reference's host solver
fluid_solver_cpu (src/fluid_solver_cpu.cpp:6-215) reproduced on the GPU, bit for bit.

Checked against the golden fixtures written by the compiled reference itself, and against
the oracle's restatement of the host solver on seeded workloads, sizes from 3 to the
largest grid the method accepts, and iteration counts other than the reference's 20/20."""
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


def test_largest_grid(fluid, wl):
    n = fluid.gauss_seidel_max_size()
    assert n >= 200
    w = wl.small_sources(n - 2, seed=5)
    with _gs(fluid, n) as s:
        s.upload(w.d, w.u, w.v)
        s.upload_sources(w.ds, w.us, w.vs)
        s.step(w.diffusion, w.viscosity, w.dt, 4)
        gd, gu, gv = s.download()
    od, ou, ov = oracle.cpu_solve(w.d, w.ds, w.diffusion, w.u, w.v, w.us, w.vs, w.viscosity, w.dt, nsteps=4)
    for g_, o in ((gd, od), (gu, ou), (gv, ov)):
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
