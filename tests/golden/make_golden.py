"""Generate the golden fixtures in this directory.

Run in a checkout where the reference sources exist (FLUID2D_REF_SRC, default
/root/reference/src):  python tests/golden/make_golden.py

* ref_cpu_*.npz   inputs and outputs of the reference's unmodified host solver
                  (src/fluid_solver_cpu.cpp, compiled by oracle/build_oracle.py into
                  oracle/_ref/libref_cpu.so). These pin the oracle's "cpu" semantics
                  bit-exactly, and with them the arithmetic the reference's two solvers
                  share (add_sources, both advections, divergence, gradient subtract).
* oracle_gpu_*.npz outputs of the oracle's "gpu" semantics (fluid_solver_gpu.cu,
                  Jacobi) on the same inputs, so the oracle rebuilt on another machine
                  can be checked to produce the same bits.

Inputs are stored in the fixtures (not regenerated), so numpy's platform-dependent
transcendental functions cannot change them between machines.
"""
from __future__ import annotations

import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
from fluid2d_gb300 import workloads  # noqa: E402
import oracle  # noqa: E402

CASES = [
    # name, builder, steps
    ("n34_sources", lambda: workloads.small_sources(32, seed=3), 5),
    ("n130_sources", lambda: workloads.small_sources(128, seed=1), 20),
    ("n66_vortex", lambda: workloads.vortex_field(64, seed=5, kd=20, kp=20, dt=0.1, rate=1e-3, vortices=6,
                                                  rmin=4, rmax=12), 10),
]


def rand_case(n, seed):
    d, u, v, ds, us, vs = workloads.random_state(n, n, seed, vmax=0.05)
    return workloads.Workload(f"rand{n}", n, n, 0.1, 1e-2, 1e-2, 20, 20, d, u, v, ds, us, vs)


CASES += [("n5_random", lambda: rand_case(5, 21), 10), ("n3_random", lambda: rand_case(3, 22), 4)]


def main():
    if oracle.ref_lib() is None:
        raise SystemExit("reference sources not found; cannot generate reference fixtures")
    for name, make, steps in CASES:
        w = make()
        inputs = dict(d=w.d, u=w.u, v=w.v, ds=w.ds, us=w.us, vs=w.vs)
        params = np.array([w.diffusion, w.viscosity, w.dt], np.float32)
        rd, ru, rv = oracle.ref_cpu_solve(w.d, w.ds, w.diffusion, w.u, w.v, w.us, w.vs, w.viscosity, w.dt,
                                          nsteps=steps)
        np.savez_compressed(HERE / f"ref_cpu_{name}.npz", params=params, steps=np.int32(steps), **inputs,
                            out_d=rd, out_u=ru, out_v=rv)
        kd, kp = 15, 20
        gd, gu, gv = oracle.gpu_solve(w.d, w.ds, w.diffusion, w.u, w.v, w.us, w.vs, w.viscosity, w.dt, kd=kd,
                                      kp=kp, nsteps=steps)
        np.savez_compressed(HERE / f"oracle_gpu_{name}.npz", params=params, steps=np.int32(steps),
                            iters=np.array([kd, kp], np.int32), **inputs, out_d=gd, out_u=gu, out_v=gv)
        print(name, "ok")


if __name__ == "__main__":
    main()
