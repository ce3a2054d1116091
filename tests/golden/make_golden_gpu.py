"""Generate the reference-GPU golden fixtures in this directory (ref_gpu_*.npz).

The outputs come from the reference's own GPU solver: src/fluid_solver_gpu.cu compiled
unmodified for sm_103a (oracle/_ref/ref_gpu.fatbin, by oracle/build_oracle.py where the
reference checkout exists) and driven in the reference's order by
oracle/ref_gpu_runner.cpp. It needs a GB300, so it runs on a GPU host that received the
prebuilt fatbinary:

    python -c "import __graft_entry__ as g; g.build()" && python tests/golden/make_golden_gpu.py [OUT_DIR]

(OUT_DIR defaults to this directory.)

Fixtures (the reference's own 15 diffusion / 20 pressure sweeps unless named otherwise):
* ref_gpu_<case>.npz for the five ref_cpu_<case>.npz input sets (3x3 ... 130x130, up to
  20 steps): full output fields; the inputs are read from the ref_cpu fixture.
* ref_gpu_app800.npz: the reference app's own configuration (src/app.cpp:8, 30-34,
  105-115): an 800x800 grid, diffusion 0.5, viscosity 1e-6, dt 0.02 s, started from rest,
  driven by a seeded drag script of density 0.075 and velocity 0.05 x direction per step,
  scaled by width x height (src/simulation.cpp:44-51), 100 steps; the events are stored.
* ref_gpu_n2050_k15.npz / ref_gpu_n2050_k40.npz: 2050x2050 (2048 interior) smooth seeded
  fields from workloads.portable_state, dt 0.05, rates 1e-5, with 15/20 and with 40/40
  sweeps (the benchmark's counts run through the reference's kernels).
The large cases store outputs at a few checkpoints on a lattice of sampled rows and
columns (every 7th or 16th, plus both edges), with the full field's max |value| (corners
excluded) and float64 sum, so the relative L-infinity error over the samples is
normalised like the full-field metric.
"""
from __future__ import annotations

import hashlib
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

OUT = HERE
SMALL = ["n3_random", "n5_random", "n34_sources", "n66_vortex", "n130_sources"]


def lattice(n, stride):
    return np.array(sorted(set(range(0, n, stride)) | {0, 1, n - 2, n - 1}), np.int32)


def field_stats(x):
    m = np.ones(x.shape, bool)
    m[0, 0] = m[0, -1] = m[-1, 0] = m[-1, -1] = False
    return float(np.max(np.abs(x[m]))), float(np.sum(x, dtype=np.float64))


def digest(*arrays):
    h = hashlib.sha1()
    for a in arrays:
        h.update(np.ascontiguousarray(a, np.float32).tobytes())
    return h.hexdigest()


def app800_case(steps=100, checkpoints=(1, 10, 50, 100)):
    n = 800
    events = workloads.drag_script(n, n, steps, seed=7, density=0.075, speed=0.05)
    ev = np.array(events, np.float64)
    d = np.zeros((n, n), np.float32)
    u = d.copy()
    v = d.copy()
    ir, ic = lattice(n, 7), lattice(n, 7)
    out = {}
    k = 0
    for s in range(1, steps + 1):
        ds, us, vs, k = oracle.script_sources(d.shape, events, k, s - 1)
        d, u, v = oracle.ref_gpu_solve(d, ds, 0.5, u, v, us, vs, 1e-6, 0.02, kd=15, kp=20, nsteps=1)
        if s in checkpoints:
            for name, x in zip("duv", (d, u, v)):
                mx, sm = field_stats(x)
                out[f"s{s}_{name}"] = x[np.ix_(ir, ic)]
                out[f"s{s}_{name}_max"] = np.float64(mx)
                out[f"s{s}_{name}_sum"] = np.float64(sm)
    np.savez_compressed(OUT / "ref_gpu_app800.npz", n=np.int32(n), events=ev,
                        params=np.array([0.5, 1e-6, 0.02], np.float32), iters=np.array([15, 20], np.int32),
                        checkpoints=np.array(checkpoints, np.int32), idx_r=ir, idx_c=ic, **out)
    print("app800 ok")


def n2050_case(kd, kp, steps, seed=9):
    n = 2050
    d, u, v = workloads.portable_state(n, n, seed)
    z = np.zeros_like(d)
    h = digest(d, u, v)
    ir, ic = lattice(n, 16), lattice(n, 16)
    out = {}
    for s in range(1, steps + 1):
        d, u, v = oracle.ref_gpu_solve(d, z, 1e-5, u, v, z, z, 1e-5, 0.05, kd=kd, kp=kp, nsteps=1)
        for name, x in zip("duv", (d, u, v)):
            mx, sm = field_stats(x)
            out[f"s{s}_{name}"] = x[np.ix_(ir, ic)]
            out[f"s{s}_{name}_max"] = np.float64(mx)
            out[f"s{s}_{name}_sum"] = np.float64(sm)
    np.savez_compressed(OUT / f"ref_gpu_n2050_k{kd}.npz", n=np.int32(n), seed=np.int32(seed), input_sha1=h,
                        params=np.array([1e-5, 1e-5, 0.05], np.float32), iters=np.array([kd, kp], np.int32),
                        checkpoints=np.arange(1, steps + 1, dtype=np.int32), idx_r=ir, idx_c=ic, **out)
    print(f"n2050 k{kd} ok")


def main():
    global OUT
    if len(sys.argv) > 1:
        OUT = pathlib.Path(sys.argv[1])
        OUT.mkdir(parents=True, exist_ok=True)
    if oracle.ref_gpu_lib() is None:
        raise SystemExit("reference GPU kernels unavailable (no fatbinary or no GPU driver)")
    for name in SMALL:
        f = np.load(HERE / f"ref_cpu_{name}.npz")
        diff, visc, dt = (float(x) for x in f["params"])
        steps = int(f["steps"])
        rd, ru, rv = oracle.ref_gpu_solve(f["d"], f["ds"], diff, f["u"], f["v"], f["us"], f["vs"], visc, dt,
                                          kd=15, kp=20, nsteps=steps)
        np.savez_compressed(OUT / f"ref_gpu_{name}.npz", inputs=f"ref_cpu_{name}.npz", steps=np.int32(steps),
                            iters=np.array([15, 20], np.int32), out_d=rd, out_u=ru, out_v=rv)
        print(name, "ok")
    app800_case()
    n2050_case(15, 20, 2)
    n2050_case(40, 40, 3)


if __name__ == "__main__":
    main()
