"""Benchmark of the fluid-2d solver step on GB300.

Workload (default): a single 2048x2048-interior grid (2050^2 with boundary), fp32,
dt 0.05, diffusion = viscosity = 1e-5, 40 diffusion and 40 pressure Jacobi sweeps per
projection, initial velocity the sum of 64 seeded Gaussian-core vortices, density
seeded low-frequency noise, no sources. Metric: interior cell-steps per second.

  value     device-resident stepping (fs_step, graph replay), inputs already in HBM;
            every timed step is bracketed by CUDA events on the solver's stream and
            L2 is flushed (a 256 MiB write) between timed steps.
  e2e       the same metric through fs_solve_host() with pinned host buffers: each
            step uploads the state and sources and downloads the state, like the
            reference's fluid_solver_gpu::solve.
  roofline  stencil kernels (the dominant kind): the bytes each pass must move (every
            array it reads or writes, once: 12 B per interior cell and field for a
            middle pass) over the passes' CUDA-event time in a profiled step, against
            the measured HBM copy bandwidth. The profiled step has the timed graph's
            launches and streams, with an event around each launch. Beside it: the
            per-sweep model (12 B per cell and field per sweep, what the reference's
            one kernel per sweep moves) as model_equivalent_*, DRAM traffic per launch
            from ncu (traffic, dram_frac) and the resource that binds the pass.
  cpu_baseline  the oracle's Jacobi restatement of the same step (OpenMP, all host
            cores) on a bounded sample.

--impl reference times the reference's own CPU solver algorithm (fluid_solver_cpu,
restated in the oracle and pinned bit-exactly against the compiled reference) on the
host cores, single-threaded as the reference is.

Multi-GPU: the path does not shard (one grid per handle); --gpus N runs N
independent replicas, one per rank, and `value` sums their throughput.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--size", type=int, default=2048, help="interior cells per side")
    ap.add_argument("--kd", type=int, default=40)
    ap.add_argument("--kp", type=int, default=40)
    ap.add_argument("--sweeps", type=int, default=0, help="temporal-blocking depth (0 = default)")
    ap.add_argument("--tile-rows", type=int, default=0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile-steps", type=int, default=3)
    ap.add_argument("--samples", type=int, default=20000, help="learned: training pairs")
    ap.add_argument("--epochs", type=int, default=8, help="learned: training epochs")
    ap.add_argument("--weights", default="", help="learned: save trained parameters here (.npy)")
    ap.add_argument("--load-weights", default="", help="learned: skip training and load parameters")
    ap.add_argument("--eval-sizes", default="1024,2048")
    ap.add_argument("--tols", default="1e-1,1e-2,1e-3,1e-4")
    ap.add_argument("--workload", choices=("vortex", "small", "batch", "residual", "learned", "gauss-seidel",
                                           "depth"),
                    default="vortex",
                    help="vortex: the default 2048^2 line; small: 130^2 with sources, 20/20 sweeps; "
                         "batch: 256 uneven grids, 30/30 sweeps, batch vs looped handles; "
                         "residual: pressure to a relative-residual target")
    ap.add_argument("--tol", type=float, default=1e-4)
    ap.add_argument("--max-iters", type=int, default=None,
                    help="sweep cap per projection (default: residual 2000, learned 20000, depth 400)")
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--batch-sizes", default="",
                    help="batch: comma-separated interior sizes, one grid each (default: --count seeded "
                         "sizes in 64..1024)")
    ap.add_argument("--gs-size", type=int, default=128, help="gauss-seidel: interior cells per side")
    ap.add_argument("--depth-target-steps", type=int, default=0,
                    help="depth: also time coarse-corrected solves that reach --tol, for this many steps")
    ap.add_argument("--tune", action="store_true", help="autotune the tiling before timing")
    ap.add_argument("--cycles", type=int, default=0, help="learned: most corrections per projection (0 = cap / cycle-iters)")
    ap.add_argument("--cycle-iters", type=int, default=0,
                    help="learned: Jacobi sweeps after each correction (0 = the library default, 256)")
    ap.add_argument("--coarse-cycle-iters", type=int, default=128,
                    help="learned: the same for the coarse_only mode (its fastest setting at 1e-4: 128)")
    ap.add_argument("--train-size", type=int, default=512, help="learned: grid of the training runs")
    ap.add_argument("--learned-grid", type=int, default=0, help="learned: coarse grid side (0 = default, 32, 64)")
    ap.add_argument("--modes", default="previous,learned,coarse_only",
                    help="learned: pressure starts to compare (zero, previous, learned, coarse_only)")
    ap.add_argument("--mid-solve-samples", type=int, default=0,
                    help="learned: add this many mid-solve states met by a first-round network, then retrain")
    return ap.parse_args()


# ncu on this build (profiles/stencil_kernel_2048_vortex.md): DRAM bytes read + written per
# interior cell and field by one depth-8 pass at 2048^2, and the unit that bounds the pass
NCU_DRAM_BYTES_PER_CELL_FIELD_PASS = 8.2
NCU_BINDING = ("instruction issue and latency: 2 CTAs of 8 warps per SM at 128 registers (24 % of the warp "
               "slots); ncu on a 2048^2 middle pressure pass: issue active 39 %, DRAM 15 %, L1/shared 48 %, "
               "largest stall instruction fetch")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def metric_name():
    return "cell-steps/s"


def workload_config(a, extra=None):
    cfg = {"workload": f"vortex_field single grid {a.size}x{a.size} interior fp32, dt 0.05, rates 1e-5, "
                       f"Kd={a.kd} Kp={a.kp} Jacobi sweeps, 64 vortices",
           "interior": a.size, "kd": a.kd, "kp": a.kp, "l2": "flushed between timed steps (256 MiB write)",
           "parallelism": "replicas"}
    if extra:
        cfg.update(extra)
    return cfg


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            j = json.loads(p.read_text())
            return float(j["hbm_gbs"]), "measured"
        except (ValueError, KeyError):
            pass
    return 6800.0, "fallback"


def cpu_baseline(w, kd, kp, budget_s=15.0):
    """The oracle's Jacobi restatement (same arithmetic as the CUDA path), OpenMP over
    all host cores, timed on whole steps until about budget_s seconds elapse."""
    import oracle

    cores = os.cpu_count() or 1
    d, u, v = w.state()
    steps = 0
    t0 = time.perf_counter()
    while True:
        d, u, v = oracle.gpu_solve(d, w.ds, w.diffusion, u, v, w.us, w.vs, w.viscosity, w.dt, kd=kd, kp=kp)
        steps += 1
        if time.perf_counter() - t0 > budget_s or steps >= 20:
            break
    el = time.perf_counter() - t0
    return {"value": w.interior_cells * steps / el, "unit": "cell-steps/s", "cores": cores, "kind": "port",
            "sample": f"{steps} whole steps of the {w.rows - 2}^2 workload, oracle Jacobi restatement of "
                      f"fluid_solver_gpu.cu, OpenMP {cores} threads, {el:.1f} s"}


def run_reference(a):
    """Reference arm: fluid_solver_cpu (Gauss-Seidel) restated in the oracle and pinned
    bit-exactly against the compiled reference; single-threaded like the reference."""
    __graft_entry__.load_package()
    import oracle
    from fluid2d_gb300 import workloads

    rank, world, _ = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        if rank != 0:
            dist.barrier()
            dist.destroy_process_group()
            return
    size = a.size
    w = workloads.vortex_field(size, seed=2, kd=a.kd, kp=a.kp)
    d, u, v = w.state()
    # one probe step sets the sample size so the run stays within a few minutes
    t0 = time.perf_counter()
    oracle.cpu_solve(d, w.ds, w.diffusion, u, v, w.us, w.vs, w.viscosity, w.dt, kd=a.kd, kp=a.kp)
    per = time.perf_counter() - t0
    budget = 150.0
    sample = w
    if per * (a.steps + a.warmup) > budget:
        scale = max(64, int(size * (budget / (per * (a.steps + a.warmup))) ** 0.5) // 64 * 64)
        sample = workloads.vortex_field(scale, seed=2, kd=a.kd, kp=a.kp)
    d, u, v = sample.state()
    for _ in range(a.warmup):
        d, u, v = oracle.cpu_solve(d, sample.ds, sample.diffusion, u, v, sample.us, sample.vs, sample.viscosity,
                                   sample.dt, kd=a.kd, kp=a.kp)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        d, u, v = oracle.cpu_solve(d, sample.ds, sample.diffusion, u, v, sample.us, sample.vs, sample.viscosity,
                                   sample.dt, kd=a.kd, kp=a.kp)
    el = time.perf_counter() - t0
    val = sample.interior_cells * a.steps / el
    line = {"metric": metric_name(), "value": val, "unit": "cell-steps/s", "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * el / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "impl": "reference",
            "config": workload_config(a, {"sample_interior": sample.rows - 2,
                                          "l2": "not applicable (host cores)",
                                          "method": "Gauss-Seidel (the reference's host solver), "
                                                    f"Kd={a.kd} Kp={a.kp}"}),
            "cpu_baseline": {"value": val, "unit": "cell-steps/s", "cores": 1, "kind": "port",
                             "sample": f"{a.steps} steps of a {sample.rows - 2}^2 grid (same workload family), "
                                       "fluid_solver_cpu.cpp restated (Gauss-Seidel), single thread"},
            "e2e": {"value": val, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


def run_ours(a):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    pkg = __graft_entry__.load_package()
    from fluid2d_gb300 import build_lib, workloads

    build_lib.build()
    w = workloads.vortex_field(a.size, seed=2 + rank, kd=a.kd, kp=a.kp)
    cfg = dict(diffuse_iterations=a.kd, pressure_iterations=a.kp, device=dev, check_finite=0)
    if a.sweeps:
        cfg["sweeps_per_pass"] = a.sweeps
    if a.tile_rows:
        cfg["tile_rows"] = a.tile_rows
    s = pkg.Solver(w.rows, w.cols, **cfg)
    s.upload(*w.state())
    s.upload_sources(*w.sources())
    view = s.device_view()
    stream = torch.cuda.ExternalStream(view.stream, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    # warm-up (also captures the step graph)
    s.step(w.diffusion, w.viscosity, w.dt, nsteps=max(3, a.warmup))
    launches0 = s.stats()["kernel_launches"]
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    clocks = ClockSampler(dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    t_wall = time.perf_counter()
    for k in range(a.steps):
        flush_l2()
        evs[k][0].record(stream)
        s.step(w.diffusion, w.viscosity, w.dt, nsteps=1, sync=False)
        evs[k][1].record(stream)
    s.sync()
    torch.cuda.synchronize(dev)
    t_wall = time.perf_counter() - t_wall
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in evs)
    launches = s.stats()["kernel_launches"] - launches0
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    cells = w.interior_cells
    value = cells * a.steps * world / (ms / 1e3)

    # per-kernel CUDA-event profile of steps in the timed graph's shape (same launches,
    # same streams, the density branch beside the main stream); stencil = dominant kind
    stats0 = s.stats()
    prof = None
    for _ in range(a.profile_steps):
        flush_l2()
        torch.cuda.synchronize(dev)
        p = s.profile_step(w.diffusion, w.viscosity, w.dt)
        if prof is None:
            prof = p
        else:
            for k in prof:
                for f in prof[k]:
                    prof[k][f] += p[k][f]
    peak, peak_kind = measured_peak()
    st = prof["stencil"]
    n_st = st["launches"]
    ms_launch = st["ms"] / n_st
    # achieved: the bytes each pass must move itself (every array it reads or writes,
    # once) over its event time; the per-sweep model (every array once per sweep, the
    # reference's one-kernel-per-sweep cost) is reported beside it
    achieved = (st["pass_bytes"] / n_st) / (ms_launch / 1e3) / 1e9
    model_gbps = (st["bytes"] / n_st) / (ms_launch / 1e3) / 1e9
    K = stats0["sweeps_per_pass"]
    diff_passes, proj_passes = -(-a.kd // K), -(-a.kp // K)
    field_passes = 3 * diff_passes + 2 * proj_passes
    stencil_launches = 3 * diff_passes + 2 * proj_passes - diff_passes  # u and v share a launch
    # DRAM traffic per launch: ncu's dram__bytes_read + write per field-pass of this kernel
    # at 2048^2, depth 8 (profiles/stencil_kernel_2048_vortex.md), times the field-passes of
    # an average launch of the step
    traffic = (NCU_DRAM_BYTES_PER_CELL_FIELD_PASS * cells * field_passes / stencil_launches
               if (K == 8 and a.size == 2048) else None)
    main_ms = {k: (prof[k]["ms"] - prof[k]["branch_ms"]) / a.profile_steps for k in prof}
    branch_ms = {k: prof[k]["branch_ms"] / a.profile_steps for k in prof}
    # shares of all kernel time (both streams), comparable with ncu's serialised launch list
    all_ms = sum(prof[k]["ms"] for k in prof)
    shares = {k: round(prof[k]["ms"] / all_ms, 4) for k in prof}
    per_kernel = {}
    for k in prof:
        if not prof[k]["launches"]:
            continue
        ms_k = prof[k]["ms"]
        gbps = (prof[k]["pass_bytes"] / (ms_k / 1e3) / 1e9) if ms_k > 0 else None
        per_kernel[k] = {"launches_per_step": prof[k]["launches"] / a.profile_steps,
                         "branch_launches_per_step": prof[k]["branch_launches"] / a.profile_steps,
                         "ms_per_step_main_stream": main_ms[k], "ms_per_step_branch": branch_ms[k],
                         "pass_GBps": gbps, "frac_of_hbm": gbps / peak if gbps else None}

    # end to end through the reference-shaped call with pinned host buffers
    e2e = e2e_pageable = None
    if not a.no_e2e:
        pins = [pkg.PinnedArray(w.rows, w.cols) for _ in range(6)]
        for p_, src in zip(pins, (w.d, w.ds, w.u, w.v, w.us, w.vs)):
            p_.array[...] = src
        hd, hds, hu, hv, hus, hvs = (p_.array for p_ in pins)
        e2e_steps = max(3, min(a.steps, 20))
        for _ in range(2):
            s.solve(hd, hds, w.diffusion, hu, hv, hus, hvs, w.viscosity, w.dt)
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            s.solve(hd, hds, w.diffusion, hu, hv, hus, hvs, w.viscosity, w.dt)
        el = time.perf_counter() - t0
        if world > 1:
            t = torch.tensor([el], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            el = float(t.item())
        fb = w.rows * w.cols * 4
        e2e = {"value": cells * e2e_steps * world / el, "unit": "cell-steps/s", "h2d_bytes_per_step": 6 * fb,
               "d2h_bytes_per_step": 3 * fb, "steps": e2e_steps, "ms_per_step": 1e3 * el / e2e_steps,
               "host_memory": "pinned (fs_host_alloc)"}
        for p_ in pins:
            p_.free()
        # the same call on pageable host memory, which is what the C++ drop-in adapter
        # passes (the reference's grid<float> is a std::vector)
        pg = [np.array(x, np.float32, copy=True) for x in (w.d, w.ds, w.u, w.v, w.us, w.vs)]
        for _ in range(2):
            s.solve(pg[0], pg[1], w.diffusion, pg[2], pg[3], pg[4], pg[5], w.viscosity, w.dt)
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            s.solve(pg[0], pg[1], w.diffusion, pg[2], pg[3], pg[4], pg[5], w.viscosity, w.dt)
        el = time.perf_counter() - t0
        if world > 1:
            t = torch.tensor([el], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            el = float(t.item())
        e2e_pageable = {"value": cells * e2e_steps * world / el, "unit": "cell-steps/s",
                        "h2d_bytes_per_step": 6 * fb, "d2h_bytes_per_step": 3 * fb, "steps": e2e_steps,
                        "ms_per_step": 1e3 * el / e2e_steps, "host_memory": "pageable (numpy)"}

    if e2e:
        # the host call's own step (uploads overlapped with a split diffusion on large grids)
        e2e["launches_per_step"] = s.stats()["launches_per_step"]
    if rank == 0:
        line = {"metric": metric_name(), "value": value, "unit": "cell-steps/s", "n_gpus": world,
                "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded vortex field)",
                "config": workload_config(a, {"sweeps_per_pass": stats0["sweeps_per_pass"],
                                              "tile_rows": stats0["tile_rows"],
                                              "launches_per_step": stats0["launches_per_step"],
                                              "passes_per_step": stats0["passes_per_step"]}),
                "gpu_launches": launches,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                             "kernel": "stencil_kernel", "launches_profiled": n_st,
                             "bytes_per_launch": st["pass_bytes"] / n_st,
                             "bytes_model": "each array a pass reads or writes, once (12 B per interior cell "
                                            "and field for a middle pass, 16 first, 24 last pressure)",
                             "ms_per_launch": ms_launch,
                             "traffic_source": "ncu dram__bytes_read+write per field-pass at 2048^2, depth 8 "
                                               f"({NCU_DRAM_BYTES_PER_CELL_FIELD_PASS} B per cell), "
                                               "profiles/stencil_kernel_2048_vortex.md",
                             "dram_frac": ((traffic / (ms_launch / 1e3) / 1e9) / peak) if traffic else None,
                             "model_equivalent_GBps": model_gbps, "model_equivalent_frac": model_gbps / peak,
                             "model": "per-sweep model, 12 B per cell and field per sweep (the reference's "
                                      "one-kernel-per-sweep traffic)",
                             "binding_resource": NCU_BINDING},
                "kernel_shares": shares,
                "kernels": per_kernel,
                "stencil_ms_per_step_main_stream": main_ms["stencil"],
                "step_algorithmic_bytes_per_cell": sum(prof[k]["bytes"] for k in prof) / a.profile_steps / cells,
                "clocks": clk, "wall_s": t_wall}
        if e2e:
            line["e2e"] = e2e
            line["e2e_pageable"] = e2e_pageable
        if not a.no_cpu and world == 1:
            line["cpu_baseline"] = cpu_baseline(w, a.kd, a.kp)
        print(json.dumps(line), flush=True)
    s.close()
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def _timed_steps(step, sync, stream, steps, flush_l2, torch, dev):
    """CUDA-event time of `steps` calls of step(), L2 flushed before each."""
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize(dev)
    for k in range(steps):
        flush_l2()
        evs[k][0].record(stream)
        step()
        evs[k][1].record(stream)
    sync()
    torch.cuda.synchronize(dev)
    return sum(e0.elapsed_time(e1) for e0, e1 in evs)


def run_small(a):
    """130x130 (N=128) with 4 density and 4 velocity sources, dt 0.1, rates 1e-4,
    20/20 sweeps, the reference's own CPU-runnable case."""
    import torch

    pkg = __graft_entry__.load_package()
    from fluid2d_gb300 import workloads

    w = workloads.small_sources(128, seed=1)
    s = pkg.Solver(w.rows, w.cols, diffuse_iterations=20, pressure_iterations=20, device=0, check_finite=0)
    s.upload(*w.state())
    s.upload_sources(*w.sources())
    stream = torch.cuda.ExternalStream(s.device_view().stream, device=0)
    s.step(w.diffusion, w.viscosity, w.dt, nsteps=a.warmup)
    clocks = ClockSampler(0)
    clocks.start()
    ms = _timed_steps(lambda: s.step(w.diffusion, w.viscosity, w.dt, 1, sync=False), s.sync, stream, a.steps,
                      lambda: None, torch, 0)
    clk = clocks.stop()
    line = {"metric": metric_name(), "value": w.interior_cells * a.steps / (ms / 1e3), "unit": "cell-steps/s",
            "clocks": clk,
            "n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded sources)",
            "config": {"workload": "small_sources 128x128 interior, 20/20 sweeps, dt 0.1, rates 1e-4",
                       "l2": "not flushed (working set 1.5 MB)", **{k: v for k, v in s.stats().items()
                                                                    if k in ("launches_per_step", "passes_per_step")}}}
    print(json.dumps(line), flush=True)
    s.close()


def run_depth(a):
    """Temporal-blocking depth on a large grid (8192^2 vortex field, pressure to a
    relative-residual target, 50 steps): plain Jacobi from the previous pressure under a
    sweep cap (the cap binds: Jacobi damps the smooth modes at ~pi^2/N^2 per sweep, so
    1e-4 is out of its reach at this size and every depth does the same sweeps) at depth
    1 (one sweep per HBM pass, the plain kernels), 2, 4, 8, the default and the
    autotuner's choice; then, with --depth-target-steps, the same target reached by
    coarse-corrected Jacobi cycles (the learned warm start's machinery with an all-zero
    network and the FP64 defect correction) at depth 1 and at the tuned depth."""
    import torch

    pkg = __graft_entry__.load_package()
    from fluid2d_gb300 import build_lib, workloads

    build_lib.build()
    w = workloads.vortex_field(a.size, seed=2, kd=a.kd, kp=a.kp)
    base = dict(diffuse_iterations=a.kd, pressure_tolerance=a.tol, warm_start=pkg.FS_WARM_PREVIOUS, device=0,
                check_finite=0)
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    tuned = pkg.autotune(w.rows, w.cols, w.diffusion, w.viscosity, w.dt, steps=2,
                         pressure_max_iterations=a.max_iters, **base)
    tuned["tuning_s"] = time.perf_counter() - t0
    print(json.dumps({"autotuner": tuned}), flush=True)

    def run(cfg, steps, net=None):
        s = pkg.Solver(w.rows, w.cols, **cfg)
        if net is not None:
            s.set_network(net)
        s.upload(*w.state())
        s.upload_sources(*w.sources())
        stream = torch.cuda.ExternalStream(s.device_view().stream, device=0)
        sweeps, res, ms_tot = [], [], 0.0
        for k in range(a.warmup + steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.step(w.diffusion, w.viscosity, w.dt, 1, sync=False)
            e1.record(stream)
            try:
                s.sync()
            except pkg.FluidError as e:
                if e.code != pkg.FS_ERR_NOT_CONVERGED:
                    raise
            st = s.stats()
            if k >= a.warmup:
                ms_tot += e0.elapsed_time(e1)
                sweeps += st["pressure_iterations_last"]
                res += st["pressure_residual_last"]
        s.close()
        return st, ms_tot / steps, sweeps, res

    out = []
    plans = [(d, 0, str(d)) for d in (1, 2, 4, 8)] + [(0, 0, "default"),
                                                      (tuned["sweeps_per_pass"], tuned["tile_rows"], "autotuned")]
    for depth, rows_, name in plans:
        cfg = dict(base, pressure_max_iterations=a.max_iters, sweeps_per_pass=depth, tile_rows=rows_)
        st, ms, sweeps, res = run(cfg, a.steps)
        total_sweeps = 3 * a.kd + float(np.mean(sweeps)) * 2
        out.append({"depth": st["sweeps_per_pass"], "tile_rows": st["tile_rows"], "requested": name,
                    "ms_per_step": ms, "pressure_sweeps_per_projection": float(np.mean(sweeps)),
                    "residual_max": float(np.max(res)),
                    "cell_sweeps_per_s": w.interior_cells * total_sweeps / (ms / 1e3)})
        print(json.dumps(out[-1]), flush=True)
    target = []
    if a.depth_target_steps > 0:
        from fluid2d_gb300 import learned

        zero_net = np.zeros(learned.NPARAM, np.float32)
        for depth, rows_, name in ((1, 0, "1"), (tuned["sweeps_per_pass"], tuned["tile_rows"], "autotuned")):
            cfg = dict(base, warm_start=pkg.FS_WARM_LEARNED, pressure_max_iterations=20000,
                       sweeps_per_pass=depth, tile_rows=rows_)
            st, ms, sweeps, res = run(cfg, a.depth_target_steps, zero_net)
            target.append({"depth": st["sweeps_per_pass"], "tile_rows": st["tile_rows"], "requested": name,
                           "ms_per_step": ms, "pressure_sweeps_per_projection": float(np.mean(sweeps)),
                           "residual_max": float(np.max(res)),
                           "missed_target": int(np.sum(np.array(res) > a.tol)), "steps": a.depth_target_steps})
            print(json.dumps(target[-1]), flush=True)
    line = {"metric": "ms/step by temporal-blocking depth", "unit": "ms/step", "higher_is_better": False,
            "value": out[-1]["ms_per_step"], "steps": a.steps, "warmup": a.warmup, "dtype": "f32",
            "data": "synthetic (seeded vortex field)",
            "config": {"workload": f"vortex_field {a.size}^2, Kd={a.kd}, pressure to {a.tol:g} relative residual, "
                                   f"cap {a.max_iters} sweeps (binding)", "l2": "inputs far larger than L2"},
            "autotuner": tuned, "depths": out, "to_target_coarse_corrected": target,
            "clocks": clocks.stop()}
    print(json.dumps(line), flush=True)


def run_gauss_seidel(a):
    """The reference's host solver (fluid_solver_cpu, Gauss-Seidel 20/20) reproduced on
    the GPU (FS_METHOD_GAUSS_SEIDEL): by default on its own CPU-runnable case, 130x130
    (N=128) with 4 density and 4 velocity sources, dt 0.1, rates 1e-4; with --gs-size N
    (N > 128) on the N^2 vortex field of the main workload at 20/20 sweeps (800: the
    reference app's grid, 2048: the benchmark's; the tiled form above 232 interior cells, 234 with the boundary). Device-resident
    steps (value), the reference-style host round trip per step (e2e), the oracle's
    single-thread restatement of the host solver (cpu_baseline, a bounded sample), and a
    bit-for-bit check of the state after the timed steps."""
    import torch

    pkg = __graft_entry__.load_package()
    import oracle
    from fluid2d_gb300 import workloads

    N = a.gs_size
    if N <= 128:
        w = workloads.small_sources(N, seed=1)
        desc = f"small_sources {N}x{N} interior, Gauss-Seidel 20/20 sweeps, dt 0.1, rates 1e-4"
        data = "synthetic (seeded sources)"
    else:
        w = workloads.vortex_field(N, seed=2, kd=20, kp=20)
        desc = f"vortex_field {N}x{N} interior, Gauss-Seidel 20/20 sweeps, dt 0.05, rates 1e-5"
        data = "synthetic (seeded vortex field)"
    steps = a.steps
    s = pkg.FluidSolverGaussSeidel(w.rows, device=0, check_finite=0)
    s.upload(*w.state())
    s.upload_sources(*w.sources())
    stream = torch.cuda.ExternalStream(s.device_view().stream, device=0)
    s.step(w.diffusion, w.viscosity, w.dt, nsteps=a.warmup)
    clocks = ClockSampler(0)
    clocks.start()
    ms = _timed_steps(lambda: s.step(w.diffusion, w.viscosity, w.dt, 1, sync=False), s.sync, stream, steps,
                      lambda: None, torch, 0)
    clk = clocks.stop()
    gd, gu, gv = s.download()
    od, ou, ov = w.state()
    od, ou, ov = oracle.cpu_solve(od, w.ds, w.diffusion, ou, ov, w.us, w.vs, w.viscosity, w.dt,
                                  nsteps=a.warmup + steps)
    exact = bool(np.array_equal(gd, od) and np.array_equal(gu, ou) and np.array_equal(gv, ov))
    s.close()
    # e2e: host grids in and out every step, as the reference's solve() does
    s = pkg.FluidSolverGaussSeidel(w.rows, device=0, check_finite=0)
    d, u, v = w.state()
    for _ in range(a.warmup):
        s.solve(d, w.ds, w.diffusion, u, v, w.us, w.vs, w.viscosity, w.dt)
    t0 = time.perf_counter()
    for _ in range(steps):
        s.solve(d, w.ds, w.diffusion, u, v, w.us, w.vs, w.viscosity, w.dt)
    e2e_s = time.perf_counter() - t0
    s.close()
    # CPU: the host solver restated (bit-identical to the compiled reference), one thread
    d, u, v = w.state()
    t0 = time.perf_counter()
    cpu_steps = 0
    while cpu_steps < steps and (cpu_steps == 0 or time.perf_counter() - t0 < 15.0):
        d, u, v = oracle.cpu_solve(d, w.ds, w.diffusion, u, v, w.us, w.vs, w.viscosity, w.dt)
        cpu_steps += 1
    cpu_s = time.perf_counter() - t0
    cells = w.interior_cells
    line = {"metric": f"cell-steps/s, Gauss-Seidel method (the reference's host solver), {w.rows}^2",
            "value": cells * steps / (ms / 1e3), "unit": "cell-steps/s", "n_gpus": 1, "steps": steps,
            "warmup": a.warmup, "ms_per_step": ms / steps, "higher_is_better": True, "dtype": "f32",
            "data": data, "bit_exact_vs_oracle": exact, "clocks": clk,
            "e2e": {"value": cells * steps / e2e_s, "unit": "cell-steps/s",
                    "h2d_bytes_per_step": 6 * w.rows * w.cols * 4, "d2h_bytes_per_step": 3 * w.rows * w.cols * 4},
            "cpu_baseline": {"value": cells * cpu_steps / cpu_s, "unit": "cell-steps/s", "cores": 1, "kind": "port",
                             "sample": f"the first {cpu_steps} steps, fluid_solver_cpu.cpp restated, single thread"},
            "config": {"workload": desc, "l2": "not flushed"}}
    print(json.dumps(line), flush=True)


def run_batch(a):
    """256 independent grids, N uniform in {64..1024}, 30/30 sweeps: one fs_batch
    (one launch per sub-step, graph per step; tiling from the batch autotuner unless
    --sweeps / --tile-rows fix it) vs the same grids as 256 handles. Under
    torchrun (N > 1) the grids are dealt to ranks by longest-processing-time-first on
    cells x sweeps (replicas.shard), each rank steps its own batch, and the ranks meet
    only at the barriers around the timed region; the value is all ranks' cells over the
    slowest rank's time."""
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = local if world > 1 else 0
    pkg = __graft_entry__.load_package()
    from fluid2d_gb300 import build_lib, replicas, workloads

    build_lib.build()
    kd = kp = 30
    sizes = [int(x) for x in a.batch_sizes.split(",")] if a.batch_sizes else None
    all_sims = workloads.batch(a.count, seed=4, kd=kd, kp=kp, sizes=sizes)
    mine = replicas.shard([(w.rows, w.cols) for w in all_sims], world, rank, kd, kp)
    sims = [all_sims[i] for i in mine]
    shapes = [(w.rows, w.cols) for w in sims]
    cells = sum(w.interior_cells for w in sims)
    total_cells = sum(w.interior_cells for w in all_sims)
    w0 = sims[0]
    cfg = dict(diffuse_iterations=kd, pressure_iterations=kp, device=dev, check_finite=0)
    cfg_handles = dict(cfg)  # the handles keep their own default tiling rule
    tuned = None
    if a.sweeps or a.tile_rows:
        if a.sweeps:
            cfg["sweeps_per_pass"] = cfg_handles["sweeps_per_pass"] = a.sweeps
        if a.tile_rows:
            cfg["tile_rows"] = cfg_handles["tile_rows"] = a.tile_rows
    else:
        # the batch's tiling from its autotuner (whole batch steps per candidate)
        tuned = pkg.autotune_batch(shapes, w0.diffusion, w0.viscosity, w0.dt, steps=2, **cfg)
        cfg["sweeps_per_pass"] = tuned["sweeps_per_pass"]
        cfg["tile_rows"] = tuned["tile_rows"]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    b = pkg.Batch(shapes, **cfg)
    for k, w in enumerate(sims):
        b.upload(k, *w.state())
        b.upload_sources(k, *w.sources())
    stream = torch.cuda.ExternalStream(b.stream, device=dev)

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    b.step(w0.diffusion, w0.viscosity, w0.dt, nsteps=max(3, a.warmup))
    l0 = b.stats()["kernel_launches"]
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(dev)
    clocks.start()
    ms_b = _timed_steps(lambda: b.step(w0.diffusion, w0.viscosity, w0.dt, 1, sync=False), b.sync, stream, a.steps,
                        flush_l2, torch, dev)
    clk = clocks.stop()
    if world > 1:
        torch.distributed.barrier()
        t = torch.tensor([ms_b], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_b = float(t.item())
    launches = b.stats()["kernel_launches"] - l0
    st = b.stats()
    # the batch timed the way the looped handles are below (host wall clock, steps back to
    # back, no flush), for a like-for-like ratio
    steps_w = max(2, a.steps // 4)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(steps_w):
        b.step(w0.diffusion, w0.viscosity, w0.dt, 1, sync=False)
        b.sync()
    batch_wall_ms = (time.perf_counter() - t0) * 1e3 / steps_w
    b.close()
    looped = None
    if world == 1:
        # the same grids as independent handles, stepped one after another per step
        hs = []
        for w in sims:
            s = pkg.Solver(w.rows, w.cols, **cfg_handles)
            s.upload(*w.state())
            s.upload_sources(*w.sources())
            s.step(w.diffusion, w.viscosity, w.dt, nsteps=1)
            hs.append(s)
        steps_l = max(2, a.steps // 4)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(steps_l):
            for h in hs:
                h.step(w0.diffusion, w0.viscosity, w0.dt, 1, sync=False)
            for h in hs:
                h.sync()
        ms_l = (time.perf_counter() - t0) * 1e3
        for h in hs:
            h.close()
        looped = {"value": cells * steps_l / (ms_l / 1e3), "ms_per_step": ms_l / steps_l,
                  "timing": "host wall clock, one graph per handle per step"}
    if rank == 0:
        line = {"metric": metric_name(), "value": total_cells * a.steps / (ms_b / 1e3), "unit": "cell-steps/s",
                "n_gpus": world, "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms_b / a.steps,
                "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded vortex fields + sources)", "gpu_launches": launches,
                "config": {"workload": (f"batch of {len(all_sims)} grids, N uniform in 64..1024, Kd=Kp=30, dt 0.05"
                                        if not sizes else
                                        f"batch of {len(all_sims)} grids, N = {a.batch_sizes}, Kd=Kp=30, dt 0.05"),
                           "interior_cells": total_cells, "rank0_grids": len(sims),
                           "launches_per_step": st["launches_per_step"], "sweeps_per_pass": st["sweeps_per_pass"],
                           "tile_rows": st["tile_rows"], "l2": "flushed between timed steps",
                           "parallelism": f"grids dealt to {world} rank(s) by LPT on cells x sweeps"},
                "clocks": clk}
        if tuned:
            line["autotuner"] = tuned
        line["batch_wall_clock"] = {"value": total_cells / (batch_wall_ms / 1e3), "ms_per_step": batch_wall_ms,
                                    "timing": "host wall clock, one graph per step, no flush"}
        if looped:
            line["looped_handles"] = looped
            line["batch_vs_looped"] = looped["ms_per_step"] / batch_wall_ms
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def run_residual(a):
    """Pressure solves run to a relative residual target (the to-residual mode), with
    zero or previous-pressure warm start; reports sweeps used per projection."""
    import torch

    pkg = __graft_entry__.load_package()
    from fluid2d_gb300 import build_lib, workloads

    build_lib.build()
    w = workloads.vortex_field(a.size, seed=2, kd=a.kd, kp=a.kp)
    clocks = ClockSampler(0)
    clocks.start()
    out = []
    for warm in (0, 1):
        cfg = dict(diffuse_iterations=a.kd, pressure_tolerance=a.tol, pressure_max_iterations=a.max_iters,
                   warm_start=warm, device=0, check_finite=0)
        if a.sweeps:
            cfg["sweeps_per_pass"] = a.sweeps
        if a.tile_rows:
            cfg["tile_rows"] = a.tile_rows
        s = pkg.Solver(w.rows, w.cols, **cfg)
        s.upload(*w.state())
        s.upload_sources(*w.sources())
        stream = torch.cuda.ExternalStream(s.device_view().stream, device=0)
        iters, res, ms_tot = [], [], 0.0
        for k in range(a.warmup + a.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.step(w.diffusion, w.viscosity, w.dt, 1, sync=False)
            e1.record(stream)
            try:
                s.sync()
            except pkg.FluidError as e:
                if e.code != pkg.FS_ERR_NOT_CONVERGED:
                    raise
            st = s.stats()
            if k >= a.warmup:
                ms_tot += e0.elapsed_time(e1)
                iters.append(st["pressure_iterations_last"])
                res.append(st["pressure_residual_last"])
        out.append({"warm_start": ["zero", "previous"][warm], "ms_per_step": ms_tot / a.steps,
                    "sweeps_per_projection_mean": float(np.mean(iters)), "sweeps_max": int(np.max(iters)),
                    "residual_max": float(np.max(res)), "capped_projections": int(np.sum(np.array(iters) >= a.max_iters)),
                    "sweeps_per_pass": s.stats()["sweeps_per_pass"], "tile_rows": s.stats()["tile_rows"]})
        s.close()
    line = {"metric": "ms/step to relative pressure residual", "unit": "ms/step", "higher_is_better": False,
            "value": out[1]["ms_per_step"], "steps": a.steps, "warmup": a.warmup, "dtype": "f32",
            "data": "synthetic (seeded vortex field)",
            "config": {"workload": f"vortex_field {a.size}^2, pressure to {a.tol:g} relative residual, "
                                   f"cap {a.max_iters} sweeps, Kd={a.kd}"},
            "modes": out, "clocks": clocks.stop()}
    print(json.dumps(line), flush=True)


def run_learned(a):
    """Learned pressure correction: train on (residual, exact correction) pairs from
    seeded 512^2 vortex runs, then step vortex fields at the evaluation sizes with the
    pressure solved to each residual target by (i) Jacobi from the previous pressure and
    (ii) Jacobi with the network's corrections (one before each segment of
    --cycle-iters sweeps, starting from the previous pressure) and (iii) the same with an
    all-zero network, so that only the coarse post-smoothing acts (the ablation that
    isolates what the trained network adds); report sweeps per projection, ms/step, how
    many projections missed the target within the cap, and how often a correction was
    rejected."""
    import torch

    pkg = __graft_entry__.load_package()
    from fluid2d_gb300 import build_lib, learned, train_warmstart, workloads

    build_lib.build()
    info = {}
    if a.load_weights:
        params = np.load(a.load_weights).astype(np.float32)
    else:
        t0 = time.perf_counter()
        # the 32^2 coarse grid: 512^2 runs (vortex cores 1-4 % of the side) and, for the
        # evaluation's sizes, 1024^2 runs with its vortex field (cores 20-80 cells)
        half = a.samples // 2
        X1, T1, g1 = train_warmstart.generate(half, size=a.train_size, steps_per_run=100, seed=100, g=32)
        X2, T2, g2 = train_warmstart.generate(a.samples - half, size=2 * a.train_size, steps_per_run=50, seed=500,
                                              g=32, rmin=20.0, rmax=80.0, vortices=64)
        sets = [(X1, T1), (X2, T2)]
        if a.mid_solve_samples:
            # second round: states in the middle of learned solves, met with the first round's
            # network, added to the data and the network trained again from scratch
            p0, _ = train_warmstart.train_sets(sets, epochs=a.epochs, batch=128, lr=1e-3, seed=0)
            X3, T3, _ = train_warmstart.generate(a.mid_solve_samples, size=2 * a.train_size, steps_per_run=25,
                                                 seed=900, g=32, rmin=20.0, rmax=80.0, vortices=64, params=p0)
            sets.append((X3, T3))
        t1 = time.perf_counter()
        params, hist = train_warmstart.train_sets(sets, epochs=a.epochs, batch=128, lr=1e-3, seed=0)
        t2 = time.perf_counter()
        base = [train_warmstart.evaluate_loss(learned.init_params(0), X[:2048], T[:2048]) for X, T in ((X1, T1), (X2, T2))]
        fin = [train_warmstart.evaluate_loss(params, X[:2048], T[:2048]) for X, T in ((X1, T1), (X2, T2))]
        info = {"samples": [int(X1.shape[0]), int(X2.shape[0])], "train_sizes": [a.train_size, 2 * a.train_size],
                "coarse_grids": [32, 32], "gen_s": t1 - t0, "train_s": t2 - t1, "epochs": a.epochs,
                "generation_sweeps": g1["sweeps"], "loss_init": base, "loss_trained": fin,
                "loss_first_batch": hist[0], "loss_last_batch": hist[-1],
                "mid_solve_samples": a.mid_solve_samples}
        if a.weights:
            np.save(a.weights, params)
        del X1, T1, X2, T2, sets
        torch.cuda.empty_cache()
    clocks = ClockSampler(0)
    clocks.start()
    results = []
    for size in [int(x) for x in a.eval_sizes.split(",")]:
        w = workloads.vortex_field(size, seed=3, kd=a.kd, kp=a.kp)
        for tol in [float(x) for x in a.tols.split(",")]:
            row = {"size": size, "tol": tol}
            all_modes = {"zero": (pkg.FS_WARM_ZERO, None), "previous": (pkg.FS_WARM_PREVIOUS, None),
                         "learned": (pkg.FS_WARM_LEARNED, params),
                         "coarse_only": (pkg.FS_WARM_LEARNED, np.zeros_like(params))}
            modes = [(m,) + all_modes[m] for m in a.modes.split(",")]
            for mode, warm, net_params in modes:
                s = pkg.Solver(w.rows, w.cols, diffuse_iterations=a.kd, pressure_tolerance=tol,
                               pressure_max_iterations=a.max_iters, warm_start=warm, device=0, check_finite=0,
                               learned_cycles=a.cycles,
                               learned_cycle_iterations=a.coarse_cycle_iters if mode == "coarse_only" else a.cycle_iters,
                               learned_grid=a.learned_grid)
                if warm == pkg.FS_WARM_LEARNED:
                    s.set_network(net_params)
                s.upload(*w.state())
                s.upload_sources(*w.sources())
                stream = torch.cuda.ExternalStream(s.device_view().stream, device=0)
                sweeps, res, ms = [], [], 0.0
                for k in range(a.warmup + a.steps):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    s.step(w.diffusion, w.viscosity, w.dt, 1, sync=False)
                    e1.record(stream)
                    try:
                        s.sync()
                    except pkg.FluidError as e:
                        if e.code != pkg.FS_ERR_NOT_CONVERGED:
                            raise
                    st = s.stats()
                    if k >= a.warmup:
                        ms += e0.elapsed_time(e1)
                        sweeps += st["pressure_iterations_last"]
                        res += st["pressure_residual_last"]
                st = s.stats()
                row[mode] = {"ms_per_step": ms / a.steps, "sweeps_per_projection": float(np.mean(sweeps)),
                             "missed_target": int(np.sum(np.array(res) > tol)),
                             "residual_max": float(np.max(res))}
                if warm == pkg.FS_WARM_LEARNED:
                    used, fb = st["learned_used"], st["learned_fallback"]
                    row[mode]["fallback_rate"] = fb / max(1, used + fb)
                s.close()
            if "learned" in row:
                for base in ("zero", "previous", "coarse_only"):
                    if base in row:
                        key = "speedup_ms" if base == "previous" else f"speedup_vs_{base}"
                        row[key] = row[base]["ms_per_step"] / row["learned"]["ms_per_step"]
            results.append(row)
            print(json.dumps(row), flush=True)
    line = {"metric": "ms/step to relative pressure residual, learned vs previous-pressure warm start",
            "unit": "ms/step", "higher_is_better": False, "steps": a.steps, "warmup": a.warmup, "dtype": "f32",
            "data": "synthetic (seeded vortex fields)", "training": info, "results": results,
            "clocks": clocks.stop(),
            "config": {"workload": f"vortex_field {a.eval_sizes}, Kd={a.kd}, cap {a.max_iters} sweeps",
                       "network": "8 conv layers 3x3x32, BF16 tcgen05 implicit GEMM, 32x32 coarse grid",
                       "cycles": a.cycles, "cycle_iterations": a.cycle_iters or 256,
                       "coarse_only_cycle_iterations": a.coarse_cycle_iters}}
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.max_iters is None:
        a.max_iters = {"learned": 20000, "depth": 400}.get(a.workload, 2000)
    if a.warmup < 3:
        a.warmup = 3
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "small":
        run_small(a)
    elif a.workload == "batch":
        run_batch(a)
    elif a.workload == "residual":
        run_residual(a)
    elif a.workload == "learned":
        run_learned(a)
    elif a.workload == "gauss-seidel":
        run_gauss_seidel(a)
    elif a.workload == "depth":
        run_depth(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
