"""ctypes wrappers for the oracle — TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline and
reference legs import this package, and only to check or time against it. The
product library (``fluid-2d_gb300``) never imports, links or calls anything here.

Arrays are numpy, row-major ``[rows, cols]`` including the 1-cell boundary, the
layout of the reference's ``grid<T>`` (src/grid.hpp:60-69). Every function works
on copies and returns new arrays.
"""
from __future__ import annotations

import ctypes as C
import pathlib

import numpy as np

from . import build_oracle as _b

BND_CONT, BND_OPP_H, BND_OPP_V = 0, 1, 2

_lib = None
_ref = None
_ref_gpu = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_L, _I, _F = C.c_long, C.c_int, C.c_float


def lib():
    global _lib
    if _lib is None:
        path = _b.build_oracle()
        L = C.CDLL(str(path))
        L.orc_gpu_solve_f32.argtypes = [_L, _L, _f32p, _f32p, _F, _f32p, _f32p, _f32p, _f32p, _F, _F, _I, _I, _I, _I]
        L.orc_gpu_solve_f64.argtypes = [_L, _L, _f64p, _f64p, _F, _f64p, _f64p, _f64p, _f64p, _F, _F, _I, _I, _I, _I]
        L.orc_gpu_solve_ex_f32.argtypes = [_L, _L, _f32p, _f32p, _F, _f32p, _f32p, _f32p, _f32p, _F, _F, _I, _I, _I,
                                           _I, C.c_void_p, C.c_void_p]
        L.orc_cpu_solve_f32.argtypes = [_L, _f32p, _f32p, _F, _f32p, _f32p, _f32p, _f32p, _F, _F, _I, _I, _I]
        L.orc_add_sources_f32.argtypes = [_L, _L, _f32p, _f32p, _F]
        L.orc_diffuse_f32.argtypes = [_L, _L, _f32p, _I, _F, _F, _I]
        L.orc_set_bnd_f32.argtypes = [_L, _L, _f32p, _I]
        L.orc_advect_trace_f32.argtypes = [_L, _L, _f32p, _f32p, _f32p, _F]
        L.orc_smooth_f32.argtypes = [_L, _L, _f32p]
        L.orc_advect_velocity_f32.argtypes = [_L, _L, _f32p, _f32p, _F]
        L.orc_project_f32.argtypes = [_L, _L, _f32p, _f32p, _I, C.c_void_p, C.c_void_p]
        L.orc_project_f64.argtypes = [_L, _L, _f64p, _f64p, _I, C.c_void_p, C.c_void_p]
        L.orc_residual_f32.argtypes = [_L, _L, _f32p, _f32p]
        L.orc_residual_f32.restype = C.c_double
        L.orc_residual_f64.argtypes = [_L, _L, _f64p, _f64p]
        L.orc_residual_f64.restype = C.c_double
        L.orc_set_contract.argtypes = [_I, _I]
        _lib = L
    return _lib


def ref_lib():
    """The compiled reference host solver, or None where the reference checkout is absent."""
    global _ref
    if _ref is None:
        path = _b.REF_OUT / "libref_cpu.so"
        if not path.exists():
            built = _b.build_ref()
            if built is None:
                return None
            path = built
        R = C.CDLL(str(path))
        R.ref_cpu_solve.argtypes = [_L, _f32p, _f32p, _F, _f32p, _f32p, _f32p, _f32p, _F, _F, _I]
        _ref = R
    return _ref


def ref_gpu_lib():
    """The reference's own GPU kernels (oracle/_ref/ref_gpu.fatbin, compiled from the
    reference's src/fluid_solver_gpu.cu) behind oracle/ref_gpu_runner.cpp, or None
    where the fatbinary or a CUDA driver is absent. Needs a GPU to load."""
    global _ref_gpu
    if _ref_gpu is None:
        fat = _b.build_ref_gpu()
        runner = _b.build_ref_gpu_runner()
        if fat is None or runner is None or not fat.exists():
            return None
        try:
            R = C.CDLL(str(runner))
        except OSError:
            return None
        R.ref_gpu_last_error.restype = C.c_char_p
        R.ref_gpu_load.argtypes = [C.c_char_p]
        R.ref_gpu_solve.argtypes = [_L, _L, _f32p, _f32p, _F, _f32p, _f32p, _f32p, _f32p, _F, _F, _I, _I, _I]
        R.ref_gpu_stage.argtypes = [_I, _L, _L, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, _I, _F, _F, _I]
        if R.ref_gpu_load(str(fat).encode()) != 0:
            raise RuntimeError("reference GPU kernels failed to load: " + R.ref_gpu_last_error().decode())
        _ref_gpu = R
    return _ref_gpu


def ref_gpu_solve(d, ds, diff, u, v, us, vs, visc, dt, kd=15, kp=20, nsteps=1):
    """The reference's GPU solver step (src/fluid_solver_gpu.cu:222-258) run by its own
    compiled kernels, nsteps times with constant sources. The reference hard-codes
    kd = 15, kp = 20; other counts run the same kernels with the given sweep counts."""
    R = ref_gpu_lib()
    if R is None:
        raise RuntimeError("compiled reference GPU kernels unavailable")
    d, ds, u, v, us, vs = (_c(a) for a in (d, ds, u, v, us, vs))
    if R.ref_gpu_solve(d.shape[0], d.shape[1], d, ds, diff, u, v, us, vs, visc, dt, kd, kp, nsteps) != 0:
        raise RuntimeError("reference GPU solve failed: " + R.ref_gpu_last_error().decode())
    return d, u, v


def set_contract(contract, bilinear=-1):
    """Multiply-add fusion of the "gpu" restatement: contract=1 fuses where the
    reference's compiled kernels fuse, with `bilinear` selecting the gather's pattern
    (see oracle.cpp); contract=0 rounds every product and sum separately."""
    lib().orc_set_contract(int(contract), int(bilinear))


REF_ADD_SOURCES, REF_DIFFUSE, REF_ADVECT_TRACE, REF_SMOOTH, REF_ADVECT, REF_PROJECT = range(6)


def ref_gpu_stage(stage, x=None, src=None, u=None, v=None, mode=0, rate=0.0, dt=0.0, iters=0):
    """One helper of the reference's GPU solver (add_sources, diffuse, advect(trace),
    smooth, advect, project; src/fluid_solver_gpu.cu:278-404) run by its own compiled
    kernels. Returns the updated x, or (u, v) for project."""
    R = ref_gpu_lib()
    if R is None:
        raise RuntimeError("compiled reference GPU kernels unavailable")
    arrs = [None if a is None else _c(a) for a in (x, src, u, v)]
    shape = next(a.shape for a in arrs if a is not None)
    ptr = lambda a: None if a is None else a.ctypes.data
    if R.ref_gpu_stage(stage, shape[0], shape[1], *map(ptr, arrs), mode, rate, dt, iters) != 0:
        raise RuntimeError("reference GPU stage failed: " + R.ref_gpu_last_error().decode())
    return (arrs[2], arrs[3]) if stage == REF_PROJECT else arrs[0]


def _c(a, dt=np.float32):
    return np.ascontiguousarray(a, dtype=dt).copy()


def _chk(rc):
    if rc != 0:
        raise ValueError("oracle rejected its arguments")


# ---------------------------------------------------------------- whole steps

def gpu_solve(d, ds, diff, u, v, us, vs, visc, dt, kd=15, kp=20, smooth=True, nsteps=1, f64=False):
    """fluid_solver_gpu::solve semantics (fluid_solver_gpu.cu:222-258), nsteps times."""
    t = np.float64 if f64 else np.float32
    d, ds, u, v, us, vs = (_c(a, t) for a in (d, ds, u, v, us, vs))
    fn = lib().orc_gpu_solve_f64 if f64 else lib().orc_gpu_solve_f32
    _chk(fn(d.shape[0], d.shape[1], d, ds, diff, u, v, us, vs, visc, dt, kd, kp, int(smooth), nsteps))
    return d, u, v


def gpu_solve_ex(d, ds, diff, u, v, us, vs, visc, dt, kd, kp1, kp2, smooth=True, pw=None):
    """One step with separate sweep counts for the two projections. pw = [p1, p2]
    float32 arrays used as starting pressures and overwritten with the final ones
    (previous-pressure warm start); None starts both from zero."""
    d, ds, u, v, us, vs = (_c(a) for a in (d, ds, u, v, us, vs))
    p1 = pw[0].ctypes.data if pw is not None else None
    p2 = pw[1].ctypes.data if pw is not None else None
    if pw is not None:
        for a in pw:
            assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"] and a.shape == d.shape
    _chk(lib().orc_gpu_solve_ex_f32(d.shape[0], d.shape[1], d, ds, diff, u, v, us, vs, visc, dt, kd, kp1, kp2,
                                    int(smooth), p1, p2))
    return d, u, v


def cpu_solve(d, ds, diff, u, v, us, vs, visc, dt, kd=20, kp=20, nsteps=1):
    """fluid_solver_cpu::solve semantics (fluid_solver_cpu.cpp:6-31), nsteps times."""
    d, ds, u, v, us, vs = (_c(a) for a in (d, ds, u, v, us, vs))
    _chk(lib().orc_cpu_solve_f32(d.shape[0], d, ds, diff, u, v, us, vs, visc, dt, kd, kp, nsteps))
    return d, u, v


def ref_cpu_solve(d, ds, diff, u, v, us, vs, visc, dt, nsteps=1):
    """The compiled reference host solver itself (20/20 Gauss-Seidel sweeps)."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference sources not present; compiled reference unavailable")
    d, ds, u, v, us, vs = (_c(a) for a in (d, ds, u, v, us, vs))
    _chk(R.ref_cpu_solve(d.shape[0], d, ds, diff, u, v, us, vs, visc, dt, nsteps))
    return d, u, v


# ---------------------------------------------------------------- single stages

def add_sources(x, s, dt):
    x, s = _c(x), _c(s)
    _chk(lib().orc_add_sources_f32(x.shape[0], x.shape[1], x, s, dt))
    return x


def set_bnd(x, mode):
    x = _c(x)
    _chk(lib().orc_set_bnd_f32(x.shape[0], x.shape[1], x, mode))
    return x


def diffuse(x, mode, rate, dt, iters):
    x = _c(x)
    _chk(lib().orc_diffuse_f32(x.shape[0], x.shape[1], x, mode, rate, dt, iters))
    return x


def advect_trace(d, u, v, dt):
    d, u, v = _c(d), _c(u), _c(v)
    _chk(lib().orc_advect_trace_f32(d.shape[0], d.shape[1], d, u, v, dt))
    return d


def smooth(d):
    d = _c(d)
    _chk(lib().orc_smooth_f32(d.shape[0], d.shape[1], d))
    return d


def advect_velocity(u, v, dt):
    u, v = _c(u), _c(v)
    _chk(lib().orc_advect_velocity_f32(u.shape[0], u.shape[1], u, v, dt))
    return u, v


def project(u, v, iters, p0=None, f64=False):
    """Returns (u, v, p, div). p0 is the starting pressure (zero when None)."""
    t = np.float64 if f64 else np.float32
    u, v = _c(u, t), _c(v, t)
    p = _c(p0, t) if p0 is not None else np.zeros_like(u)
    dv = np.zeros_like(u)
    fn = lib().orc_project_f64 if f64 else lib().orc_project_f32
    _chk(fn(u.shape[0], u.shape[1], u, v, iters, p.ctypes.data, dv.ctypes.data))
    return u, v, p, dv


def residual(p, div):
    """Relative Poisson residual ||div + sum(nbrs) - 4p|| / ||div|| over the interior."""
    if p.dtype == np.float64:
        return lib().orc_residual_f64(p.shape[0], p.shape[1], _c(p, np.float64), _c(div, np.float64))
    return lib().orc_residual_f32(p.shape[0], p.shape[1], _c(p), _c(div))


def rel_linf(x, y, skip_corners=True):
    """max|x - y| / max|y| over all cells, the four corners excluded by default."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    m = np.ones(x.shape, bool)
    if skip_corners:
        m[0, 0] = m[0, -1] = m[-1, 0] = m[-1, -1] = False
    den = np.max(np.abs(y[m])) if m.any() else 0.0
    num = np.max(np.abs(x[m] - y[m])) if m.any() else 0.0
    if den == 0.0:
        return float(num)
    return float(num / den)


# ---------------------------------------------------------------- render kernels

def render_density(d, multipliers):
    """grid_to_image_kernel (src/density_grid_renderer.cu:10-29): per channel
    uint8(max(0, min(255, m * d))) truncating toward zero, alpha 255; NaN -> 255."""
    d = np.asarray(d, np.float32)
    out = np.empty(d.shape + (4,), np.uint8)
    for c, m in enumerate(multipliers):
        x = np.float32(m) * d
        x = np.where(np.isnan(x), np.float32(255.0), np.minimum(np.float32(255.0), x))
        out[..., c] = np.maximum(np.float32(0.0), x).astype(np.uint8)
    out[..., 3] = 255
    return out


def render_velocity_lines(u, v, hscale, vscale):
    """velocity_to_lines_kernel (src/velocity_grid_renderer.cu:8-44): (rows*cols*2)
    vertices (x, y, r, g, b, a, u, v) in float32/uint8, row-major, start then end."""
    u = np.asarray(u, np.float32)
    v = np.asarray(v, np.float32)
    rows, cols = u.shape
    ii, jj = np.meshgrid(np.arange(rows, dtype=np.float32), np.arange(cols, dtype=np.float32), indexing="ij")
    sx = jj * np.float32(hscale)
    sy = ii * np.float32(vscale)
    norm = np.sqrt(np.float32(rows * cols))
    mark = (np.arange(rows)[:, None] % 8 == 0) & (np.arange(cols)[None, :] % 8 == 0)
    ex = np.where(mark, sx + (np.float32(250000.0) * u) / norm, sx).astype(np.float32)
    ey = np.where(mark, sy + (np.float32(250000.0) * v) / norm, sy).astype(np.float32)
    dt = np.dtype([("x", "<f4"), ("y", "<f4"), ("r", "u1"), ("g", "u1"), ("b", "u1"), ("a", "u1"),
                   ("u", "<f4"), ("v", "<f4")])
    out = np.zeros(rows * cols * 2, dt)
    out["x"][0::2], out["y"][0::2] = sx.ravel(), sy.ravel()
    out["x"][1::2], out["y"][1::2] = ex.ravel(), ey.ravel()
    for c in "rgba":
        out[c] = 255
    return out


def script_sources(shape, events, k, step):
    """Source grids of one step of a scripted run: the events of `step` (starting at
    index k) added to zeroed grids in order, source(i, j) += value * width * height in
    float32 (src/simulation.cpp:44-51). Returns (ds, us, vs, next k)."""
    rows, cols = shape
    w, h = np.float32(cols), np.float32(rows)
    ds = np.zeros(shape, np.float32)
    us = np.zeros(shape, np.float32)
    vs = np.zeros(shape, np.float32)
    while k < len(events) and events[k][0] == step:
        _, kind, i, j, a, b = events[k]
        if kind == 0:
            ds[i, j] = np.float32(ds[i, j] + np.float32(np.float32(np.float32(a) * w) * h))
        else:
            us[i, j] = np.float32(us[i, j] + np.float32(np.float32(np.float32(a) * w) * h))
            vs[i, j] = np.float32(vs[i, j] + np.float32(np.float32(np.float32(b) * w) * h))
        k += 1
    return ds, us, vs, k


def simulation_run(d, u, v, events, nsteps, diff, visc, dt, kd=15, kp=20, smooth=True):
    """The reference's simulation driver around the GPU-semantics step: before step k
    the events of step k are added to zeroed source grids in order, source(i, j) +=
    value * width * height in float32 (src/simulation.cpp:44-51), then the step runs and
    the sources are cleared (src/simulation.cpp:53-64). events: (step, kind, i, j,
    value, value2), kind 0 = density, 1 = velocity."""
    d, u, v = (_c(a) for a in (d, u, v))
    k = 0
    for step in range(nsteps):
        ds, us, vs, k = script_sources(d.shape, events, k, step)
        d, u, v = gpu_solve(d, ds, diff, u, v, us, vs, visc, dt, kd=kd, kp=kp, smooth=smooth)
    return d, u, v
