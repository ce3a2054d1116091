"""fluid2d_gb300 — Python host mirror of the GB300 solver step for mworchel/fluid-2d.

The reference's interface is the C++ class ``fluid_solver`` with one method,
``solve(density, density_src, diffusion_rate, u, v, u_src, v_src, viscosity, dt)``
(src/fluid_solver.hpp:16-24), implemented on the GPU by ``fluid_solver_gpu``
(src/fluid_solver_gpu.cu:222-258). :class:`FluidSolverGPU` mirrors that class over
the C ABI in ``include/fluid2d_gb300.h``: constructed with ``(rows, cols)``
including the boundary, ``solve`` updates ``density``, ``u`` and ``v`` in place.
Arrays are float32 numpy arrays of shape (rows, cols), the reference grid layout.

There is no CPU fallback: every call runs the CUDA library, and importing a handle
without the built library raises. Build it with ``build_lib.build()`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib

import numpy as np

from . import build_lib

FS_OK, FS_ERR_ARG, FS_ERR_CUDA, FS_ERR_NONFINITE, FS_ERR_NOT_CONVERGED, FS_ERR_TIMEOUT, FS_ERR_NOMEM, \
    FS_ERR_STATE = range(8)
FS_WARM_ZERO, FS_WARM_PREVIOUS, FS_WARM_LEARNED = 0, 1, 2
FS_METHOD_JACOBI, FS_METHOD_GAUSS_SEIDEL = 0, 1
STAGE_DIFFUSE_DENSITY, STAGE_ADVECT_DENSITY, STAGE_DIFFUSE_VELOCITY, STAGE_PROJECT, STAGE_ADVECT_VELOCITY = 1, 2, 3, 4, 5

LIB_PATH = build_lib.LIB


class FluidError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class fs_config(C.Structure):
    _fields_ = [("rows", C.c_int), ("cols", C.c_int), ("diffuse_iterations", C.c_int),
                ("pressure_iterations", C.c_int), ("smooth", C.c_int), ("sweeps_per_pass", C.c_int),
                ("tile_rows", C.c_int), ("use_graph", C.c_int), ("device", C.c_int), ("warm_start", C.c_int),
                ("pressure_tolerance", C.c_float), ("pressure_max_iterations", C.c_int),
                ("check_finite", C.c_int), ("capture", C.c_int), ("method", C.c_int),
                ("learned_cycles", C.c_int), ("learned_cycle_iterations", C.c_int), ("learned_grid", C.c_int),
                ("learned_defect", C.c_int)]


class fs_stats(C.Structure):
    _fields_ = [("steps", C.c_longlong), ("kernel_launches", C.c_longlong), ("launches_per_step", C.c_int),
                ("passes_per_step", C.c_int), ("sweeps_per_pass", C.c_int), ("tile_rows", C.c_int),
                ("pressure_iterations_last", C.c_int * 2), ("pressure_residual_last", C.c_double * 2),
                ("nonfinite", C.c_int), ("learned_used", C.c_longlong), ("learned_fallback", C.c_longlong)]


FS_NUM_KINDS = 6
KIND_NAMES = ("stencil", "splat", "finish", "advect", "memset", "gradient")


class fs_kernel_times(C.Structure):
    _fields_ = [("launches", C.c_int * FS_NUM_KINDS), ("ms", C.c_double * FS_NUM_KINDS),
                ("algorithmic_bytes", C.c_double * FS_NUM_KINDS), ("pass_bytes", C.c_double * FS_NUM_KINDS),
                ("branch_launches", C.c_int * FS_NUM_KINDS), ("branch_ms", C.c_double * FS_NUM_KINDS)]


class fs_device_view(C.Structure):
    _fields_ = [("density", C.c_void_p), ("u", C.c_void_p), ("v", C.c_void_p), ("density_source", C.c_void_p),
                ("u_source", C.c_void_p), ("v_source", C.c_void_p), ("rows", C.c_int), ("cols", C.c_int),
                ("pitch", C.c_int), ("stream", C.c_void_p)]


FS_SOURCE_DENSITY, FS_SOURCE_VELOCITY = 0, 1


class fs_source_event(C.Structure):
    _fields_ = [("step", C.c_int), ("kind", C.c_int), ("i", C.c_int), ("j", C.c_int), ("value", C.c_float),
                ("value2", C.c_float)]


# Every symbol the C header declares, with its ctypes signature.
_P = C.c_void_p
_F = C.c_float
_I = C.c_int
SIGNATURES = {
    "fs_config_init": (C.c_int, [C.POINTER(fs_config), _I, _I]),
    "fs_create": (C.c_int, [C.POINTER(fs_config), C.POINTER(_P)]),
    "fs_destroy": (C.c_int, [_P]),
    "fs_last_error": (C.c_char_p, []),
    "fs_solve_host": (C.c_int, [_P, _P, _P, _F, _P, _P, _P, _P, _F, _F]),
    "fs_upload": (C.c_int, [_P, _P, _P, _P]),
    "fs_upload_sources": (C.c_int, [_P, _P, _P, _P]),
    "fs_step": (C.c_int, [_P, _F, _F, _F, _I]),
    "fs_download": (C.c_int, [_P, _P, _P, _P]),
    "fs_sync": (C.c_int, [_P]),
    "fs_set_barrier_poll_limit": (C.c_int, [_P, C.c_uint]),
    "fs_get_stats": (C.c_int, [_P, C.POINTER(fs_stats)]),
    "fs_device_view_get": (C.c_int, [_P, C.POINTER(fs_device_view)]),
    "fs_stage": (C.c_int, [_P, _I, _F, _F]),
    "fs_add_density_source": (C.c_int, [_P, _I, _I, _F]),
    "fs_add_velocity_source": (C.c_int, [_P, _I, _I, _F, _F]),
    "fs_update": (C.c_int, [_P, _F, _F, _F]),
    "fs_run_script": (C.c_int, [_P, C.POINTER(fs_source_event), _I, _I, _F, _F, _F]),
    "fs_profile_step": (C.c_int, [_P, _F, _F, _F, C.POINTER(fs_kernel_times)]),
    "fs_project_noalloc": (C.c_int, [_P, _P, _P, _P, _I, _I, _I, _I, _P]),
    "fs_batch_create": (C.c_int, [C.POINTER(fs_config), _I, C.POINTER(_I), C.POINTER(_I), C.POINTER(_P)]),
    "fs_batch_destroy": (C.c_int, [_P]),
    "fs_batch_upload": (C.c_int, [_P, _I, _P, _P, _P]),
    "fs_batch_upload_sources": (C.c_int, [_P, _I, _P, _P, _P]),
    "fs_batch_step": (C.c_int, [_P, _F, _F, _F, _I]),
    "fs_batch_download": (C.c_int, [_P, _I, _P, _P, _P]),
    "fs_batch_sync": (C.c_int, [_P]),
    "fs_batch_get_stats": (C.c_int, [_P, C.POINTER(fs_stats)]),
    "fs_batch_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "fs_autotune": (C.c_int, [C.POINTER(fs_config), _F, _F, _F, _I, C.c_char_p, C.POINTER(C.c_double)]),
    "fs_batch_autotune": (C.c_int, [C.POINTER(fs_config), _I, C.POINTER(_I), C.POINTER(_I), _F, _F, _F, _I,
                                    C.c_char_p, C.POINTER(C.c_double)]),
    "fs_conv_pack_weights": (C.c_int, [_P, _P, _P]),
    "fs_conv3x3": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P, _P]),
    "fs_net_avgpool2": (C.c_int, [_P, _P, _I, _I, _P]),
    "fs_net_avgpool2_bwd": (C.c_int, [_P, _P, _I, _I, _P]),
    "fs_net_upsample2_bwd": (C.c_int, [_P, _P, _I, _I, _P]),
    "fs_net_relu_bwd": (C.c_int, [_P, _P, _P, _P, _P, C.c_longlong, _I, _P]),
    "fs_net_weight_grad": (C.c_int, [_P, _P, _P, _P, _I, _I, _I, _I, _P]),
    "fs_net_weight_grad_tc_work_floats": (C.c_longlong, [_I, _I]),
    "fs_net_infer32": (C.c_int, [_P, _P, _P, _P, _P, _I, _P, _P]),
    "fs_net_weight_grad_tc": (C.c_int, [_P, _P, _P, _P, _P, C.c_longlong, _I, _I, _I, _I, _P, _P]),
    "fs_net_flip_weights": (C.c_int, [_P, _P, _P]),
    "fs_net_mse": (C.c_int, [_P, _P, _P, _P, C.c_longlong, _P]),
    "fs_net_adam": (C.c_int, [_P, _P, _P, _P, C.c_longlong, _F, _F, _F, _F, _I, _P, _P]),
    "fs_net_restrict": (C.c_int, [_P, _P, _I, _I, _I, _I, _P, _P, _P, _P, _P]),
    "fs_net_prolong": (C.c_int, [_P, _P, _P, _I, _I, _I, _I, _P, _F, _P]),
    "fs_set_network": (C.c_int, [_P, _P, C.c_longlong]),
    "fs_capture_view": (C.c_int, [_P, _I, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    "fs_memcpy_device": (C.c_int, [_P, _P, C.c_ulonglong, _P]),
    "fs_render_density": (C.c_int, [_P, _I, _I, _I, _F, _F, _F, _P, _P]),
    "fs_render_velocity_lines": (C.c_int, [_P, _P, _I, _I, _I, _F, _F, _P, _P]),
    "fs_checkpoint_save": (C.c_int, [_P, C.c_char_p]),
    "fs_checkpoint_load": (C.c_int, [_P, C.c_char_p]),
    "fs_host_alloc": (C.c_int, [C.POINTER(_P), C.c_ulonglong]),
    "fs_host_free": (C.c_int, [_P]),
    "fs_version": (C.c_char_p, []),
    "fs_gauss_seidel_max_size": (C.c_int, [C.POINTER(C.c_int)]),
}

_lib = None


def load(path: str | pathlib.Path | None = None):
    """Load the CUDA library (raises if it has not been built). The FLUID2D_LIB
    environment variable names an alternative build of the same library."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    env = os.environ.get("FLUID2D_LIB")
    p = pathlib.Path(path) if path else (pathlib.Path(env) if env else LIB_PATH)
    if not p.exists():
        raise RuntimeError(f"fluid2d_gb300: CUDA library not built ({p}); run build_lib.build()")
    L = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


def _check(rc):
    if rc != FS_OK:
        msg = _lib.fs_last_error().decode() if _lib is not None else ""
        raise FluidError(rc, msg)


def _ptr(a: np.ndarray, writable=False):
    if a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"] or (writable and not a.flags["WRITEABLE"]):
        raise TypeError("grids must be C-contiguous float32 numpy arrays")
    return a.ctypes.data


def default_config(rows: int, cols: int, **kw) -> fs_config:
    L = load()
    cfg = fs_config()
    _check(L.fs_config_init(C.byref(cfg), rows, cols))
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise AttributeError(f"unknown config field {k}")
        setattr(cfg, k, v)
    return cfg


def autotune(rows, cols, diffusion_rate, viscosity, dt, steps=5, cache_path=None, **config) -> dict:
    """Pick tile_rows / sweeps_per_pass for this grid and sweep plan by timing steps on
    the device (fs_autotune). Returns the chosen fields and the time per step."""
    L = load()
    cfg = default_config(rows, cols, **config)
    ms = C.c_double()
    path = str(cache_path).encode() if cache_path else None
    _check(L.fs_autotune(C.byref(cfg), diffusion_rate, viscosity, dt, steps, path, C.byref(ms)))
    return {"tile_rows": cfg.tile_rows, "sweeps_per_pass": cfg.sweeps_per_pass, "ms_per_step": ms.value}


def autotune_batch(shapes, diffusion_rate, viscosity, dt, steps=3, cache_path=None, **config) -> dict:
    """Pick tile_rows / sweeps_per_pass for a batch of grids of these (rows, cols) shapes
    by timing whole batch steps on the device (fs_batch_autotune). Returns the chosen
    fields and the time per step."""
    L = load()
    cfg = default_config(3, 3, **config)
    n = len(shapes)
    rows = (C.c_int * n)(*[int(r) for r, _ in shapes])
    cols = (C.c_int * n)(*[int(c) for _, c in shapes])
    ms = C.c_double()
    path = str(cache_path).encode() if cache_path else None
    _check(L.fs_batch_autotune(C.byref(cfg), n, rows, cols, diffusion_rate, viscosity, dt, steps, path, C.byref(ms)))
    return {"tile_rows": cfg.tile_rows, "sweeps_per_pass": cfg.sweeps_per_pass, "ms_per_step": ms.value}


class Solver:
    """One grid resident on one GPU (a handle of the C ABI)."""

    def __init__(self, rows: int, cols: int, **config):
        self._lib = load()
        self.rows, self.cols = rows, cols
        self.config = default_config(rows, cols, **config)
        h = C.c_void_p()
        _check(self._lib.fs_create(C.byref(self.config), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _shape(self, *arrs):
        for a in arrs:
            if a.shape != (self.rows, self.cols):
                raise ValueError(f"grid shape {a.shape} != ({self.rows}, {self.cols})")

    def upload(self, d, u, v):
        self._shape(d, u, v)
        _check(self._lib.fs_upload(self._h, _ptr(d), _ptr(u), _ptr(v)))
        _check(self._lib.fs_sync(self._h))

    def upload_sources(self, ds, us, vs):
        self._shape(ds, us, vs)
        _check(self._lib.fs_upload_sources(self._h, _ptr(ds), _ptr(us), _ptr(vs)))
        _check(self._lib.fs_sync(self._h))

    def step(self, diffusion_rate, viscosity, dt, nsteps=1, sync=True):
        _check(self._lib.fs_step(self._h, diffusion_rate, viscosity, dt, nsteps))
        if sync:
            _check(self._lib.fs_sync(self._h))

    # ---- the reference's simulation driver (src/simulation.cpp:44-64), device-resident
    def add_density_source(self, i, j, value):
        _check(self._lib.fs_add_density_source(self._h, int(i), int(j), float(value)))

    def add_velocity_source(self, i, j, horizontal, vertical):
        _check(self._lib.fs_add_velocity_source(self._h, int(i), int(j), float(horizontal), float(vertical)))

    def update(self, diffusion_rate, viscosity, dt, sync=True):
        _check(self._lib.fs_update(self._h, diffusion_rate, viscosity, dt))
        if sync:
            _check(self._lib.fs_sync(self._h))

    def run_script(self, events, nsteps, diffusion_rate, viscosity, dt, sync=True):
        """events: sequence of (step, kind, i, j, value, value2), sorted by step."""
        arr = (fs_source_event * max(1, len(events)))(*[fs_source_event(*e) for e in events])
        _check(self._lib.fs_run_script(self._h, arr, len(events), nsteps, diffusion_rate, viscosity, dt))
        if sync:
            _check(self._lib.fs_sync(self._h))

    def stage(self, stage, rate, dt):
        _check(self._lib.fs_stage(self._h, stage, rate, dt))
        _check(self._lib.fs_sync(self._h))

    def download(self):
        d = np.empty((self.rows, self.cols), np.float32)
        u = np.empty_like(d)
        v = np.empty_like(d)
        _check(self._lib.fs_download(self._h, _ptr(d, True), _ptr(u, True), _ptr(v, True)))
        _check(self._lib.fs_sync(self._h))
        return d, u, v

    def sync(self):
        _check(self._lib.fs_sync(self._h))

    def set_barrier_poll_limit(self, polls: int):
        """Bound of the residual solve's grid-barrier wait, in polls (0 = default)."""
        _check(self._lib.fs_set_barrier_poll_limit(self._h, int(polls)))

    def solve(self, density, density_src, diffusion_rate, u, v, u_src, v_src, viscosity, dt):
        """fluid_solver::solve: one step on host grids, density/u/v updated in place."""
        self._shape(density, density_src, u, v, u_src, v_src)
        _check(self._lib.fs_solve_host(self._h, _ptr(density, True), _ptr(density_src), diffusion_rate,
                                       _ptr(u, True), _ptr(v, True), _ptr(u_src), _ptr(v_src), viscosity, dt))

    def stats(self) -> dict:
        st = fs_stats()
        _check(self._lib.fs_get_stats(self._h, C.byref(st)))
        return {"steps": st.steps, "kernel_launches": st.kernel_launches,
                "launches_per_step": st.launches_per_step, "passes_per_step": st.passes_per_step,
                "sweeps_per_pass": st.sweeps_per_pass, "tile_rows": st.tile_rows,
                "pressure_iterations_last": list(st.pressure_iterations_last),
                "pressure_residual_last": list(st.pressure_residual_last), "nonfinite": st.nonfinite,
                "learned_used": st.learned_used, "learned_fallback": st.learned_fallback}

    def profile_step(self, diffusion_rate, viscosity, dt) -> dict:
        """One eager step in the graph's shape with CUDA events around every launch on its
        own stream; per kernel kind: launches, milliseconds, per-sweep-model bytes, pass
        bytes, and the launches / milliseconds that ran on the concurrent density branch."""
        t = fs_kernel_times()
        _check(self._lib.fs_profile_step(self._h, diffusion_rate, viscosity, dt, C.byref(t)))
        return {KIND_NAMES[k]: {"launches": t.launches[k], "ms": t.ms[k], "bytes": t.algorithmic_bytes[k],
                                "pass_bytes": t.pass_bytes[k], "branch_launches": t.branch_launches[k],
                                "branch_ms": t.branch_ms[k]}
                for k in range(FS_NUM_KINDS)}

    def render_density(self, multipliers=(1.0, 1.0, 1.0)) -> np.ndarray:
        """RGBA8 image (rows, cols, 4) of the resident density (grid_to_image_kernel)."""
        v = self.device_view()
        dev = _DeviceBuffer(self.rows * self.cols * 4)
        _check(self._lib.fs_render_density(v.density, v.rows, v.cols, v.pitch, *map(float, multipliers), dev.ptr,
                                           v.stream))
        img = dev.to_host(v.stream).reshape(self.rows, self.cols, 4)
        dev.free()
        return img

    def render_velocity_lines(self, hscale: float, vscale: float) -> np.ndarray:
        """Line vertices (rows*cols*2 records of x, y, r, g, b, a, u, v) of the resident
        velocity (velocity_to_lines_kernel)."""
        v = self.device_view()
        n = self.rows * self.cols * 2
        dev = _DeviceBuffer(n * 20)
        _check(self._lib.fs_render_velocity_lines(v.u, v.v, v.rows, v.cols, v.pitch, hscale, vscale, dev.ptr, v.stream))
        raw = dev.to_host(v.stream)
        dev.free()
        return raw.view(VERTEX_DTYPE)

    def save_checkpoint(self, path):
        _check(self._lib.fs_checkpoint_save(self._h, str(path).encode()))

    def load_checkpoint(self, path):
        _check(self._lib.fs_checkpoint_load(self._h, str(path).encode()))

    def set_network(self, params: np.ndarray):
        params = np.ascontiguousarray(params, np.float32)
        _check(self._lib.fs_set_network(self._h, params.ctypes.data, params.size))

    def capture_view(self, slot: int):
        d, p0, p1 = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _check(self._lib.fs_capture_view(self._h, slot, C.byref(d), C.byref(p0), C.byref(p1)))
        return d.value, p0.value, p1.value

    def device_view(self) -> fs_device_view:
        v = fs_device_view()
        _check(self._lib.fs_device_view_get(self._h, C.byref(v)))
        return v

    @property
    def handle(self):
        return self._h


class Batch:
    """Many independent grids of uneven size stepped together (fs_batch_*)."""

    def __init__(self, shapes, **config):
        self._lib = load()
        self.shapes = [(int(r), int(c)) for r, c in shapes]
        self.config = default_config(3, 3, **config)
        n = len(self.shapes)
        rows = (C.c_int * n)(*[r for r, _ in self.shapes])
        cols = (C.c_int * n)(*[c for _, c in self.shapes])
        h = C.c_void_p()
        _check(self._lib.fs_batch_create(C.byref(self.config), n, rows, cols, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __len__(self):
        return len(self.shapes)

    def _shape(self, k, *arrs):
        for a in arrs:
            if a.shape != self.shapes[k]:
                raise ValueError(f"grid {k}: shape {a.shape} != {self.shapes[k]}")

    def upload(self, k, d, u, v):
        self._shape(k, d, u, v)
        _check(self._lib.fs_batch_upload(self._h, k, _ptr(d), _ptr(u), _ptr(v)))
        _check(self._lib.fs_batch_sync(self._h))

    def upload_sources(self, k, ds, us, vs):
        self._shape(k, ds, us, vs)
        _check(self._lib.fs_batch_upload_sources(self._h, k, _ptr(ds), _ptr(us), _ptr(vs)))
        _check(self._lib.fs_batch_sync(self._h))

    def step(self, diffusion_rate, viscosity, dt, nsteps=1, sync=True):
        _check(self._lib.fs_batch_step(self._h, diffusion_rate, viscosity, dt, nsteps))
        if sync:
            _check(self._lib.fs_batch_sync(self._h))

    def sync(self):
        _check(self._lib.fs_batch_sync(self._h))

    def download(self, k):
        r, c = self.shapes[k]
        d = np.empty((r, c), np.float32)
        u = np.empty_like(d)
        v = np.empty_like(d)
        _check(self._lib.fs_batch_download(self._h, k, _ptr(d, True), _ptr(u, True), _ptr(v, True)))
        _check(self._lib.fs_batch_sync(self._h))
        return d, u, v

    def stats(self) -> dict:
        st = fs_stats()
        _check(self._lib.fs_batch_get_stats(self._h, C.byref(st)))
        return {"steps": st.steps, "kernel_launches": st.kernel_launches,
                "launches_per_step": st.launches_per_step, "passes_per_step": st.passes_per_step,
                "sweeps_per_pass": st.sweeps_per_pass, "tile_rows": st.tile_rows}

    @property
    def stream(self):
        p = C.c_void_p()
        _check(self._lib.fs_batch_stream(self._h, C.byref(p)))
        return p.value


class FluidSolverGPU(Solver):
    """Drop-in for the reference's fluid_solver_gpu (src/fluid_solver_gpu.cuh:9-70)."""

    def __init__(self, rows: int, cols: int, **config):
        super().__init__(rows, cols, **config)


class FluidSolverGaussSeidel(Solver):
    """Drop-in for the reference's fluid_solver_cpu (src/fluid_solver_cpu.hpp:8-50) that
    runs on the GPU and returns the host solver's results bit for bit: square grids only
    (the host solver's grid reads cols as rows), 20 diffusion and 20 pressure sweeps."""

    def __init__(self, n: int, **config):
        config.setdefault("diffuse_iterations", 20)
        config.setdefault("pressure_iterations", 20)
        config.setdefault("smooth", 0)
        super().__init__(n, n, method=FS_METHOD_GAUSS_SEIDEL, **config)


def gauss_seidel_max_size() -> int:
    """Largest grid side the Gauss-Seidel method accepts on the current device."""
    n = C.c_int(0)
    _check(load().fs_gauss_seidel_max_size(C.byref(n)))
    return n.value


VERTEX_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("r", "u1"), ("g", "u1"), ("b", "u1"), ("a", "u1"),
                         ("u", "<f4"), ("v", "<f4")])


class _DeviceBuffer:
    """Raw device allocation through the CUDA runtime that the library links."""

    def __init__(self, nbytes):
        import torch

        self._t = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        self.ptr = C.c_void_p(self._t.data_ptr())

    def to_host(self, stream):
        import torch

        torch.cuda.synchronize()
        return self._t.cpu().numpy()

    def free(self):
        self._t = None


class PinnedArray:
    """A float32 (rows, cols) numpy view of page-locked host memory (fs_host_alloc)."""

    def __init__(self, rows, cols):
        self._lib = load()
        p = C.c_void_p()
        _check(self._lib.fs_host_alloc(C.byref(p), rows * cols * 4))
        self._p = p
        buf = (C.c_float * (rows * cols)).from_address(p.value)
        self.array = np.ctypeslib.as_array(buf).reshape(rows, cols)

    def free(self):
        if getattr(self, "_p", None):
            self.array = None
            self._lib.fs_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
