"""Seeded synthetic inputs for the solver step.

The reference has no benchmark inputs of its own (its only driver is an
interactive window, src/app.cpp:92-123), so every workload here is synthetic and
seeded. One generator feeds the CUDA path, the oracle and the benchmark, so each
sees the same bytes. All arrays are float32, row-major [rows, cols] including the
1-cell boundary, like the reference's grid<float> (src/grid.hpp:60-69).

Workloads (N = interior size, n = N + 2):
  small_sources   N=128, dt 0.1, diffusion = viscosity = 1e-4, 20/20 sweeps,
                  4 Gaussian density sources (sigma 6 cells, amplitude 100) and 4
                  velocity impulses (|v| <= 5) at uniform random positions.
  vortex_field    N=2048 (or 8192), dt 0.05, rates 1e-5, 40/40 sweeps; velocity is
                  a sum of 64 Gaussian-core vortices (radius 20-80 cells,
                  circulation uniform in +-50), density is low-frequency noise in
                  [0, 1], no sources.
  batch           256 independent grids with N drawn from {64, 128, ..., 1024}.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    rows: int
    cols: int
    dt: float
    diffusion: float
    viscosity: float
    kd: int
    kp: int
    d: np.ndarray
    u: np.ndarray
    v: np.ndarray
    ds: np.ndarray
    us: np.ndarray
    vs: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def interior_cells(self) -> int:
        return (self.rows - 2) * (self.cols - 2)

    def state(self):
        return self.d.copy(), self.u.copy(), self.v.copy()

    def sources(self):
        return self.ds, self.us, self.vs


def _gauss_blobs(rows, cols, centres, sigma, amps):
    out = np.zeros((rows, cols), np.float64)
    ii = np.arange(rows, dtype=np.float64)[:, None]
    jj = np.arange(cols, dtype=np.float64)[None, :]
    for (ci, cj), a in zip(centres, amps):
        out += a * np.exp(-((ii - ci) ** 2 + (jj - cj) ** 2) / (2.0 * sigma * sigma))
    out[0, :] = out[-1, :] = 0.0
    out[:, 0] = out[:, -1] = 0.0
    return out


def reflect_boundaries(u, v):
    """Reflecting walls: normal component negated, tangential copied (edges only,
    corners untouched), the fills of fluid_solver_gpu.cu:26-54."""
    u[1:-1, 0] = -u[1:-1, 1]
    u[1:-1, -1] = -u[1:-1, -2]
    u[0, 1:-1] = u[1, 1:-1]
    u[-1, 1:-1] = u[-2, 1:-1]
    v[0, 1:-1] = -v[1, 1:-1]
    v[-1, 1:-1] = -v[-2, 1:-1]
    v[1:-1, 0] = v[1:-1, 1]
    v[1:-1, -1] = v[1:-1, -2]


def small_sources(n_interior: int = 128, seed: int = 1, kd: int = 20, kp: int = 20,
                  dt: float = 0.1, rate: float = 1e-4, blobs: int = 4) -> Workload:
    rng = np.random.default_rng(seed)
    n = n_interior + 2
    lo, hi = 1.0, float(n - 2)
    dc = rng.uniform(lo, hi, size=(blobs, 2))
    ds = _gauss_blobs(n, n, dc, 6.0, [100.0] * blobs)
    vc = rng.uniform(lo, hi, size=(blobs, 2))
    amps = []
    while len(amps) < blobs:
        a = rng.uniform(-5.0, 5.0, size=2)
        if np.hypot(a[0], a[1]) <= 5.0:
            amps.append(a)
    amps = np.array(amps)
    us = _gauss_blobs(n, n, vc, 6.0, amps[:, 0])
    vs = _gauss_blobs(n, n, vc, 6.0, amps[:, 1])
    z = np.zeros((n, n), np.float32)
    return Workload("small_sources", n, n, dt, rate, rate, kd, kp, z.copy(), z.copy(), z.copy(),
                    ds.astype(np.float32), us.astype(np.float32), vs.astype(np.float32),
                    {"seed": seed, "blobs": blobs})


def vortex_velocity(rows, cols, count, seed, rmin=20.0, rmax=80.0, gamma=50.0, dtype=np.float64):
    """Sum of Gaussian-core (Lamb-Oseen) vortices, v_theta = G/(2 pi r) (1 - exp(-r^2/R^2)),
    in cells per unit time; the displacement per step is dt0 * v cells."""
    rng = np.random.default_rng(seed)
    cy = rng.uniform(1.0, rows - 2.0, count)
    cx = rng.uniform(1.0, cols - 2.0, count)
    rad = rng.uniform(rmin, rmax, count)
    gam = rng.uniform(-gamma, gamma, count)
    u = np.zeros((rows, cols), dtype)
    v = np.zeros((rows, cols), dtype)
    ii = np.arange(rows, dtype=dtype)[:, None]
    jj = np.arange(cols, dtype=dtype)[None, :]
    for k in range(count):
        dy = ii - cy[k]
        dx = jj - cx[k]
        r2 = dx * dx + dy * dy
        r2 = np.maximum(r2, dtype(1e-12))
        f = gam[k] / (2.0 * np.pi * r2) * (-np.expm1(-r2 / (rad[k] * rad[k])))
        u -= f * dy
        v += f * dx
    u = u.astype(np.float32)
    v = v.astype(np.float32)
    reflect_boundaries(u, v)
    return u, v


def lowfreq_noise(rows, cols, seed, modes=8):
    rng = np.random.default_rng(seed)
    ii = np.arange(rows, dtype=np.float64)[:, None] / rows
    jj = np.arange(cols, dtype=np.float64)[None, :] / cols
    out = np.zeros((rows, cols), np.float64)
    for _ in range(modes):
        kx, ky = rng.integers(1, 5, size=2)
        ph = rng.uniform(0, 2 * np.pi)
        a = rng.uniform(0.2, 1.0)
        out += a * np.sin(2 * np.pi * (kx * jj + ky * ii) + ph)
    out -= out.min()
    m = out.max()
    if m > 0:
        out /= m
    return out.astype(np.float32)


def vortex_field(n_interior: int = 2048, seed: int = 2, kd: int = 40, kp: int = 40, dt: float = 0.05,
                 rate: float = 1e-5, vortices: int = 64, rmin=20.0, rmax=80.0) -> Workload:
    n = n_interior + 2
    big = n * n > 16_000_000
    u, v = vortex_velocity(n, n, vortices, seed, rmin, rmax, dtype=np.float32 if big else np.float64)
    d = lowfreq_noise(n, n, seed + 1)
    z = np.zeros((n, n), np.float32)
    return Workload("vortex_field", n, n, dt, rate, rate, kd, kp, d, u, v, z, z.copy(), z.copy(),
                    {"seed": seed, "vortices": vortices})


def batch_sizes(count=256, seed=4, choices=tuple(range(64, 1025, 64))):
    rng = np.random.default_rng(seed)
    return [int(x) for x in rng.choice(np.array(choices), size=count)]


def batch(count=256, seed=4, kd=30, kp=30, dt=0.05, rate=1e-5, sizes=None):
    """Independent simulations of uneven size, each with its own vortex field and
    density sources (vortex count and radii scaled with the grid). `sizes` (interior
    cells per side, one per grid) replaces the seeded draw of `count` sizes."""
    sims = []
    for k, N in enumerate(sizes if sizes else batch_sizes(count, seed)):
        n = N + 2
        scale = N / 2048.0
        cnt = max(2, int(round(16 * (N / 1024.0) ** 2)))
        u, v = vortex_velocity(n, n, cnt, seed * 1000 + k, max(3.0, 20 * scale * 2), max(6.0, 80 * scale * 2))
        d = lowfreq_noise(n, n, seed * 1000 + k + 500)
        rng = np.random.default_rng(seed * 7919 + k)
        ds = _gauss_blobs(n, n, rng.uniform(1, n - 2, size=(2, 2)), max(2.0, 6 * scale * 4), [100.0, 100.0])
        z = np.zeros((n, n), np.float32)
        sims.append(Workload(f"batch[{k}]", n, n, dt, rate, rate, kd, kp, d, u, v,
                             ds.astype(np.float32), z.copy(), z.copy(), {"N": N}))
    return sims


def portable_state(rows, cols, seed, coarse=32, vmax=0.2):
    """Smooth seeded fields (d in [0, 1], u and v in +-vmax, reflecting walls) that every
    host generates bit for bit: coarse uniform samples upsampled bilinearly with IEEE
    +, -, * and / only, in a fixed order (no library transcendental whose last bit may
    differ between x86 and Arm). Used where a fixture made on one machine is checked
    against inputs regenerated on another."""
    rng = np.random.default_rng(seed)
    y = np.arange(rows, dtype=np.float64) * (coarse / (rows - 1.0))
    x = np.arange(cols, dtype=np.float64) * (coarse / (cols - 1.0))
    i0 = np.minimum(np.floor(y).astype(np.int64), coarse - 1)
    j0 = np.minimum(np.floor(x).astype(np.int64), coarse - 1)
    fy = (y - i0)[:, None]
    fx = (x - j0)[None, :]

    def field(lo, hi):
        c = rng.uniform(lo, hi, size=(coarse + 1, coarse + 1))
        top = c[i0][:, j0] * (1.0 - fx) + c[i0][:, j0 + 1] * fx
        bot = c[i0 + 1][:, j0] * (1.0 - fx) + c[i0 + 1][:, j0 + 1] * fx
        return np.ascontiguousarray((top * (1.0 - fy) + bot * fy).astype(np.float32))

    d = field(0.0, 1.0)
    u = field(-vmax, vmax)
    v = field(-vmax, vmax)
    reflect_boundaries(u, v)
    return d, u, v


def random_state(rows, cols, seed, vmax=1.0):
    """Unstructured random fields for kernel-level tests (odd sizes, tile edges)."""
    rng = np.random.default_rng(seed)
    f = lambda lo, hi: rng.uniform(lo, hi, size=(rows, cols)).astype(np.float32)
    return f(0, 1), f(-vmax, vmax), f(-vmax, vmax), f(0, 10), f(-1, 1), f(-1, 1)


def drag_script(rows, cols, nsteps, seed=0, density=0.075, speed=0.05):
    """A seeded stand-in for the reference app's mouse drag (src/app.cpp:100-118): a
    manipulation point moves along a smooth random path; every step it adds `density`
    at its cell and `speed` times its unit movement direction as velocity. Returns
    events (step, kind, i, j, value, value2) sorted by step."""
    rng = np.random.default_rng(seed)
    y, x = rng.uniform(0.3, 0.7) * rows, rng.uniform(0.3, 0.7) * cols
    ang = rng.uniform(0, 2 * np.pi)
    events = []
    for k in range(nsteps):
        ang += rng.normal(0.0, 0.3)
        dy, dx = np.sin(ang), np.cos(ang)
        y = min(max(y + 0.8 * dy, 1.0), rows - 2.0)
        x = min(max(x + 0.8 * dx, 1.0), cols - 2.0)
        i, j = int(y), int(x)
        events.append((k, 0, i, j, float(density), 0.0))
        events.append((k, 1, i, j, float(speed * dx), float(speed * dy)))
    return events
