"""Training data and training loop for the learned pressure correction.

Data: seeded random-vortex runs of the solver itself (previous-pressure warm start,
fixed sweep counts, capture on). For every projection the solver keeps the divergence
it projected, the pressure it started from and the pressure it ended with; each of the
two pressures gives one sample, so the data holds both the residuals the network sees
first in a step (of the previous step's pressure) and those it sees after a segment of
Jacobi sweeps. The exact solution p* of the same discrete Neumann problem (4p - sum of
neighbours = div on the interior, edges equal to their inner neighbour) is computed in
FP64 with the discrete cosine transform that diagonalises it; the training target is
the block-mean correction p*_c - p_c on the coarse grid, zero mean, in network units.
Inputs come from the same restriction kernel the solver runs (fs_net_restrict), so
training and inference see identical preprocessing.

Training: Adam on mean squared error, forward and backward on the project's kernels
(learned.Net). torch supplies device buffers and the FP64 DCT matrices only.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import learned as Lm

G = Lm.G


def _torch():
    import torch

    return torch


def dct_basis(n, device):
    """Orthonormal DCT-II matrix C (C @ x transforms along the first axis) and the
    eigenvalues 2 - 2cos(pi k / n) of the 1-D reflective-Neumann second difference."""
    torch = _torch()
    k = torch.arange(n, dtype=torch.float64, device=device)[:, None]
    i = torch.arange(n, dtype=torch.float64, device=device)[None, :]
    Cm = torch.cos(math.pi * k * (2 * i + 1) / (2 * n)) * math.sqrt(2.0 / n)
    Cm[0] /= math.sqrt(2.0)
    lam = 2.0 - 2.0 * torch.cos(math.pi * torch.arange(n, dtype=torch.float64, device=device) / n)
    return Cm, lam


def neumann_solve(div, Cm, lam):
    """Exact zero-mean solution of 4p - sum(nbrs) = div on an n x n interior with
    reflective edges (the fixed point of the reference's Jacobi iteration)."""
    torch = _torch()
    dh = Cm @ div @ Cm.T
    den = lam[:, None] + lam[None, :]
    den[0, 0] = 1.0
    ph = dh / den
    ph[0, 0] = 0.0
    return Cm.T @ ph @ Cm


def _view(ptr, rows, pitch, device):
    """Copy a pitched device field (rows x pitch floats at ptr) into a torch tensor."""
    torch = _torch()
    from . import load

    out = torch.empty((rows, pitch), dtype=torch.float32, device=device)
    rc = load().fs_memcpy_device(C.c_void_p(out.data_ptr()), C.c_void_p(ptr), rows * pitch * 4, None)
    if rc != 0:
        raise RuntimeError("fs_memcpy_device failed")
    return out


def generate(n_samples, size=512, steps_per_run=100, seed=100, sweeps=(64, 256, 1024), g=None, device="cuda",
             log=None, rmin=None, rmax=None, vortices=16, params=None, cycles=(2, 4, 8, 16)):
    """Returns (X [S, g, g, 32] BF16 network inputs, T [S, g, g] FP32 targets, info).
    Run k uses sweeps[k % len(sweeps)] pressure sweeps per projection; g is the coarse
    grid (default 32); vortex core radii default to size/100 .. size/25 cells.

    With `params`, the runs use the learned corrections themselves (those parameters, 128
    sweeps per cycle) stopped after cycles[k % len(cycles)] cycles, so the final pressures
    are the states the network meets in the middle of a solve."""
    torch = _torch()
    import fluid2d_gb300 as pkg
    from fluid2d_gb300 import workloads

    g = g or G
    kappa = g * g / 16.0
    L = pkg.load()
    Cm, lam = dct_basis(size, device)
    R = size // g
    rmin = size / 100.0 if rmin is None else rmin
    rmax = size / 25.0 if rmax is None else rmax
    xs, ts = [], []
    scale = torch.zeros(1, dtype=torch.float32, device=device)
    work = torch.zeros(g * g, dtype=torch.float32, device=device)
    run = 0
    t0 = time.time()
    while len(ts) < n_samples:
        kp = sweeps[run % len(sweeps)]
        w = workloads.vortex_field(size, seed=seed + run, kd=20, kp=kp, dt=0.05, rate=1e-5, vortices=vortices,
                                   rmin=rmin, rmax=rmax)
        if params is None:
            s = pkg.Solver(w.rows, w.cols, diffuse_iterations=20, pressure_iterations=kp,
                           warm_start=pkg.FS_WARM_PREVIOUS, capture=1, check_finite=0, device=0)
        else:
            k = cycles[run % len(cycles)]
            s = pkg.Solver(w.rows, w.cols, diffuse_iterations=20, warm_start=pkg.FS_WARM_LEARNED, capture=1,
                           check_finite=0, device=0, pressure_tolerance=1e-9, pressure_max_iterations=128 * k,
                           learned_cycle_iterations=128, learned_cycles=k)
            s.set_network(np.asarray(params, np.float32))
        s.upload(*w.state())
        s.upload_sources(*w.sources())
        pitch = s.device_view().pitch
        for _ in range(steps_per_run):
            try:
                s.step(w.diffusion, w.viscosity, w.dt, 1)
            except pkg.FluidError as e:
                if e.code != pkg.FS_ERR_NOT_CONVERGED:
                    raise
            for slot in (0, 1):
                dptr, sptr, fptr = s.capture_view(slot)
                div = _view(dptr, w.rows, pitch, device)[1:-1, 1:size + 1].double()
                pstar_c = neumann_solve(div, Cm, lam).reshape(g, R, g, R).mean(dim=(1, 3)).float()
                for pptr in (sptr, fptr):
                    xin = torch.zeros((g, g, 32), dtype=torch.bfloat16, device=device)
                    pc = torch.zeros((g, g), dtype=torch.float32, device=device)
                    rc = L.fs_net_restrict(C.c_void_p(dptr), C.c_void_p(pptr), w.rows, w.cols, pitch, g,
                                           C.c_void_p(work.data_ptr()), C.c_void_p(scale.data_ptr()),
                                           C.c_void_p(xin.data_ptr()), C.c_void_p(pc.data_ptr()), None)
                    if rc != 0:
                        raise RuntimeError(L.fs_last_error().decode())
                    corr = pstar_c - pc
                    corr = corr - corr.mean()
                    xs.append(xin)
                    ts.append(corr / (scale * kappa))
                if len(ts) >= n_samples:
                    break
            if len(ts) >= n_samples:
                break
        s.close()
        run += 1
        if log:
            log(f"generated {len(ts)} samples ({run} runs, {time.time() - t0:.1f} s)")
    X = torch.stack(xs[:n_samples])
    T = torch.stack(ts[:n_samples])
    return X, T, {"runs": run, "size": size, "g": g, "seconds": time.time() - t0, "sweeps": list(sweeps)}


def train(X, T, epochs=4, batch=128, lr=1e-3, seed=0, log=None):
    """Trains the network on (X, T); returns (params as numpy, loss history)."""
    return train_sets([(X, T)], epochs=epochs, batch=batch, lr=lr, seed=seed, log=log)


def train_sets(sets, epochs=4, batch=128, lr=1e-3, seed=0, log=None):
    """Trains one network on several data sets, possibly of different coarse grid sizes
    ([(X, T), ...], X [S, g, g, 32]); batches of the sets are interleaved in a seeded
    random order. Returns (params as numpy, loss history)."""
    torch = _torch()
    dev = sets[0][0].device
    params = torch.from_numpy(Lm.init_params(seed)).to(dev)
    nets = {}
    for X, _ in sets:
        g = int(X.shape[1])
        if g not in nets:
            nets[g] = Lm.Net(B=batch, params=params, g=g)
    first = next(iter(nets.values()))
    opt = Lm.Adam(first, lr=lr)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    hist = []
    for ep in range(epochs):
        order = []
        for si, (X, _) in enumerate(sets):
            perm = torch.randperm(X.shape[0], generator=gen)
            order += [(si, perm[b0:b0 + batch]) for b0 in range(0, X.shape[0] - batch + 1, batch)]
        for k in torch.randperm(len(order), generator=gen).tolist():
            si, idx = order[k]
            X, T = sets[si]
            g = int(X.shape[1])
            net = nets[g]
            net.repack()  # the shared parameters changed since this net last packed them
            idx = idx.to(dev)
            x0 = X[idx].reshape(batch * g, g, 32).contiguous()
            t = T[idx].reshape(batch * g, g).contiguous()
            net.forward(x0)
            loss, dy = Lm.mse_loss(net, t)
            grad = net.backward(x0, dy)
            opt.step(grad)
            hist.append(float(loss))
        if log:
            log(f"epoch {ep}: loss {np.mean(hist[-max(1, len(order)):]):.4e}")
    return params.cpu().numpy(), hist


def evaluate_loss(params, X, T, batch=128):
    torch = _torch()
    g = int(X.shape[1])
    net = Lm.Net(B=batch, params=torch.from_numpy(np.asarray(params, np.float32)).to(X.device), g=g)
    tot, n = 0.0, 0
    for b0 in range(0, X.shape[0] - batch + 1, batch):
        x0 = X[b0:b0 + batch].reshape(batch * g, g, 32).contiguous()
        t = T[b0:b0 + batch].reshape(batch * g, g).contiguous()
        net.forward(x0)
        loss, _ = Lm.mse_loss(net, t)
        tot += float(loss)
        n += 1
    return tot / max(n, 1)
