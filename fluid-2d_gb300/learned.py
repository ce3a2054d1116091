"""Learned pressure correction: a small convolutional network that maps the residual of
the current pressure (the divergence and the previous pressure combined) to a correction.

No counterpart in the reference (its pressure solve always starts from zero,
src/fluid_solver_gpu.cu:364). The network runs on a coarse grid of G x G cells (G = 32),
each covering an R x R block of the fine interior: its input (channel 0) is the block
SUM of the Poisson residual r = div + sum(nbrs p) - 4p of the current pressure p,
divided by the RMS of those sums (`scale`); when p is the previous step's pressure this
is the divergence and the previous pressure in one field, and when p is zero it is the
block-summed divergence. Its output (channel 0, times scale * KAPPA) is the block mean
of the correction e that solves the residual equation (4e - sum(nbrs e) = r), which is
interpolated bilinearly back to the fine grid and added to p. The coarse problem has the
same units at every fine size that G divides, so one network serves them all.

The solver corrects the previous pressure once before a fixed-count solve, and the
current pressure before every segment of Jacobi sweeps of a solve to a residual target.
Each correction offers two candidates, the network's (post-smoothed on the coarse grid)
and the coarse smoothing alone, and keeps the one that brings the pressure closest to
the solution in the A-norm, or neither. On 1024^2 and larger grids both candidates are
refined on a second, 64x64 coarse level before they reach the fine grid.

Architecture (8 conv layers, 3x3, 32 channels, BF16 operands, FP32 accumulation; two
average-pool downsamples and two nearest upsamples with additive skips):
    e1 (G) -> pool -> e2, e3 (G/2) -> pool -> b1, b2 (G/4) -> up -> d1 (+e3) (G/2)
    -> up -> d2 (+e1) (G) -> out (G, channel 0)

Every convolution, forward and backward-data, runs on the tcgen05 tensor-core kernel
(fs_conv3x3); weight gradients, pooling, losses and Adam run on the CUDA-core kernels
of net.cu. torch only provides device buffers.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

G = 32
KAPPA = G * G / 16.0
CH = 32
NPARAM_LAYER = CH * 9 * CH + CH

# name, level (0: G, 1: G/2, 2: G/4), input is upsampled, skip source, relu
LAYERS = [
    ("e1", 0, False, None, True),
    ("e2", 1, False, None, True),
    ("e3", 1, False, None, True),
    ("b1", 2, False, None, True),
    ("b2", 2, False, None, True),
    ("d1", 1, True, "e3", True),
    ("d2", 0, True, "e1", True),
    ("out", 0, False, None, False),
]
NLAYER = len(LAYERS)
NPARAM = NLAYER * NPARAM_LAYER


def _lib():
    from . import load

    return load()


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _chk(rc):
    from . import _check

    _check(rc)


def frozen_mask() -> np.ndarray:
    """Weights that stay zero: e1 reads only input channels 0-1, `out` writes only
    channel 0 (its other output rows and biases are zero)."""
    m = np.zeros(NPARAM, np.uint8)
    for li, (name, *_r) in enumerate(LAYERS):
        base = li * NPARAM_LAYER
        w = m[base:base + CH * 9 * CH].reshape(CH, 9, CH)
        b = m[base + CH * 9 * CH:base + NPARAM_LAYER]
        if name == "e1":
            w[:, :, 2:] = 1
        if name == "out":
            w[1:, :, :] = 1
            b[1:] = 1
    return m


def init_params(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    out = np.zeros(NPARAM, np.float32)
    for li, (name, *_r) in enumerate(LAYERS):
        base = li * NPARAM_LAYER
        fan_in = 9 * (2 if name == "e1" else CH)
        w = rng.standard_normal((CH, 9, CH)).astype(np.float32) * np.sqrt(2.0 / fan_in)
        if name == "out":
            w *= 0.1
        out[base:base + CH * 9 * CH] = w.ravel()
    out[frozen_mask() == 1] = 0.0
    return out


@dataclass
class Net:
    """Device-side parameters and scratch for a batch of B coarse grids."""

    B: int
    params: object  # torch float32 [NPARAM]
    g: int = G      # coarse grid side (32 or 64)

    def __post_init__(self):
        import torch

        self.torch = torch
        dev = self.params.device
        self.dev = dev
        f32, bf = torch.float32, torch.bfloat16
        self.wpk = torch.empty((NLAYER, CH * 9 * CH), dtype=bf, device=dev)
        self.wflip = torch.empty((NLAYER, CH * 9 * CH), dtype=f32, device=dev)
        self.wflip_pk = torch.empty((NLAYER, CH * 9 * CH), dtype=bf, device=dev)
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        g = self.g
        self.shapes = {0: (self.B * g, g), 1: (self.B * g // 2, g // 2), 2: (self.B * g // 4, g // 4)}
        self.act = {}
        for name, lvl, *_r in LAYERS:
            r, c = self.shapes[lvl]
            self.act[name] = torch.zeros((r, c, CH), dtype=bf, device=dev)
        self.pool1 = torch.zeros((*self.shapes[1], CH), dtype=bf, device=dev)
        self.pool2 = torch.zeros((*self.shapes[2], CH), dtype=bf, device=dev)
        self.y = torch.zeros((*self.shapes[0], CH), dtype=f32, device=dev)
        self.repack()

    def w(self, li):
        return self.params[li * NPARAM_LAYER: li * NPARAM_LAYER + CH * 9 * CH]

    def b(self, li):
        return self.params[li * NPARAM_LAYER + CH * 9 * CH: (li + 1) * NPARAM_LAYER]

    def repack(self, stream=None):
        L = _lib()
        for li in range(NLAYER):
            _chk(L.fs_conv_pack_weights(_p(self.w(li)), _p(self.wpk[li]), stream))
            _chk(L.fs_net_flip_weights(_p(self.w(li)), _p(self.wflip[li]), stream))
            _chk(L.fs_conv_pack_weights(_p(self.wflip[li]), _p(self.wflip_pk[li]), stream))

    # ------------------------------------------------------------- forward
    def forward(self, x0, stream=None, tensor_cores=True):
        """x0: BF16 [B*g, g, 32]; returns the FP32 output [B*g, g, 32] (channel 0)."""
        L = _lib()
        tc = 1 if tensor_cores else 0
        a = self.act
        names = [n for n, *_r in LAYERS]

        def conv(li, x, y, yf, lvl, up, skip, relu):
            r, c = self.shapes[lvl]
            _chk(L.fs_conv3x3(_p(x), _p(self.wpk[li]), _p(self.w(li)), _p(self.b(li)), _p(skip), _p(y), _p(yf), r, c,
                              self.g >> lvl, int(up), int(relu), tc, _p(self.err), stream))

        conv(0, x0, a["e1"], None, 0, False, None, True)
        _chk(L.fs_net_avgpool2(_p(a["e1"]), _p(self.pool1), *self.shapes[1], stream))
        conv(1, self.pool1, a["e2"], None, 1, False, None, True)
        conv(2, a["e2"], a["e3"], None, 1, False, None, True)
        _chk(L.fs_net_avgpool2(_p(a["e3"]), _p(self.pool2), *self.shapes[2], stream))
        conv(3, self.pool2, a["b1"], None, 2, False, None, True)
        conv(4, a["b1"], a["b2"], None, 2, False, None, True)
        conv(5, a["b2"], a["d1"], None, 1, True, a["e3"], True)
        conv(6, a["d1"], a["d2"], None, 0, True, a["e1"], True)
        conv(7, a["d2"], a["out"], self.y, 0, False, None, False)
        del names
        return self.y

    # ------------------------------------------------------------- backward
    def backward(self, x0, dy, stream=None, tensor_cores=True):
        """Gradient of the loss w.r.t. all parameters (FP32 [NPARAM]) given dL/dy. With
        tensor_cores the weight gradients run as tcgen05 implicit GEMMs over the pixels
        (BF16 dz), otherwise on CUDA cores (FP32 dz, the checked reference)."""
        torch = self.torch
        L = _lib()
        a = self.act
        if tensor_cores and getattr(self, "wg_work", None) is None:
            self.wg_work = torch.empty(int(L.fs_net_weight_grad_tc_work_floats(0, 0)), dtype=torch.float32,
                                       device=self.dev)
        grad = torch.zeros(NPARAM, dtype=torch.float32, device=self.dev)
        gw = lambda li: grad[li * NPARAM_LAYER: li * NPARAM_LAYER + CH * 9 * CH]
        gb = lambda li: grad[li * NPARAM_LAYER + CH * 9 * CH: (li + 1) * NPARAM_LAYER]

        def zeros(lvl):
            return torch.zeros((*self.shapes[lvl], CH), dtype=torch.float32, device=self.dev)

        def back(li, da, da2, out_act, x_in, lvl_out, up, want_dx=True):
            """ReLU backward, weight gradient and backward-data for layer li. Returns the
            gradient w.r.t. the layer input (at the input's level) and dz (skip branch)."""
            relu = LAYERS[li][4]
            r, c = self.shapes[lvl_out]
            n = r * c * CH
            dz = torch.empty((r, c, CH), dtype=torch.float32, device=self.dev)
            dzb = torch.empty((r, c, CH), dtype=torch.bfloat16, device=self.dev)
            _chk(L.fs_net_relu_bwd(_p(da), _p(da2), _p(out_act), _p(dz), _p(dzb), n, int(relu), stream))
            if tensor_cores:
                _chk(L.fs_net_weight_grad_tc(_p(dzb), _p(x_in), _p(gw(li)), _p(gb(li)), _p(self.wg_work),
                                             self.wg_work.numel(), r, c, self.g >> lvl_out, int(up), _p(self.err),
                                             stream))
            else:
                _chk(L.fs_net_weight_grad(_p(dz), _p(x_in), _p(gw(li)), _p(gb(li)), r, c, self.g >> lvl_out,
                                          int(up), stream))
            if not want_dx:
                return None, dz
            dxh = torch.empty((r, c, CH), dtype=torch.float32, device=self.dev)
            _chk(L.fs_conv3x3(_p(dzb), _p(self.wflip_pk[li]), _p(self.wflip[li]), None, None, None, _p(dxh), r, c,
                              self.g >> lvl_out, 0, 0, 1, _p(self.err), stream))
            if not up:
                return dxh, dz
            lo = zeros(lvl_out + 1)
            _chk(L.fs_net_upsample2_bwd(_p(dxh), _p(lo), *self.shapes[lvl_out + 1], stream))
            return lo, dz

        d_d2, _ = back(7, dy, None, a["out"], a["d2"], 0, False)
        d_d1, dz_d2 = back(6, d_d2, None, a["d2"], a["d1"], 0, True)       # dz_d2 -> e1 skip
        d_b2, dz_d1 = back(5, d_d1, None, a["d1"], a["b2"], 1, True)       # dz_d1 -> e3 skip
        d_b1, _ = back(4, d_b2, None, a["b2"], a["b1"], 2, False)
        d_p2, _ = back(3, d_b1, None, a["b1"], self.pool2, 2, False)
        d_e3 = zeros(1)
        _chk(L.fs_net_avgpool2_bwd(_p(d_p2), _p(d_e3), *self.shapes[1], stream))
        d_e2, _ = back(2, d_e3, dz_d1, a["e3"], a["e2"], 1, False)
        d_p1, _ = back(1, d_e2, None, a["e2"], self.pool1, 1, False)
        d_e1 = zeros(0)
        _chk(L.fs_net_avgpool2_bwd(_p(d_p1), _p(d_e1), *self.shapes[0], stream))
        back(0, d_e1, dz_d2, a["e1"], x0, 0, False, want_dx=False)
        return grad


class Adam:
    def __init__(self, net: Net, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        torch = net.torch
        self.net, self.lr, self.b1, self.b2, self.eps = net, lr, b1, b2, eps
        self.m = torch.zeros_like(net.params)
        self.v = torch.zeros_like(net.params)
        self.frozen = torch.from_numpy(frozen_mask()).to(net.dev)
        self.t = 0

    def step(self, grad, stream=None):
        self.t += 1
        _chk(_lib().fs_net_adam(_p(self.net.params), _p(grad), _p(self.m), _p(self.v), NPARAM, self.lr, self.b1, self.b2,
                                self.eps, self.t, _p(self.frozen), stream))
        self.net.repack(stream)


def mse_loss(net: Net, target, stream=None):
    """target: FP32 [B*g, g] coarse correction in network units. Returns (loss, dy)."""
    torch = net.torch
    n = net.B * net.g * net.g
    dy = torch.empty_like(net.y)
    parts = torch.empty((n + 255) // 256, dtype=torch.float32, device=net.dev)
    _chk(_lib().fs_net_mse(_p(net.y), _p(target), _p(dy), _p(parts), n, stream))
    return parts.sum() / n, dy
