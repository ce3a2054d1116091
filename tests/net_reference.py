"""FP64 CPU reference of the learned warm start's network (test helper).

The network (8 layers of 3x3 convolutions, 32 channels, two average-pool downsamples
and two nearest upsamples with additive skips) restated in torch on the CPU with FP64
arithmetic, BF16-rounded weights and BF16 rounding of every stored activation, as the
GPU kernels store them. The GPU forward and the gradients of its backward kernels are
checked against this (tests/test_gpu_learned.py). Not part of the product.
"""
import numpy as np

from fluid2d_gb300 import learned as Lm


def cpu_forward(params: np.ndarray, x0: np.ndarray):
    """The same network in torch on the CPU, FP64, with BF16-rounded weights and BF16
    rounding of every stored activation (as the GPU stores them). x0: [B, G, G, 32].
    Returns (y [B, G, G, 32], list of parameter tensors requiring grad)."""
    import torch
    import torch.nn.functional as F

    def bf(t):
        return t.to(torch.bfloat16).to(torch.float64)

    ps = []
    xs = torch.from_numpy(x0).permute(0, 3, 1, 2).to(torch.float64)

    CH, NL = Lm.CH, Lm.NPARAM_LAYER

    def conv(li, x, up, skip, relu):
        w = torch.from_numpy(params[li * NL: li * NL + CH * 9 * CH].copy()).reshape(CH, 9, CH)
        b = torch.from_numpy(params[li * NL + CH * 9 * CH:(li + 1) * NL].copy())
        w = w.to(torch.float64).requires_grad_(True)
        b = b.to(torch.float64).requires_grad_(True)
        ps.append((w, b))
        wk = bf(w).reshape(CH, 3, 3, CH).permute(0, 3, 1, 2)
        if up:
            x = F.interpolate(x, scale_factor=2, mode="nearest")
        y = F.conv2d(x, wk, b, padding=1)
        if skip is not None:
            y = y + skip
        if relu:
            y = torch.clamp(y, min=0)
        return y

    q = lambda t: t + (bf(t) - t).detach()  # BF16 storage rounding, straight-through
    e1 = q(conv(0, xs, False, None, True))
    p1 = q(F.avg_pool2d(e1, 2))
    e2 = q(conv(1, p1, False, None, True))
    e3 = q(conv(2, e2, False, None, True))
    p2 = q(F.avg_pool2d(e3, 2))
    b1 = q(conv(3, p2, False, None, True))
    b2 = q(conv(4, b1, False, None, True))
    d1 = q(conv(5, b2, True, e3, True))
    d2 = q(conv(6, d1, True, e1, True))
    y = conv(7, d2, False, None, False)
    return y.permute(0, 2, 3, 1), ps
