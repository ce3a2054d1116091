"""The BF16 3x3 convolution of the learned warm start: tensor-core (tcgen05) kernel vs
the CUDA-core reference kernel vs torch's CPU conv2d in FP32 on the same BF16 values."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _cpu_conv(x, w, bias, skip, relu, up):
    """x: (H', W', 32) float32 (BF16-rounded), w: (32, 9, 32) [co][tap][ci] -> (H, W, 32)."""
    import torch
    import torch.nn.functional as F

    xt = torch.from_numpy(x).permute(2, 0, 1)[None]
    if up:
        xt = F.interpolate(xt, scale_factor=2, mode="nearest")
    wt = torch.from_numpy(w.reshape(32, 3, 3, 32)).permute(0, 3, 1, 2).contiguous()
    y = F.conv2d(xt.double(), wt.double(), torch.from_numpy(bias).double(), padding=1)[0].permute(1, 2, 0)
    if skip is not None:
        y = y + torch.from_numpy(skip).double()
    if relu:
        y = torch.clamp(y, min=0)
    return y.numpy()


@pytest.mark.parametrize("H,W,up,relu,skip", [(16, 16, 0, 0, 0), (12, 40, 0, 1, 1), (64, 64, 1, 1, 0),
                                              (130, 7, 0, 1, 0), (256, 256, 0, 1, 1), (96, 128, 1, 0, 1)])
def test_conv3x3_tensor_cores_match_reference(fluid, H, W, up, relu, skip):
    import torch

    L = fluid.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(H * 1000 + W + up)
    hin, win = (H // 2, W // 2) if up else (H, W)
    x = rng.standard_normal((hin, win, 32)).astype(np.float32)
    w = (rng.standard_normal((32, 9, 32)) * 0.1).astype(np.float32)
    b = rng.standard_normal(32).astype(np.float32)
    s = rng.standard_normal((H, W, 32)).astype(np.float32) if skip else None
    xb = torch.from_numpy(x).to(torch.bfloat16)
    wb = torch.from_numpy(w).to(torch.bfloat16).float().numpy()
    sb = torch.from_numpy(s).to(torch.bfloat16) if skip else None
    want = _cpu_conv(xb.float().numpy(), wb, b, sb.float().numpy() if skip else None, relu, up)
    xd, w32 = xb.to(dev), torch.from_numpy(w).to(dev)
    bd = torch.from_numpy(b).to(dev)
    sd = sb.to(dev) if skip else None
    wpk = torch.empty(32 * 288, dtype=torch.bfloat16, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    assert L.fs_conv_pack_weights(_ptr(w32), _ptr(wpk), None) == 0
    outs = {}
    for tc in (0, 1):
        yf = torch.empty((H, W, 32), dtype=torch.float32, device=dev)
        yb = torch.empty((H, W, 32), dtype=torch.bfloat16, device=dev)
        rc = L.fs_conv3x3(_ptr(xd), _ptr(wpk), _ptr(w32), _ptr(bd), _ptr(sd), _ptr(yb), _ptr(yf), H, W, H, up, relu,
                          tc, _ptr(err), None)
        assert rc == 0, L.fs_last_error()
        torch.cuda.synchronize()
        outs[tc] = (yf.cpu().numpy(), yb.float().cpu().numpy())
    assert int(err.item()) == 0
    scale = np.abs(want).max()
    for tc in (0, 1):
        yf, yb = outs[tc]
        assert np.abs(yf - want).max() <= 1e-4 * scale, (tc, np.abs(yf - want).max() / scale)
        assert np.abs(yb - want).max() <= 8e-3 * scale
    assert np.abs(outs[0][0] - outs[1][0]).max() <= 1e-4 * scale


def _cpu_wgrad(x, dz, img_h, up):
    """x: (H', W', 32), dz: (H, W, 32) float64 -> dw [co][tap][ci], db [co] (FP64)."""
    import torch
    import torch.nn.functional as F

    H, W = dz.shape[:2]
    n = H // img_h
    xt = torch.from_numpy(x).double().reshape(n, x.shape[0] // n, x.shape[1], 32).permute(0, 3, 1, 2)
    if up:
        xt = F.interpolate(xt, scale_factor=2, mode="nearest")
    cols = F.unfold(xt, 3, padding=1)  # (n, 32*9, img_h*W), rows ci*9 + tap
    d = torch.from_numpy(dz).double().reshape(n, img_h * W, 32)
    g = torch.einsum("nkp,npc->ck", cols, d)  # (co, ci*9 + tap)
    dw = g.reshape(32, 32, 9).permute(0, 2, 1).contiguous()  # [co][tap][ci]
    return dw.numpy(), d.sum(dim=(0, 1)).numpy()


@pytest.mark.parametrize("imgs,img_h,W,up", [(1, 20, 20, 0), (3, 32, 32, 0), (128, 32, 32, 0), (4, 16, 16, 1),
                                             (128, 8, 8, 0), (2, 30, 14, 1)])
def test_weight_grad_tensor_cores(fluid, imgs, img_h, W, up):
    """tcgen05 weight gradient (BF16 dz and x, FP32 accumulation) against an FP64 sum of
    the same BF16 values, and against the CUDA-core kernel (FP32 dz)."""
    import torch

    L = fluid.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(imgs * 100 + img_h + up)
    H = imgs * img_h
    hin, win = (H // 2, W // 2) if up else (H, W)
    x = torch.from_numpy(rng.standard_normal((hin, win, 32)).astype(np.float32)).to(torch.bfloat16)
    dz = rng.standard_normal((H, W, 32)).astype(np.float32)
    dzb = torch.from_numpy(dz).to(torch.bfloat16)
    want_w, want_b = _cpu_wgrad(x.float().numpy(), dzb.float().numpy(), img_h, up)
    xd, dzd, dzbd = x.to(dev), torch.from_numpy(dz).to(dev), dzb.to(dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    work = torch.empty(int(L.fs_net_weight_grad_tc_work_floats(H, W)), dtype=torch.float32, device=dev)
    dw = torch.full((32 * 288,), 0.5, dtype=torch.float32, device=dev)  # the kernel adds
    db = torch.full((32,), 0.25, dtype=torch.float32, device=dev)
    assert L.fs_net_weight_grad_tc(_ptr(dzbd), _ptr(xd), _ptr(dw), _ptr(db), _ptr(work), work.numel(), H, W, img_h,
                                   up, _ptr(err), None) == 0
    dw_ref = torch.zeros(32 * 288, dtype=torch.float32, device=dev)
    db_ref = torch.zeros(32, dtype=torch.float32, device=dev)
    assert L.fs_net_weight_grad(_ptr(dzd), _ptr(xd), _ptr(dw_ref), _ptr(db_ref), H, W, img_h, up, None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    gw = dw.cpu().numpy().reshape(32, 9, 32) - 0.5
    gb = db.cpu().numpy() - 0.25
    scale = np.abs(want_w).max()
    np.testing.assert_allclose(gw, want_w, rtol=0, atol=2e-5 * scale + 1e-6)
    np.testing.assert_allclose(gb, want_b, rtol=0, atol=2e-5 * np.abs(want_b).max() + 1e-6)
    # the CUDA-core kernel sums the FP32 dz: equal to BF16 rounding of dz
    ref_w = dw_ref.cpu().numpy().reshape(32, 9, 32)
    assert np.linalg.norm(gw - ref_w) <= 1e-2 * np.linalg.norm(ref_w)
