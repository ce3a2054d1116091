"""fs_project_noalloc — the projection for callers that cannot allocate device memory
(host frameworks that own all device memory, plug-ins handed device buffers but no
allocator, frame loops that must not allocate after start-up).

The entry point is called through the C ABI on caller-owned device buffers and its
output is checked against the handle-based projection stage (fs_stage with
FS_STAGE_PROJECT) and against the oracle's projection on the same inputs, for two
different inputs called back to back, at the tolerance the other projection tests use
(relative L-infinity 1e-6). Free device memory is checked to stay the same across calls.
This file is collected last so a failure here cannot hide the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
TOL = 1e-6


def _reference_projection(fluid, u, v, iters):
    rows, cols = u.shape
    with fluid.Solver(rows, cols, pressure_iterations=iters, device=0) as s:
        s.upload(np.zeros_like(u), u, v)
        s.stage(fluid.STAGE_PROJECT, 0.0, 0.1)
        _, pu, pv = s.download()
    return pu, pv


@pytest.mark.parametrize("rows,cols,pitch,iters", [(130, 130, 160, 20), (67, 200, 200, 40), (5, 9, 9, 7)])
def test_noalloc_projection_matches_handle_projection_twice(fluid, wl, rows, cols, pitch, iters):
    import torch

    L = fluid.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    bufs = [torch.zeros((rows, pitch), dtype=torch.float32, device=dev) for _ in range(4)]
    u_d, v_d, uo_d, vo_d = bufs
    for call, seed in enumerate((rows * 7 + 1, rows * 7 + 2)):
        _, u, v, _, _, _ = wl.random_state(rows, cols, seed, vmax=1.0)
        want_u, want_v = _reference_projection(fluid, u, v, iters)
        u_d[:, :cols].copy_(torch.from_numpy(u))
        v_d[:, :cols].copy_(torch.from_numpy(v))
        rc = L.fs_project_noalloc(u_d.data_ptr(), v_d.data_ptr(), uo_d.data_ptr(), vo_d.data_ptr(), rows, cols,
                                  pitch, iters, C.c_void_p(stream.cuda_stream))
        assert rc == fluid.FS_OK, L.fs_last_error()
        torch.cuda.synchronize(dev)
        got_u = uo_d[:, :cols].cpu().numpy()
        got_v = vo_d[:, :cols].cpu().numpy()
        assert oracle.rel_linf(got_u, want_u) <= TOL, f"call {call}"
        assert oracle.rel_linf(got_v, want_v) <= TOL, f"call {call}"
        ou, ov, _, _ = oracle.project(u, v, iters)
        assert oracle.rel_linf(got_u, ou) <= TOL, f"call {call} vs oracle"
        assert oracle.rel_linf(got_v, ov) <= TOL, f"call {call} vs oracle"


def test_noalloc_calls_leave_free_device_memory_unchanged(fluid, wl):
    import torch

    L = fluid.load()
    dev = torch.device("cuda", 0)
    rows, cols, pitch = 96, 90, 96
    bufs = [torch.zeros((rows, pitch), dtype=torch.float32, device=dev) for _ in range(4)]
    ptrs = [b.data_ptr() for b in bufs]
    # a first call does the one-time set-up (symbol lookup, kernel loading)
    assert L.fs_project_noalloc(*ptrs, rows, cols, pitch, 20, None) == fluid.FS_OK, L.fs_last_error()
    torch.cuda.synchronize(dev)
    free0, _ = torch.cuda.mem_get_info(dev)
    for _ in range(3):
        assert L.fs_project_noalloc(*ptrs, rows, cols, pitch, 20, None) == fluid.FS_OK, L.fs_last_error()
    torch.cuda.synchronize(dev)
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0


def test_noalloc_rejects_oversize_and_aliasing(fluid):
    import torch

    L = fluid.load()
    dev = torch.device("cuda", 0)
    a = torch.zeros(16, device=dev)
    p = a.data_ptr()
    # 1024 x 1025 > FS_NOALLOC_MAX_CELLS
    rc = L.fs_project_noalloc(p, p + 4, p + 8, p + 12, 1024, 1025, 1025, 20, None)
    assert rc == fluid.FS_ERR_ARG and b"FS_NOALLOC_MAX_CELLS" in L.fs_last_error()
    rc = L.fs_project_noalloc(p, p + 4, p, p + 12, 10, 10, 10, 20, None)
    assert rc == fluid.FS_ERR_ARG
    # partial overlaps (10 x 10 floats = 400 B per array): an output starting inside an
    # input's extent; nothing is launched for rejected calls
    b = torch.zeros(4 * 100 + 16, device=dev)
    q = b.data_ptr()
    rc = L.fs_project_noalloc(q, q + 400, q + 4 * 3, q + 1200, 10, 10, 10, 20, None)  # u_out = u + 3 floats
    assert rc == fluid.FS_ERR_ARG and b"overlaps" in L.fs_last_error()
    rc = L.fs_project_noalloc(q, q + 400, q + 800, q + 400 + 4 * 50, 10, 10, 10, 20, None)  # v_out inside v
    assert rc == fluid.FS_ERR_ARG
