"""The learned pressure warm start: network forward and gradients (tensor-core convs and
CUDA-core weight gradients) against a CPU reference, the exact Neumann solver used for
training targets against the oracle's Jacobi, training, and the solver's learned mode."""
import pathlib

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"


def _mods():
    from fluid2d_gb300 import learned as Lm
    from fluid2d_gb300 import train_warmstart as T

    return Lm, T


def test_forward_and_gradients_match_cpu_reference(fluid):
    import torch

    Lm, _ = _mods()
    G, B = Lm.G, 2
    rng = np.random.default_rng(0)
    params = Lm.init_params(3)
    params += (rng.standard_normal(params.size) * 0.02).astype(np.float32) * (1 - Lm.frozen_mask())
    x0 = np.zeros((B, G, G, 32), np.float32)
    x0[..., :2] = rng.standard_normal((B, G, G, 2))
    x0 = torch.from_numpy(x0).to(torch.bfloat16).float().numpy()
    target = rng.standard_normal((B, G, G)).astype(np.float32)
    # CPU reference, FP64 with BF16 weights / activations
    from net_reference import cpu_forward

    y_ref, ps = cpu_forward(params, x0)
    loss = ((y_ref[..., 0] - torch.from_numpy(target).double()) ** 2).mean()
    loss.backward()
    g_ref = np.concatenate([np.concatenate([w.grad.numpy().ravel(), b.grad.numpy().ravel()]) for w, b in ps])
    # GPU
    dev = torch.device("cuda", 0)
    net = Lm.Net(B=B, params=torch.from_numpy(params).to(dev))
    xg = torch.from_numpy(x0).to(torch.bfloat16).to(dev).reshape(B * G, G, 32)
    y = net.forward(xg)
    lg, dy = Lm.mse_loss(net, torch.from_numpy(target).to(dev).reshape(B * G, G))
    grad = net.backward(xg, dy).cpu().numpy()
    assert int(net.err.item()) == 0
    y0 = y.cpu().numpy().reshape(B, G, G, 32)[..., 0]
    yr = y_ref.detach().numpy()[..., 0]
    assert np.abs(y0 - yr).max() <= 2e-2 * np.abs(yr).max()
    loss = float(loss.detach())
    assert abs(float(lg) - loss) <= 2e-2 * loss
    live = Lm.frozen_mask() == 0
    cos = np.dot(grad[live], g_ref[live]) / (np.linalg.norm(grad[live]) * np.linalg.norm(g_ref[live]))
    assert cos > 0.999, cos
    for li in range(Lm.NLAYER):
        sl = slice(li * Lm.NPARAM_LAYER, (li + 1) * Lm.NPARAM_LAYER)
        m = live[sl]
        err = np.linalg.norm(grad[sl][m] - g_ref[sl][m]) / max(np.linalg.norm(g_ref[sl][m]), 1e-30)
        assert err < 5e-2, (Lm.LAYERS[li][0], err)
    assert np.all(grad[~live] == 0.0)


def test_fused_inference_matches_layer_by_layer(fluid):
    """fs_net_infer32 (the whole network in one launch, activations in shared memory)
    gives the same output as the eight per-layer tensor-core convolutions and two pools."""
    import ctypes as C

    import torch

    Lm, _ = _mods()
    G, B = Lm.G, 3
    rng = np.random.default_rng(5)
    params = Lm.init_params(4)
    params += (rng.standard_normal(params.size) * 0.05).astype(np.float32) * (1 - Lm.frozen_mask())
    x0 = np.zeros((B, G, G, 32), np.float32)
    x0[..., :2] = rng.standard_normal((B, G, G, 2))
    dev = torch.device("cuda", 0)
    net = Lm.Net(B=B, params=torch.from_numpy(params).to(dev))
    xg = torch.from_numpy(x0).to(torch.bfloat16).to(dev).reshape(B * G, G, 32)
    want = net.forward(xg).clone()
    e1 = torch.empty_like(xg)
    got = torch.full_like(want, float("nan"))
    L = fluid.load()
    p = lambda t: C.c_void_p(t.data_ptr())
    assert L.fs_net_infer32(p(xg), p(net.wpk), p(net.params), p(e1), p(got), B, p(net.err), None) == 0
    torch.cuda.synchronize()
    assert int(net.err.item()) == 0
    w, g = want.cpu().numpy(), got.cpu().numpy()
    assert np.isfinite(g).all()
    np.testing.assert_array_equal(g, w)


def test_training_reduces_the_loss(fluid):
    _, T = _mods()
    X, Y, info = T.generate(256, size=128, steps_per_run=64, seed=7)
    assert X.shape[0] == 256 and info["runs"] >= 1
    before = T.evaluate_loss(__import__("fluid2d_gb300.learned", fromlist=["x"]).init_params(0), X, Y, batch=64)
    params, hist = T.train(X, Y, epochs=8, batch=64, lr=2e-3, seed=0)
    after = T.evaluate_loss(params, X, Y, batch=64)
    assert np.isfinite(hist).all()
    assert after < 0.5 * before, (before, after)


def test_learned_mode_keeps_parity_from_the_start_it_used(fluid, wl):
    """With the learned warm start, each projection starts from the network's guess or
    the previous pressure; given that captured start, the oracle reproduces the step."""
    Lm, _ = _mods()
    w = wl.vortex_field(64, seed=5, kd=15, kp=20, dt=0.1, rate=1e-3, vortices=6, rmin=4, rmax=12)
    d, u, v = w.state()
    with fluid.Solver(w.rows, w.cols, warm_start=fluid.FS_WARM_LEARNED, capture=1, device=0) as s:
        s.set_network(Lm.init_params(1))
        for _ in range(4):
            od, ou, ov = d.copy(), u.copy(), v.copy()
            s.solve(d, w.ds, w.diffusion, u, v, w.us, w.vs, w.viscosity, w.dt)
            starts = []
            for slot in (0, 1):
                _, sp, _ = s.capture_view(slot)
                import torch

                from fluid2d_gb300 import train_warmstart as T

                t = T._view(sp, w.rows, s.device_view().pitch, "cuda")
                starts.append(np.ascontiguousarray(t[:, :w.cols].cpu().numpy()))
            pw = [starts[0].copy(), starts[1].copy()]
            # the oracle starts each projection from the captured start pressure
            od, ou, ov = oracle.gpu_solve_ex(od, w.ds, w.diffusion, ou, ov, w.us, w.vs, w.viscosity, w.dt, 15, 20, 20,
                                             pw=pw)
            for g_, o in ((d, od), (u, ou), (v, ov)):
                assert oracle.rel_linf(g_, o) <= 1e-5
        st = s.stats()
        assert st["learned_used"] + st["learned_fallback"] == 8


def _field(fluid, ptr, rows, cols, pitch):
    from fluid2d_gb300 import train_warmstart as T

    return np.ascontiguousarray(T._view(ptr, rows, pitch, "cuda")[:, :cols].cpu().numpy())


@pytest.mark.parametrize("trained", [False, True])
def test_learned_cycles_reach_the_target_and_keep_parity(fluid, wl, trained):
    """Residual-target projections with network corrections: every projection meets the
    target (the residual of the pressure it ended with, recomputed by the oracle), and
    the step equals the oracle's step that projects with those final pressures. With
    untrained weights the acceptance rule rejects the corrections and the solve still converges."""
    Lm, T = _mods()
    if trained:
        X, Y, _ = T.generate(512, size=128, steps_per_run=32, seed=21, sweeps=(32, 128))
        params, _ = T.train(X, Y, epochs=6, batch=64, lr=2e-3, seed=0)
    else:
        params = Lm.init_params(1)
    w = wl.vortex_field(128, seed=5, kd=15, kp=20, dt=0.1, rate=1e-3, vortices=6, rmin=4, rmax=12)
    d, u, v = w.state()
    tol = 2e-2
    with fluid.Solver(w.rows, w.cols, warm_start=fluid.FS_WARM_LEARNED, capture=1, device=0,
                      pressure_tolerance=tol, pressure_max_iterations=60000, learned_cycles=3,
                      learned_cycle_iterations=64) as s:
        s.set_network(params)
        pitch = s.device_view().pitch
        for _ in range(3):
            od, ou, ov = d.copy(), u.copy(), v.copy()
            s.solve(d, w.ds, w.diffusion, u, v, w.us, w.vs, w.viscosity, w.dt)
            st = s.stats()
            assert max(st["pressure_residual_last"]) <= tol
            finals = []
            for slot in (0, 1):
                dptr, _, fptr = s.capture_view(slot)
                pf = _field(fluid, fptr, w.rows, w.cols, pitch)
                dv = _field(fluid, dptr, w.rows, w.cols, pitch)
                assert oracle.residual(pf, dv) <= tol * 1.001
                finals.append(pf)
            od, ou, ov = oracle.gpu_solve_ex(od, w.ds, w.diffusion, ou, ov, w.us, w.vs, w.viscosity, w.dt, 15, 0, 0,
                                             pw=[finals[0].copy(), finals[1].copy()])
            for g_, o in ((d, od), (u, ou), (v, ov)):
                assert oracle.rel_linf(g_, o) <= 1e-5
        st = s.stats()
        assert st["learned_used"] + st["learned_fallback"] >= 6
        if trained:
            assert st["learned_used"] >= 1


def _sweeps(fluid, w, warm, params, tol, steps=3, cap=20000):
    total = 0
    with fluid.Solver(w.rows, w.cols, diffuse_iterations=20, warm_start=warm, device=0, check_finite=0,
                      pressure_tolerance=tol, pressure_max_iterations=cap) as s:
        if params is not None:
            s.set_network(params)
        s.upload(*w.state())
        s.upload_sources(*w.sources())
        for _ in range(steps):
            s.step(w.diffusion, w.viscosity, w.dt, 1, sync=False)
            try:
                s.sync()
            except fluid.FluidError as e:
                if e.code != fluid.FS_ERR_NOT_CONVERGED:
                    raise
            total += sum(s.stats()["pressure_iterations_last"])
    return total


def test_trained_network_cuts_sweeps(fluid, wl):
    """What the trained network gains: the committed parameters (trained on the GPU by
    `bench.py --workload learned --samples 20000 --epochs 12 --weights ...` on 512^2 and
    1024^2 runs) against the previous-pressure warm start and against an all-zero
    network (coarse post-smoothing alone), on a 258^2 vortex field solved to a 5e-2
    residual."""
    params = np.load(GOLDEN / "warmstart_params.npy").astype(np.float32)
    w = wl.vortex_field(256, seed=8, kd=20, kp=20, dt=0.05, rate=1e-5, vortices=32, rmin=5, rmax=20)
    prev = _sweeps(fluid, w, fluid.FS_WARM_PREVIOUS, None, 5e-2)
    learned = _sweeps(fluid, w, fluid.FS_WARM_LEARNED, params, 5e-2)
    coarse = _sweeps(fluid, w, fluid.FS_WARM_LEARNED, np.zeros_like(params), 5e-2)
    print(f"sweeps over 3 steps: previous {prev}, learned {learned}, coarse smoothing only {coarse}")
    assert learned <= 0.5 * prev
    assert learned <= coarse


def test_learned_cycles_do_not_stall_on_small_divergence(fluid, wl):
    """1026^2 vortex field solved to 1e-3 for 4 steps with the committed parameters:
    every projection meets the target. Once the flow has been projected, the first
    projection of a step sees a small divergence; without the damped steps before each
    correction, FP32 noise in the checkerboard mode (which plain Jacobi never damps)
    held its residual at 3-5 %."""
    params = np.load(GOLDEN / "warmstart_params.npy").astype(np.float32)
    w = wl.vortex_field(1024, seed=3, kd=40, kp=40)
    with fluid.Solver(w.rows, w.cols, diffuse_iterations=40, warm_start=fluid.FS_WARM_LEARNED, device=0,
                      check_finite=0, pressure_tolerance=1e-3, pressure_max_iterations=20000) as s:
        s.set_network(params)
        s.upload(*w.state())
        s.upload_sources(*w.sources())
        for _ in range(4):
            s.step(w.diffusion, w.viscosity, w.dt, 1)  # raises FS_ERR_NOT_CONVERGED on a miss
            st = s.stats()
            assert max(st["pressure_residual_last"]) <= 1e-3
            assert max(st["pressure_iterations_last"]) < 20000


def test_defect_correction_meets_targets_below_the_fp32_floor(fluid, wl):
    """Learned residual solves to 1e-6 on a 258^2 vortex field. The pressure kept in
    FP32 alone stalls near its rounding floor (about 4 eps |p| per cell against a small,
    smooth divergence); with mixed-precision defect correction (the default) every
    projection meets the target, and the step still equals the oracle's step that
    projects with the FP32 pressure it ended with."""
    params = np.load(GOLDEN / "warmstart_params.npy").astype(np.float32)
    w = wl.vortex_field(256, seed=8, kd=20, kp=20, dt=0.05, rate=1e-5, vortices=32, rmin=5, rmax=20)
    tol = 1e-6
    outcome = {}
    for defect in (0, 1):
        d, u, v = w.state()
        missed, worst = 0, 0.0
        with fluid.Solver(w.rows, w.cols, diffuse_iterations=20, warm_start=fluid.FS_WARM_LEARNED, device=0,
                          check_finite=0, capture=1, pressure_tolerance=tol, pressure_max_iterations=20000,
                          learned_defect=defect) as s:
            s.set_network(params)
            pitch = s.device_view().pitch
            for _ in range(3):
                od, ou, ov = d.copy(), u.copy(), v.copy()
                try:
                    s.solve(d, w.ds, w.diffusion, u, v, w.us, w.vs, w.viscosity, w.dt)
                except fluid.FluidError as e:
                    if e.code != fluid.FS_ERR_NOT_CONVERGED:
                        raise
                res = s.stats()["pressure_residual_last"]
                missed += sum(r > tol for r in res)
                worst = max(worst, max(res))
                if defect:
                    finals = [_field(fluid, s.capture_view(slot)[2], w.rows, w.cols, pitch) for slot in (0, 1)]
                    od, ou, ov = oracle.gpu_solve_ex(od, w.ds, w.diffusion, ou, ov, w.us, w.vs, w.viscosity, w.dt,
                                                     20, 0, 0, pw=[finals[0].copy(), finals[1].copy()])
                    for g_, o in ((d, od), (u, ou), (v, ov)):
                        assert oracle.rel_linf(g_, o) <= 1e-5
        outcome[defect] = (missed, worst)
    print(f"relative residual at 1e-6: FP32 pressure missed {outcome[0][0]} of 6 (worst {outcome[0][1]:.2e}); "
          f"defect correction missed {outcome[1][0]} (worst {outcome[1][1]:.2e})")
    assert outcome[1][0] == 0, outcome
