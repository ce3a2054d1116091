"""The learned pressure warm start: network forward and gradients (tensor-core convs and
CUDA-core weight gradients) against a CPU reference, the exact Neumann solver used for
training targets against the oracle's Jacobi, training, and the solver's learned mode."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


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
    y_ref, ps = Lm.cpu_forward(params, x0)
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
    assert abs(float(lg) - float(loss)) <= 2e-2 * float(loss)
    live = Lm.frozen_mask() == 0
    cos = np.dot(grad[live], g_ref[live]) / (np.linalg.norm(grad[live]) * np.linalg.norm(g_ref[live]))
    assert cos > 0.999, cos
    for li in range(Lm.NLAYER):
        sl = slice(li * Lm.NPARAM_LAYER, (li + 1) * Lm.NPARAM_LAYER)
        m = live[sl]
        err = np.linalg.norm(grad[sl][m] - g_ref[sl][m]) / max(np.linalg.norm(g_ref[sl][m]), 1e-30)
        assert err < 5e-2, (Lm.LAYERS[li][0], err)
    assert np.all(grad[~live] == 0.0)


def test_exact_neumann_solve_is_the_jacobi_fixed_point(wl):
    import torch

    _, T = _mods()
    n = 24
    _, u, v, _, _, _ = wl.random_state(n + 2, n + 2, 9, vmax=1.0)
    wl.reflect_boundaries(u, v)
    _, _, p_jac, div = oracle.project(u, v, 30000, f64=True)
    Cm, lam = T.dct_basis(n, "cpu")
    p = T.neumann_solve(torch.from_numpy(div[1:-1, 1:-1]), Cm, lam).numpy()
    pj = p_jac[1:-1, 1:-1] - p_jac[1:-1, 1:-1].mean()
    assert np.abs(p - pj).max() <= 1e-6 * np.abs(pj).max()


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
