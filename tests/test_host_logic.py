"""Host-side logic that needs no GPU: the exact Neumann solve behind the training
targets, the network's parameter layout, the driver oracle and the scripted sources."""
import numpy as np
import pytest

import oracle


def _T():
    from fluid2d_gb300 import train_warmstart as T

    return T


def test_exact_neumann_solve_is_the_jacobi_fixed_point(wl):
    """The DCT solve used for training targets equals the oracle's Jacobi run to
    convergence (FP64) on the same divergence, up to the constant null space."""
    torch = pytest.importorskip("torch")
    T = _T()
    n = 24
    _, u, v, _, _, _ = wl.random_state(n + 2, n + 2, 9, vmax=1.0)
    wl.reflect_boundaries(u, v)
    _, _, p_jac, div = oracle.project(u, v, 30000, f64=True)
    Cm, lam = T.dct_basis(n, "cpu")
    p = T.neumann_solve(torch.from_numpy(div[1:-1, 1:-1]), Cm, lam).numpy()
    pj = p_jac[1:-1, 1:-1] - p_jac[1:-1, 1:-1].mean()
    assert np.abs(p - pj).max() <= 1e-6 * np.abs(pj).max()


def test_dct_basis_is_orthonormal():
    torch = pytest.importorskip("torch")
    Cm, lam = _T().dct_basis(16, "cpu")
    np.testing.assert_allclose((Cm @ Cm.T).numpy(), np.eye(16), atol=1e-12)
    assert float(lam[0]) == 0.0 and bool((lam[1:] > 0).all())


def test_network_parameter_layout():
    from fluid2d_gb300 import learned as Lm

    assert Lm.NPARAM == 8 * (32 * 9 * 32 + 32)
    p = Lm.init_params(0)
    assert p.shape == (Lm.NPARAM,) and p.dtype == np.float32
    # frozen weights stay zero: e1 reads only the two input channels, `out` writes channel 0
    assert not p[Lm.frozen_mask() == 1].any()
    assert Lm.NPARAM == 73984


def test_driver_oracle_applies_events_in_order(wl):
    """simulation.cpp:44-51 restated: value * width * height added per event, in order,
    in float32; events of later steps wait for their step."""
    n = 10
    z = np.zeros((n, n), np.float32)
    ev = [(0, 0, 4, 5, 0.1, 0.0), (0, 0, 4, 5, 0.2, 0.0), (1, 1, 3, 3, 0.05, -0.05)]
    d1, u1, v1 = oracle.simulation_run(z, z, z, ev, 1, 0.0, 0.0, 0.1)
    ds = np.zeros_like(z)
    w, h = np.float32(n), np.float32(n)
    ds[4, 5] = np.float32(np.float32(np.float32(np.float32(0.1) * w) * h) + np.float32(np.float32(np.float32(0.2) * w) * h))
    want = oracle.gpu_solve(z, ds, 0.0, z, z, z, z, 0.0, 0.1)
    for a, b in zip((d1, u1, v1), want):
        np.testing.assert_array_equal(a, b)


def test_drag_script_is_seeded_sorted_and_inside(wl):
    a = wl.drag_script(66, 80, 50, seed=3)
    b = wl.drag_script(66, 80, 50, seed=3)
    assert a == b and a != wl.drag_script(66, 80, 50, seed=4)
    steps = [e[0] for e in a]
    assert steps == sorted(steps) and len(a) == 100
    for step, kind, i, j, x, y in a:
        assert 1 <= i <= 64 and 1 <= j <= 78 and kind in (0, 1)
        if kind == 1:
            assert abs(np.hypot(x, y) - 0.05) < 1e-6


def test_batch_workload_sizes(wl):
    """The batch workload draws its seeded sizes from 64..1024 in steps of 64, or takes
    explicit interior sizes (bench.py --batch-sizes), one grid each, boundary added."""
    drawn = wl.batch_sizes(256, seed=4)
    assert len(drawn) == 256 and set(drawn) <= set(range(64, 1025, 64))
    assert drawn == wl.batch_sizes(256, seed=4)
    sims = wl.batch(sizes=[64, 30], kd=30, kp=30)
    assert [(w.rows, w.cols) for w in sims] == [(66, 66), (32, 32)]
    for w in sims:
        d, u, v = w.state()
        assert d.dtype == np.float32 and d.shape == (w.rows, w.cols)
        assert np.isfinite(u).all() and np.isfinite(v).all()
