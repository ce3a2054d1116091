"""Headless render kernels vs the oracle's restatement of the reference's two render
kernels (byte and float output compared exactly)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rows,cols", [(34, 34), (130, 130), (9, 17)])
def test_density_rgba_and_velocity_lines(fluid, wl, rows, cols):
    d, u, v, _, _, _ = wl.random_state(rows, cols, rows + cols, vmax=0.01)
    d = (d * 3.0 - 0.5).astype(np.float32)
    d[0, 0] = np.nan
    d[1, 1] = 1e9
    with fluid.Solver(rows, cols, device=0) as s:
        s.upload(d, u, v)
        img = s.render_density((255.0, 64.0, 7.5))
        lines = s.render_velocity_lines(800.0 / cols, 800.0 / rows)
    np.testing.assert_array_equal(img, oracle.render_density(d, (255.0, 64.0, 7.5)))
    want = oracle.render_velocity_lines(u, v, 800.0 / cols, 800.0 / rows)
    for f in want.dtype.names:
        np.testing.assert_array_equal(lines[f], want[f])
