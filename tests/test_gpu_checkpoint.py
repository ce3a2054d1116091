"""Checkpoint / resume: a run stopped, saved, reloaded into a fresh handle and resumed
matches the uninterrupted run (fields and warm-start pressures)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("warm", [0, 1])
def test_resume_matches_uninterrupted_run(fluid, wl, tmp_path, warm):
    w = wl.small_sources(64, seed=31)
    cfg = dict(warm_start=warm, device=0)
    with fluid.Solver(w.rows, w.cols, **cfg) as s:
        s.upload(*w.state())
        s.upload_sources(*w.sources())
        s.step(w.diffusion, w.viscosity, w.dt, nsteps=10)
        full = s.download()
    with fluid.Solver(w.rows, w.cols, **cfg) as s:
        s.upload(*w.state())
        s.upload_sources(*w.sources())
        s.step(w.diffusion, w.viscosity, w.dt, nsteps=6)
        s.save_checkpoint(tmp_path / "ck.bin")
    with fluid.Solver(w.rows, w.cols, **cfg) as s:
        s.load_checkpoint(tmp_path / "ck.bin")
        assert s.stats()["steps"] == 6
        s.step(w.diffusion, w.viscosity, w.dt, nsteps=4)
        resumed = s.download()
    for a, b in zip(full, resumed):
        assert oracle.rel_linf(a, b) <= 1e-6


def test_checkpoint_rejects_other_sizes(fluid, tmp_path):
    with fluid.Solver(20, 20, device=0) as s:
        s.save_checkpoint(tmp_path / "a.bin")
    with fluid.Solver(22, 22, device=0) as s:
        with pytest.raises(fluid.FluidError):
            s.load_checkpoint(tmp_path / "a.bin")
