"""The C ABI without a GPU: every declared symbol is exported, arguments are validated
before any CUDA call, and the product fails loudly (never silently) without a device.
With a GPU (marked gpu), the C++ adapter is built and driven like the reference app."""
import ctypes as C
import pathlib
import re
import subprocess

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_symbols():
    names = set()
    for h in HEADERS:
        names |= set(re.findall(r"^FS_API\s+[\w\s\*]+?\b(fs_\w+)\s*\(", h.read_text(), flags=re.M))
    return names


def test_header_declares_api():
    names = declared_symbols()
    for must in ("fs_create", "fs_destroy", "fs_solve_host", "fs_step", "fs_upload", "fs_download"):
        assert must in names


def test_library_exports_every_declared_symbol(fluid):
    lib = C.CDLL(str(fluid.LIB_PATH))
    names = declared_symbols()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python mirror binds every one of them
    assert names <= set(fluid.SIGNATURES), names - set(fluid.SIGNATURES)


def test_config_defaults_are_the_reference_counts(fluid):
    cfg = fluid.default_config(130, 130)
    assert (cfg.diffuse_iterations, cfg.pressure_iterations, cfg.smooth) == (15, 20, 1)
    assert cfg.warm_start == fluid.FS_WARM_ZERO


def test_argument_errors_before_cuda(fluid):
    L = fluid.load()
    h = C.c_void_p()
    for rows, cols in ((2, 10), (10, 2), (0, 0), (-5, 9)):
        cfg = fluid.default_config(10, 10)
        cfg.rows, cfg.cols = rows, cols
        assert L.fs_create(C.byref(cfg), C.byref(h)) == fluid.FS_ERR_ARG
        assert L.fs_last_error()
    cfg = fluid.default_config(10, 10)
    cfg.diffuse_iterations = -1
    assert L.fs_create(C.byref(cfg), C.byref(h)) == fluid.FS_ERR_ARG
    cfg = fluid.default_config(10, 10)
    cfg.tile_rows = 96
    assert L.fs_create(C.byref(cfg), C.byref(h)) == fluid.FS_ERR_ARG
    assert L.fs_create(None, C.byref(h)) == fluid.FS_ERR_ARG
    assert L.fs_destroy(None) == fluid.FS_OK
    assert L.fs_step(None, 0.0, 0.0, 0.1, 1) == fluid.FS_ERR_ARG
    assert L.fs_solve_host(None, None, None, 0.0, None, None, None, None, 0.0, 0.1) == fluid.FS_ERR_ARG
    assert L.fs_version().startswith(b"fluid2d_gb300")


def test_no_device_fails_loudly(fluid):
    """Without a GPU the product raises; there is no CPU fallback path."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(fluid.FluidError) as e:
        fluid.FluidSolverGPU(34, 34)
    assert e.value.code in (fluid.FS_ERR_CUDA, fluid.FS_ERR_NOMEM)


def _build_adapter(tmp_path, include_dirs, extra=()):
    exe = tmp_path / "adapter"
    lib_dir = ROOT / "fluid-2d_gb300" / "lib"
    cmd = ["g++", "-std=c++14", *extra, f"-I{ROOT / 'include'}", *[f"-I{d}" for d in include_dirs],
           str(ROOT / "tests" / "adapter_main.cpp"), f"-L{lib_dir}", "-lfluid2d_gb300",
           f"-Wl,-rpath,{lib_dir}", "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe


def test_adapter_builds_against_reference_headers(fluid, tmp_path):
    from oracle import build_oracle

    ref = build_oracle.REF_SRC  # the reference checkout the oracle recipe builds from
    if not (ref / "fluid_solver.hpp").exists():
        pytest.skip("reference sources not present on this machine")
    exe = _build_adapter(tmp_path, [ref], extra=("-include", "cstddef"))
    import torch

    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == (0 if torch.cuda.is_available() else 3), r.stdout + r.stderr


@pytest.mark.gpu
def test_adapter_runs_like_the_reference_app(fluid, tmp_path):
    exe = _build_adapter(tmp_path, [ROOT / "tests" / "ref_iface"])
    for mode in ("jacobi", "gauss-seidel"):
        r = subprocess.run([str(exe), "4", mode], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "mass" in r.stdout
