"""Build recipe for the oracle libraries (test infrastructure, never shipped).

* ``oracle/_build/liboracle.so`` — the CPU restatement in ``oracle/oracle.cpp``.
  Built everywhere (x86 container and Arm GPU host) with ``-ffp-contract=off`` so
  no fused multiply-add changes the reference's rounding on either machine.
* ``oracle/_ref/libref_cpu.so`` — the reference's unmodified host solver
  (``src/fluid_solver_cpu.cpp``) compiled from the reference checkout, plus the
  C shim ``oracle/ref_cpu_shim.cpp``. Built only where the checkout exists
  (``FLUID2D_REF_SRC``, default ``/root/reference/src``); it is used to generate
  and check the golden fixtures under ``tests/golden``.
* ``oracle/_ref/ref_gpu.fatbin`` — the reference's unmodified GPU solver
  (``src/fluid_solver_gpu.cu``) compiled for sm_103a as device code only. Built
  where the checkout exists; device code does not depend on the host CPU, so the
  file is usable on any GB300 host it is copied to.
* ``oracle/_build/libref_gpu_runner.so`` — ``oracle/ref_gpu_runner.cpp`` (own
  code), which loads that fatbinary with the CUDA driver API and drives the
  reference's kernels in the reference's order. Built wherever CUDA is installed.
"""
from __future__ import annotations

import os
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REF_SRC = pathlib.Path(os.environ.get("FLUID2D_REF_SRC", "/root/reference/src"))

COMMON = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(out: pathlib.Path, srcs) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(pathlib.Path(s).stat().st_mtime > t for s in srcs)


def build_oracle(force: bool = False) -> pathlib.Path:
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "liboracle.so"
    src = HERE / "oracle.cpp"
    if force or _stale(out, [src]):
        tmp = out.with_suffix(".so.tmp")
        _run(["g++", "-std=c++17", "-fopenmp", *COMMON, str(src), "-o", str(tmp)])
        os.replace(tmp, out)
    return out


def build_ref(force: bool = False) -> pathlib.Path | None:
    """Compile the reference host solver where its sources are present."""
    solver = REF_SRC / "fluid_solver_cpu.cpp"
    if not solver.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "libref_cpu.so"
    shim = HERE / "ref_cpu_shim.cpp"
    if force or _stale(out, [solver, shim]):
        tmp = out.with_suffix(".so.tmp")
        # grid.hpp uses size_t without <cstddef>; g++ 13 needs it force-included.
        _run(["g++", "-std=c++14", *COMMON, "-include", "cstddef", f"-I{REF_SRC}",
              str(solver), str(shim), "-o", str(tmp)])
        os.replace(tmp, out)
    return out


REF_GPU_FATBIN = REF_OUT / "ref_gpu.fatbin"
CUDA_HOME = pathlib.Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def build_ref_gpu(force: bool = False) -> pathlib.Path | None:
    """Compile the reference GPU solver's kernels where its sources are present."""
    solver = REF_SRC / "fluid_solver_gpu.cu"
    if not solver.exists():
        return REF_GPU_FATBIN if REF_GPU_FATBIN.exists() else None
    REF_OUT.mkdir(exist_ok=True)
    if force or _stale(REF_GPU_FATBIN, [solver]):
        tmp = REF_OUT / "ref_gpu.fatbin.tmp"
        # Default nvcc flags (FMA contraction on), as the reference's CMake build compiles it;
        # grid.hpp needs <cstddef> force-included.
        _run([str(CUDA_HOME / "bin" / "nvcc"), "-std=c++14", "-fatbin", "-gencode", "arch=compute_103a,code=sm_103a",
              "-include", "cstddef", f"-I{REF_SRC}", str(solver), "-o", str(tmp)])
        os.replace(tmp, REF_GPU_FATBIN)
    return REF_GPU_FATBIN


def build_ref_gpu_runner(force: bool = False) -> pathlib.Path | None:
    """The driver-API runner for that fatbinary (own code); None without a CUDA toolkit."""
    hdr = CUDA_HOME / "include" / "cuda.h"
    stubs = CUDA_HOME / "lib64" / "stubs"
    if not hdr.exists():
        return None
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "libref_gpu_runner.so"
    src = HERE / "ref_gpu_runner.cpp"
    if force or _stale(out, [src]):
        tmp = out.with_suffix(".so.tmp")
        _run(["g++", "-std=c++17", *COMMON, f"-I{CUDA_HOME / 'include'}", str(src), "-o", str(tmp),
              f"-L{stubs}", "-lcuda"])
        os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
    print(build_ref_gpu(force=True))
    print(build_ref_gpu_runner(force=True))
