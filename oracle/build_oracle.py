"""Build recipe for the oracle libraries (test infrastructure, never shipped).

* ``oracle/_build/liboracle.so`` — the CPU restatement in ``oracle/oracle.cpp``.
  Built everywhere (x86 container and Arm GPU host) with ``-ffp-contract=off`` so
  no fused multiply-add changes the reference's rounding on either machine.
* ``oracle/_ref/libref_cpu.so`` — the reference's unmodified host solver
  (``src/fluid_solver_cpu.cpp``) compiled from the reference checkout, plus the
  C shim ``oracle/ref_cpu_shim.cpp``. Built only where the checkout exists
  (``FLUID2D_REF_SRC``, default ``/root/reference/src``); it is used to generate
  and check the golden fixtures under ``tests/golden``.
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


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
