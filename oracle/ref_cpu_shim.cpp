// C entry point around the reference's own host solver — TEST INFRASTRUCTURE ONLY.
//
// Compiled together with mworchel/fluid-2d src/fluid_solver_cpu.cpp, read from the
// reference checkout at build time (see oracle/build_oracle.py), into
// oracle/_ref/libref_cpu.so. It exists to pin the oracle's "cpu" semantics against
// the unmodified reference code (golden fixtures in tests/golden) and is never
// part of the product.
//
// The reference's solve() takes grid<float> objects (src/grid.hpp:8-66) and the
// abstract interface src/fluid_solver.hpp:16-24; this shim copies flat row-major
// arrays into grids, calls solve() nsteps times, and copies the state back.

#include "fluid_solver_cpu.hpp"

#include <algorithm>
#include <cstddef>

extern "C" int ref_cpu_solve(long n, float* d, const float* ds, float diff, float* u, float* v,
                             const float* us, const float* vs, float visc, float dt, int nsteps) {
    if (n < 3) return 1;
    const size_t N = (size_t)n;
    grid<float> D(N, N, 0.f), DS(N, N, 0.f), U(N, N, 0.f), V(N, N, 0.f), US(N, N, 0.f), VS(N, N, 0.f);
    std::copy(d, d + N * N, D.data());
    std::copy(ds, ds + N * N, DS.data());
    std::copy(u, u + N * N, U.data());
    std::copy(v, v + N * N, V.data());
    std::copy(us, us + N * N, US.data());
    std::copy(vs, vs + N * N, VS.data());
    fluid_solver_cpu solver;
    for (int s = 0; s < nsteps; ++s) solver.solve(D, DS, diff, U, V, US, VS, visc, dt);
    std::copy(D.data(), D.data() + N * N, d);
    std::copy(U.data(), U.data() + N * N, u);
    std::copy(V.data(), V.data() + N * N, v);
    return 0;
}
