// Oracle for the fluid-2d solver step — TEST INFRASTRUCTURE ONLY.
//
// This file is the CPU restatement that the CUDA path is checked against. Only the
// tests, the smoke check and bench.py's CPU-baseline / reference legs may load it;
// the product library never links or calls it.
//
// Two semantics are restated, both sequentially and with -ffp-contract=off so that
// every float operation happens in the order the reference source writes it, and fused
// multiply-adds only where written out (std::fma):
//
//  * "gpu" semantics (oracle B): mworchel/fluid-2d src/fluid_solver_gpu.cu, the
//    reference's CUDA solver. Jacobi sweeps, boundary fills that never write the
//    four corners, the double-precision diffusion divisor, density smoothing after
//    the forward (splat) advection, and the multiply-add fusions of the compiled
//    kernels (see "contractions" below). The reference hard-codes 15 diffusion and 20
//    pressure sweeps; here both counts are parameters. Pinned against the reference's
//    own compiled kernels by the ref_gpu_* fixtures in tests/golden.
//  * "cpu" semantics: src/fluid_solver_cpu.cpp, the reference's single-threaded
//    host solver. In-place (lexicographic Gauss-Seidel) sweeps, corner averaging,
//    float divisor, no smoothing. Pinned bit-exactly against the compiled reference
//    by the golden fixtures in tests/golden.
//
// Layout: row-major [rows][cols], element (i, j) at i*cols + j, exactly the
// reference's grid<T> (src/grid.hpp:60-69). Rows/cols include the 1-cell boundary.
//
// Every function is instantiated for float (the reference precision) and double
// (the FP64 rerun used to state drift). In the double instantiation the float
// literals of the reference (0.2f, 0.5f, ...) are kept as written.

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

enum Bnd { BND_CONT = 0, BND_OPP_H = 1, BND_OPP_V = 2 };

// ---------------------------------------------------------------- contractions
// nvcc compiles the reference's kernels with multiply-add contraction on (its default,
// --fmad=true): where the source writes a*b + c the compiled kernel computes
// fma(a, b, c), one rounding instead of two. The "gpu" restatement fuses the same
// operations (`g_contract` = 1): add_sources (x + dt*s), the diffusion numerator
// (x0 + a*sum), both advections' positions (j +- dt0*u) and the gather's bilinear sum,
// where several fusions are possible and `g_bilinear` picks one:
//   -1  no fusion;  bits 0 / 1: which product of the top / bottom row sum is fused
//   (0: fma(s1, A, s0*B), 1: fma(s0, B, s1*A)); bit 2: which row of the outer sum
//   (0: fma(s3, top, s2*bot), 1: fma(s2, bot, s3*top)).
// The defaults were fixed by running the reference's own compiled kernels
// (oracle/ref_gpu_runner.cpp) on random inputs and comparing stage by stage: with
// g_contract = 1 and g_bilinear = 3, add_sources, diffuse, smooth, the gather advection
// and project match bit for bit at 130^2 and 1026^2, and the splat to within the
// ordering of its atomics; with g_contract = 0 the gather differs by 1.1e-4 relative at
// 1026^2 (the unfused position j - dt0*u rounds at ulp(j)). g_contract = 0 gives the
// source's plain two-rounding arithmetic.
int g_contract = 1;
int g_bilinear = 3;

template <class T> inline T madd(T a, T b, T c) { return g_contract ? std::fma(a, b, c) : a * b + c; }

template <class T> inline T bilinear(T s0, T s1, T s2, T s3, T A, T B, T C, T D) {
    const int m = g_contract ? g_bilinear : -1;
    if (m < 0) {
        T top = s1 * A + s0 * B;
        T bot = s1 * C + s0 * D;
        return s3 * top + s2 * bot;
    }
    const T top = (m & 1) ? std::fma(s0, B, s1 * A) : std::fma(s1, A, s0 * B);
    const T bot = (m & 2) ? std::fma(s0, D, s1 * C) : std::fma(s1, C, s0 * D);
    return (m & 4) ? std::fma(s2, bot, s3 * top) : std::fma(s3, top, s2 * bot);
}

template <class T> struct Field {
    T* p;
    long rows, cols;
    T& operator()(long i, long j) const { return p[i * cols + j]; }
};

// ---------------------------------------------------------------- gpu semantics

// set_boundary_{continuous,opposite_horizontal,opposite_vertical}_kernel,
// fluid_solver_gpu.cu:11-54. Edges copy (or negate) the inner neighbour; the loops
// run 1..n-2 so the corners are never written.
template <class T> void gpu_set_bnd(Field<T> x, int mode) {
    const long R = x.rows, C = x.cols;
    for (long i = 1; i < R - 1; ++i) {
        if (mode == BND_OPP_H) {
            x(i, 0) = -x(i, 1);
            x(i, C - 1) = -x(i, C - 2);
        } else {
            x(i, 0) = x(i, 1);
            x(i, C - 1) = x(i, C - 2);
        }
    }
    for (long j = 1; j < C - 1; ++j) {
        if (mode == BND_OPP_V) {
            x(0, j) = -x(1, j);
            x(R - 1, j) = -x(R - 2, j);
        } else {
            x(0, j) = x(1, j);
            x(R - 1, j) = x(R - 2, j);
        }
    }
}

// add_sources_kernel, fluid_solver_gpu.cu:56-67 (interior only).
template <class T> void gpu_add_sources(Field<T> x, const T* s, float dt) {
    Field<const T> S{s, x.rows, x.cols};
    for (long i = 1; i < x.rows - 1; ++i)
        for (long j = 1; j < x.cols - 1; ++j) x(i, j) = madd((T)dt, S(i, j), x(i, j));
}

// diffuse, fluid_solver_gpu.cu:290-312, with diffuse_iteration_kernel 69-85:
//   a = dt * T(rows*cols) * rate
//   x = (x0 + a*(L + R + U + D)) / (1.0 + 4.0*a)      -- the divisor is double
// followed by a boundary fill after every sweep.
template <class T> void gpu_diffuse(Field<T> x, int mode, float rate, float dt, int iters) {
    const long R = x.rows, C = x.cols, n = R * C;
    std::vector<T> x0(x.p, x.p + n), prev(n);
    const T a = (T)dt * static_cast<T>((size_t)R * (size_t)C) * (T)rate;
    const double div = 1.0 + 4.0 * (double)a;
    for (int k = 0; k < iters; ++k) {
        std::memcpy(prev.data(), x.p, sizeof(T) * n);
        Field<T> P{prev.data(), R, C}, X0{x0.data(), R, C};
#pragma omp parallel for schedule(static)
        for (long i = 1; i < R - 1; ++i)
            for (long j = 1; j < C - 1; ++j) {
                T sum = P(i, j - 1) + P(i, j + 1);
                sum = sum + P(i - 1, j);
                sum = sum + P(i + 1, j);
                T num = madd(a, sum, X0(i, j));
                x(i, j) = (T)((double)num / div);
            }
        gpu_set_bnd(x, mode);
    }
}

// smooth_kernel, fluid_solver_gpu.cu:87-97 (via smooth 314-323): 5-point box
// average of the interior, no boundary fill afterwards.
template <class T> void gpu_smooth(Field<T> x) {
    const long R = x.rows, C = x.cols;
    std::vector<T> s(x.p, x.p + R * C);
    Field<T> S{s.data(), R, C};
#pragma omp parallel for schedule(static)
    for (long i = 1; i < R - 1; ++i)
        for (long j = 1; j < C - 1; ++j) {
            T sum = S(i, j) + S(i, j - 1);
            sum = sum + S(i, j + 1);
            sum = sum + S(i - 1, j);
            sum = sum + S(i + 1, j);
            x(i, j) = (T)0.2f * sum;
        }
}

// dt0 = sqrt(rows*cols) * dt, computed in double on the host and stored as float
// (fluid_solver_gpu.cu:334).
template <class T> T gpu_dt0(long R, long C, float dt) {
    return (T)(std::sqrt((double)((size_t)R * (size_t)C)) * (double)dt);
}

// advect_kernel, fluid_solver_gpu.cu:99-129: backtrace, clamp to
// [1.5, n-1.5], bilinear gather of the initial field. Boundary fill afterwards
// (advect, 325-356).
template <class T>
void gpu_advect_gather(Field<T> x, const T* x0p, const T* up, const T* vp, int mode, float dt) {
    const long R = x.rows, C = x.cols;
    Field<const T> X0{x0p, R, C}, U{up, R, C}, V{vp, R, C};
    const T dt0 = gpu_dt0<T>(R, C, dt);
    const T lo = (T)1.5f, hx = (T)C - (T)1.5f, hy = (T)R - (T)1.5f;
#pragma omp parallel for schedule(static)
    for (long i = 1; i < R - 1; ++i)
        for (long j = 1; j < C - 1; ++j) {
            T xx = madd(-dt0, U(i, j), (T)j);
            T yy = madd(-dt0, V(i, j), (T)i);
            xx = std::fmax(lo, std::fmin(hx, xx));
            yy = std::fmax(lo, std::fmin(hy, yy));
            long j0 = (long)(size_t)xx, i0 = (long)(size_t)yy;
            long j1 = j0 + 1, i1 = i0 + 1;
            T s0 = xx - (T)j0, s1 = (T)1 - s0, s2 = yy - (T)i0, s3 = (T)1 - s2;
            x(i, j) = bilinear(s0, s1, s2, s3, X0(i0, j0), X0(i0, j1), X0(i1, j0), X0(i1, j1));
        }
    gpu_set_bnd(x, mode);
}

// advect_trace_kernel, fluid_solver_gpu.cu:131-162 (via advect 325-356): the
// whole field is cleared, every interior cell is pushed forward along +dt0*(u,v)
// and splatted bilinearly into four cells; targets outside [0.5, n-1.5] are
// skipped. The CUDA kernel uses atomicAdd; this restatement adds in raster order
// of the source cell, which is one valid serialisation of those atomics.
template <class T> void gpu_advect_trace(Field<T> x, const T* up, const T* vp, float dt) {
    const long R = x.rows, C = x.cols;
    std::vector<T> init(x.p, x.p + R * C);
    Field<const T> X0{init.data(), R, C}, U{up, R, C}, V{vp, R, C};
    const T dt0 = gpu_dt0<T>(R, C, dt);
    std::fill(x.p, x.p + R * C, (T)0);
    for (long i = 1; i < R - 1; ++i)
        for (long j = 1; j < C - 1; ++j) {
            T xx = madd(dt0, U(i, j), (T)j);
            T yy = madd(dt0, V(i, j), (T)i);
            if (xx < (T)0.5f || xx > (T)C - (T)1.5f || yy < (T)0.5f || yy > (T)R - (T)1.5f) continue;
            long j0 = (long)(size_t)xx, i0 = (long)(size_t)yy;
            long j1 = j0 + 1, i1 = i0 + 1;
            T s0 = xx - (T)j0, s1 = (T)1 - s0, s2 = yy - (T)i0, s3 = (T)1 - s2;
            T d = X0(i, j);
            x(i0, j0) = x(i0, j0) + s1 * s3 * d;
            x(i1, j0) = x(i1, j0) + s1 * s2 * d;
            x(i0, j1) = x(i0, j1) + s0 * s3 * d;
            x(i1, j1) = x(i1, j1) + s0 * s2 * d;
        }
    gpu_set_bnd(x, BND_CONT);
}

// h = 1.0f / sqrtf(rows*cols) (fluid_solver_gpu.cu:367).
template <class T> T gpu_h(long R, long C) {
    if (sizeof(T) == sizeof(float)) return (T)(1.0f / sqrtf((float)((size_t)R * (size_t)C)));
    return (T)(1.0 / std::sqrt((double)((size_t)R * (size_t)C)));
}

// project, fluid_solver_gpu.cu:358-404, with calculate_divergence_kernel 164-177,
// p_iteration_kernel 179-191 and remove_p_kernel 193-206. The pressure starts at
// zero (p_buffer.clear(0), line 364). When p_inout is non-null it supplies the
// starting pressure instead and receives the final one (the warm-start hook).
template <class T> void gpu_project(Field<T> u, Field<T> v, int iters, T* p_inout, T* div_out) {
    const long R = u.rows, C = u.cols, n = R * C;
    std::vector<T> divv(n, (T)0), pv(n, (T)0), pprev(n);
    if (p_inout) std::memcpy(pv.data(), p_inout, sizeof(T) * n);
    Field<T> D{divv.data(), R, C}, P{pv.data(), R, C}, PP{pprev.data(), R, C};
    const T h = gpu_h<T>(R, C);
    const T c = (T)-0.5f * h;
    for (long i = 1; i < R - 1; ++i)
        for (long j = 1; j < C - 1; ++j) {
            T s = u(i, j + 1) - u(i, j - 1);
            s = s + v(i + 1, j);
            s = s - v(i - 1, j);
            D(i, j) = c * s;
        }
    gpu_set_bnd(D, BND_CONT);
    for (int k = 0; k < iters; ++k) {
        std::memcpy(pprev.data(), pv.data(), sizeof(T) * n);
#pragma omp parallel for schedule(static)
        for (long i = 1; i < R - 1; ++i)
            for (long j = 1; j < C - 1; ++j) {
                T s = D(i, j) + PP(i, j + 1);
                s = s + PP(i, j - 1);
                s = s + PP(i + 1, j);
                s = s + PP(i - 1, j);
                P(i, j) = s / (T)4.0f;
            }
        gpu_set_bnd(P, BND_CONT);
    }
    for (long i = 1; i < R - 1; ++i)
        for (long j = 1; j < C - 1; ++j) {
            u(i, j) = u(i, j) - (T)0.5f * (P(i, j + 1) - P(i, j - 1)) / h;
            v(i, j) = v(i, j) - (T)0.5f * (P(i + 1, j) - P(i - 1, j)) / h;
        }
    gpu_set_bnd(u, BND_OPP_H);
    gpu_set_bnd(v, BND_OPP_V);
    if (p_inout) std::memcpy(p_inout, pv.data(), sizeof(T) * n);
    if (div_out) std::memcpy(div_out, divv.data(), sizeof(T) * n);
}

// fluid_solver_gpu::solve, fluid_solver_gpu.cu:222-258, with the iteration counts
// as parameters (the reference uses kd = 15, kp = 20). kp1/kp2 are the sweeps of the
// two projections; pw1/pw2 (nullable) are their starting pressures in and final
// pressures out (the previous-pressure warm start; null = start from zero).
template <class T>
void gpu_solve_ex(long R, long C, T* d, const T* ds, float diff, T* u, T* v, const T* us, const T* vs,
                  float visc, float dt, int kd, int kp1, int kp2, int smooth, T* pw1, T* pw2) {
    Field<T> D{d, R, C}, U{u, R, C}, V{v, R, C};
    gpu_add_sources(D, ds, dt);
    gpu_diffuse(D, BND_CONT, diff, dt, kd);
    gpu_advect_trace(D, u, v, dt);
    if (smooth) gpu_smooth(D);
    gpu_add_sources(U, us, dt);
    gpu_add_sources(V, vs, dt);
    gpu_diffuse(U, BND_OPP_H, visc, dt, kd);
    gpu_diffuse(V, BND_OPP_V, visc, dt, kd);
    gpu_project(U, V, kp1, pw1, (T*)nullptr);
    std::vector<T> u0(u, u + R * C), v0(v, v + R * C);
    gpu_advect_gather(U, u0.data(), u0.data(), v0.data(), BND_OPP_H, dt);
    gpu_advect_gather(V, v0.data(), u0.data(), v0.data(), BND_OPP_V, dt);
    gpu_project(U, V, kp2, pw2, (T*)nullptr);
}

template <class T>
void gpu_solve(long R, long C, T* d, const T* ds, float diff, T* u, T* v, const T* us, const T* vs,
               float visc, float dt, int kd, int kp, int smooth) {
    Field<T> D{d, R, C}, U{u, R, C}, V{v, R, C};
    gpu_add_sources(D, ds, dt);
    gpu_diffuse(D, BND_CONT, diff, dt, kd);
    gpu_advect_trace(D, u, v, dt);
    if (smooth) gpu_smooth(D);
    gpu_add_sources(U, us, dt);
    gpu_add_sources(V, vs, dt);
    gpu_diffuse(U, BND_OPP_H, visc, dt, kd);
    gpu_diffuse(V, BND_OPP_V, visc, dt, kd);
    gpu_project(U, V, kp, (T*)nullptr, (T*)nullptr);
    std::vector<T> u0(u, u + R * C), v0(v, v + R * C);
    gpu_advect_gather(U, u0.data(), u0.data(), v0.data(), BND_OPP_H, dt);
    gpu_advect_gather(V, v0.data(), u0.data(), v0.data(), BND_OPP_V, dt);
    gpu_project(U, V, kp, (T*)nullptr, (T*)nullptr);
}

// ---------------------------------------------------------------- cpu semantics

// set_boundary_*, fluid_solver_cpu.cpp:33-83: full edge loops (corners included)
// then the four corners are averaged from their two edge neighbours.
template <class T> void cpu_corners(Field<T> g) {
    const long R = g.rows, C = g.cols;
    g(0, 0) = (T)0.5f * (g(0, 1) + g(1, 0));
    g(0, C - 1) = (T)0.5f * (g(0, C - 2) + g(1, C - 1));
    g(R - 1, 0) = (T)0.5f * (g(R - 1, 1) + g(R - 2, 0));
    g(R - 1, C - 1) = (T)0.5f * (g(R - 1, C - 2) + g(R - 2, C - 1));
}

template <class T> void cpu_set_bnd(Field<T> g, int mode) {
    const long R = g.rows, C = g.cols;
    if (mode == BND_OPP_V) {
        for (long j = 0; j < C; ++j) {
            g(0, j) = -g(1, j);
            g(R - 1, j) = -g(R - 2, j);
        }
        for (long i = 0; i < R; ++i) {
            g(i, 0) = g(i, 1);
            g(i, C - 1) = g(i, C - 2);
        }
    } else {
        for (long i = 0; i < R; ++i) {
            if (mode == BND_OPP_H) {
                g(i, 0) = -g(i, 1);
                g(i, C - 1) = -g(i, C - 2);
            } else {
                g(i, 0) = g(i, 1);
                g(i, C - 1) = g(i, C - 2);
            }
        }
        for (long j = 0; j < C; ++j) {
            g(0, j) = g(1, j);
            g(R - 1, j) = g(R - 2, j);
        }
    }
    cpu_corners(g);
}

// diffuse, fluid_solver_cpu.cpp:95-114: in-place sweeps, float divisor, sum
// order up, down, left, right.
template <class T> void cpu_diffuse(Field<T> g, int mode, float rate, float dt, int iters) {
    const long R = g.rows, C = g.cols;
    const T a = (T)dt * static_cast<T>((size_t)R * (size_t)C) * (T)rate;
    std::vector<T> init(g.p, g.p + R * C);
    Field<T> X0{init.data(), R, C};
    const T den = (T)1.f + (T)4.f * a;
    for (int k = 0; k < iters; ++k) {
        for (long i = 1; i < R - 1; ++i)
            for (long j = 1; j < C - 1; ++j) {
                T s = g(i - 1, j) + g(i + 1, j);
                s = s + g(i, j - 1);
                s = s + g(i, j + 1);
                g(i, j) = (X0(i, j) + a * s) / den;
            }
        cpu_set_bnd(g, mode);
    }
}

// advect, fluid_solver_cpu.cpp:116-177. Same arithmetic as the CUDA kernels but
// dt0 = sqrt(float(rows*cols)) * dt in float.
template <class T>
void cpu_advect(Field<T> g, const T* up, const T* vp, int mode, float dt, bool trace) {
    const long R = g.rows, C = g.cols;
    std::vector<T> init(g.p, g.p + R * C);
    Field<const T> X0{init.data(), R, C}, U{up, R, C}, V{vp, R, C};
    const T dt0 = (T)std::sqrt(static_cast<T>((size_t)R * (size_t)C)) * (T)dt;
    if (trace) {
        std::fill(g.p, g.p + R * C, (T)0);
        for (long i = 1; i < R - 1; ++i)
            for (long j = 1; j < C - 1; ++j) {
                T x = (T)j + dt0 * U(i, j);
                T y = (T)i + dt0 * V(i, j);
                if (x < (T)0.5f || x > (T)C - (T)1.5f || y < (T)0.5f || y > (T)R - (T)1.5f) continue;
                long j0 = (long)(size_t)x, i0 = (long)(size_t)y, j1 = j0 + 1, i1 = i0 + 1;
                T s0 = x - (T)j0, s1 = (T)1 - s0, s2 = y - (T)i0, s3 = (T)1 - s2;
                g(i0, j0) = g(i0, j0) + s1 * s3 * X0(i, j);
                g(i1, j0) = g(i1, j0) + s1 * s2 * X0(i, j);
                g(i0, j1) = g(i0, j1) + s0 * s3 * X0(i, j);
                g(i1, j1) = g(i1, j1) + s0 * s2 * X0(i, j);
            }
    } else {
        for (long i = 1; i < R - 1; ++i)
            for (long j = 1; j < C - 1; ++j) {
                T x = (T)j - dt0 * U(i, j);
                T y = (T)i - dt0 * V(i, j);
                // std::max(1.5f, std::min(cols - 1.5f, x))
                T hx = (T)C - (T)1.5f, hy = (T)R - (T)1.5f;
                x = (x < hx) ? x : hx;
                x = ((T)1.5f < x) ? x : (T)1.5f;
                y = (y < hy) ? y : hy;
                y = ((T)1.5f < y) ? y : (T)1.5f;
                long j0 = (long)(size_t)x, i0 = (long)(size_t)y, j1 = j0 + 1, i1 = i0 + 1;
                T s0 = x - (T)j0, s1 = (T)1 - s0, s2 = y - (T)i0, s3 = (T)1 - s2;
                g(i, j) = s3 * (s1 * X0(i0, j0) + s0 * X0(i0, j1)) + s2 * (s1 * X0(i1, j0) + s0 * X0(i1, j1));
            }
    }
    cpu_set_bnd(g, mode);
}

// project, fluid_solver_cpu.cpp:179-215: in-place pressure sweeps from p = 0.
template <class T> void cpu_project(Field<T> u, Field<T> v, int iters) {
    const long R = u.rows, C = u.cols;
    const T h = (T)1.0f / (T)std::sqrt(static_cast<T>((size_t)R * (size_t)C));
    std::vector<T> dv(R * C, (T)0), pv(R * C, (T)0);
    Field<T> D{dv.data(), R, C}, P{pv.data(), R, C};
    for (long i = 1; i < R - 1; ++i)
        for (long j = 1; j < C - 1; ++j) {
            T s = u(i, j + 1) - u(i, j - 1);
            s = s + v(i + 1, j);
            s = s - v(i - 1, j);
            D(i, j) = (T)-0.5f * h * s;
        }
    cpu_set_bnd(D, BND_CONT);
    for (int k = 0; k < iters; ++k) {
        for (long i = 1; i < R - 1; ++i)
            for (long j = 1; j < C - 1; ++j) {
                T s = D(i, j) + P(i, j + 1);
                s = s + P(i, j - 1);
                s = s + P(i + 1, j);
                s = s + P(i - 1, j);
                P(i, j) = s / (T)4.0f;
            }
        cpu_set_bnd(P, BND_CONT);
    }
    for (long i = 1; i < R - 1; ++i)
        for (long j = 1; j < C - 1; ++j) {
            u(i, j) = u(i, j) - (T)0.5f * (P(i, j + 1) - P(i, j - 1)) / h;
            v(i, j) = v(i, j) - (T)0.5f * (P(i + 1, j) - P(i - 1, j)) / h;
        }
    cpu_set_bnd(u, BND_OPP_H);
    cpu_set_bnd(v, BND_OPP_V);
}

// fluid_solver_cpu::solve, fluid_solver_cpu.cpp:6-31 (the reference uses kd = kp = 20).
template <class T>
void cpu_solve(long R, T* d, const T* ds, float diff, T* u, T* v, const T* us, const T* vs, float visc,
               float dt, int kd, int kp) {
    const long C = R;  // grid<T>::cols() returns rows (grid.hpp:20-22): square only
    Field<T> D{d, R, C}, U{u, R, C}, V{v, R, C};
    for (long i = 1; i < R - 1; ++i)
        for (long j = 1; j < C - 1; ++j) D(i, j) = D(i, j) + (T)dt * ds[i * C + j];
    cpu_diffuse(D, BND_CONT, diff, dt, kd);
    cpu_advect(D, u, v, BND_CONT, dt, true);
    for (long i = 1; i < R - 1; ++i)
        for (long j = 1; j < C - 1; ++j) {
            U(i, j) = U(i, j) + (T)dt * us[i * C + j];
            V(i, j) = V(i, j) + (T)dt * vs[i * C + j];
        }
    cpu_diffuse(U, BND_OPP_H, visc, dt, kd);
    cpu_diffuse(V, BND_OPP_V, visc, dt, kd);
    cpu_project(U, V, kp);
    std::vector<T> tu(u, u + R * C), tv(v, v + R * C);
    cpu_advect(U, tu.data(), tv.data(), BND_OPP_H, dt, false);
    cpu_advect(V, tu.data(), tv.data(), BND_OPP_V, dt, false);
    cpu_project(U, V, kp);
}

// Relative Poisson residual ||div + sum(p nbrs) - 4p||_2 / ||div||_2 over the
// interior (the convergence measure of the pressure solve).
template <class T> double residual(long R, long C, const T* p, const T* dv) {
    double num = 0, den = 0;
    for (long i = 1; i < R - 1; ++i)
        for (long j = 1; j < C - 1; ++j) {
            double r = (double)dv[i * C + j] + (double)p[i * C + j + 1] + (double)p[i * C + j - 1] +
                       (double)p[(i + 1) * C + j] + (double)p[(i - 1) * C + j] - 4.0 * (double)p[i * C + j];
            num += r * r;
            den += (double)dv[i * C + j] * (double)dv[i * C + j];
        }
    return den > 0 ? std::sqrt(num / den) : std::sqrt(num);
}

bool bad(long rows, long cols) { return rows < 3 || cols < 3; }

}  // namespace

extern "C" {

// Whole steps ----------------------------------------------------------------

int orc_gpu_solve_f32(long rows, long cols, float* d, const float* ds, float diff, float* u, float* v,
                      const float* us, const float* vs, float visc, float dt, int kd, int kp,
                      int smooth, int nsteps) {
    if (bad(rows, cols)) return 1;
    for (int s = 0; s < nsteps; ++s) gpu_solve<float>(rows, cols, d, ds, diff, u, v, us, vs, visc, dt, kd, kp, smooth);
    return 0;
}

int orc_gpu_solve_f64(long rows, long cols, double* d, const double* ds, float diff, double* u, double* v,
                      const double* us, const double* vs, float visc, float dt, int kd, int kp,
                      int smooth, int nsteps) {
    if (bad(rows, cols)) return 1;
    for (int s = 0; s < nsteps; ++s) gpu_solve<double>(rows, cols, d, ds, diff, u, v, us, vs, visc, dt, kd, kp, smooth);
    return 0;
}

// One step with separate projection sweep counts and optional warm-start pressures.
int orc_gpu_solve_ex_f32(long rows, long cols, float* d, const float* ds, float diff, float* u, float* v,
                         const float* us, const float* vs, float visc, float dt, int kd, int kp1, int kp2,
                         int smooth, float* pw1, float* pw2) {
    if (bad(rows, cols)) return 1;
    gpu_solve_ex<float>(rows, cols, d, ds, diff, u, v, us, vs, visc, dt, kd, kp1, kp2, smooth, pw1, pw2);
    return 0;
}

int orc_cpu_solve_f32(long n, float* d, const float* ds, float diff, float* u, float* v, const float* us,
                      const float* vs, float visc, float dt, int kd, int kp, int nsteps) {
    if (bad(n, n)) return 1;
    for (int s = 0; s < nsteps; ++s) cpu_solve<float>(n, d, ds, diff, u, v, us, vs, visc, dt, kd, kp);
    return 0;
}

// Single stages (gpu semantics) -------------------------------------------------

void orc_set_contract(int contract, int bilinear_mode) {
    g_contract = contract;
    g_bilinear = bilinear_mode;
}

int orc_add_sources_f32(long rows, long cols, float* x, const float* s, float dt) {
    if (bad(rows, cols)) return 1;
    gpu_add_sources(Field<float>{x, rows, cols}, s, dt);
    return 0;
}

int orc_diffuse_f32(long rows, long cols, float* x, int mode, float rate, float dt, int iters) {
    if (bad(rows, cols)) return 1;
    gpu_diffuse(Field<float>{x, rows, cols}, mode, rate, dt, iters);
    return 0;
}

int orc_set_bnd_f32(long rows, long cols, float* x, int mode) {
    if (bad(rows, cols)) return 1;
    gpu_set_bnd(Field<float>{x, rows, cols}, mode);
    return 0;
}

int orc_advect_trace_f32(long rows, long cols, float* d, const float* u, const float* v, float dt) {
    if (bad(rows, cols)) return 1;
    gpu_advect_trace(Field<float>{d, rows, cols}, u, v, dt);
    return 0;
}

int orc_smooth_f32(long rows, long cols, float* d) {
    if (bad(rows, cols)) return 1;
    gpu_smooth(Field<float>{d, rows, cols});
    return 0;
}

// Advects u and v together by the same (u0, v0), as fluid_solver_gpu.cu:248-251.
int orc_advect_velocity_f32(long rows, long cols, float* u, float* v, float dt) {
    if (bad(rows, cols)) return 1;
    std::vector<float> u0(u, u + rows * cols), v0(v, v + rows * cols);
    gpu_advect_gather(Field<float>{u, rows, cols}, u0.data(), u0.data(), v0.data(), BND_OPP_H, dt);
    gpu_advect_gather(Field<float>{v, rows, cols}, v0.data(), u0.data(), v0.data(), BND_OPP_V, dt);
    return 0;
}

// p_inout: optional starting pressure (in) / final pressure (out); div_out optional.
int orc_project_f32(long rows, long cols, float* u, float* v, int iters, float* p_inout, float* div_out) {
    if (bad(rows, cols)) return 1;
    gpu_project(Field<float>{u, rows, cols}, Field<float>{v, rows, cols}, iters, p_inout, div_out);
    return 0;
}

int orc_project_f64(long rows, long cols, double* u, double* v, int iters, double* p_inout, double* div_out) {
    if (bad(rows, cols)) return 1;
    gpu_project(Field<double>{u, rows, cols}, Field<double>{v, rows, cols}, iters, p_inout, div_out);
    return 0;
}

double orc_residual_f32(long rows, long cols, const float* p, const float* div) {
    return residual<float>(rows, cols, p, div);
}

double orc_residual_f64(long rows, long cols, const double* p, const double* div) {
    return residual<double>(rows, cols, p, div);
}

}  // extern "C"
