// Exact reproduction of the reference's host solver (fluid_solver_cpu, src/
// fluid_solver_cpu.cpp:6-215) on the GPU, for square grids whose field fits in one
// SM's shared memory (n <= gs_max_size(), 234 on a 227 KB part).
//
// The host solver differs from the CUDA one in method, not just rounding: its
// diffusion and pressure sweeps update in place in row-major order (lexicographic
// Gauss-Seidel), every boundary fill also averages the four corners, the diffusion
// divisor is float, there is no smoothing, and the forward splat adds in raster order.
// Here each in-place solve runs in one CTA with the field in shared memory as an
// anti-diagonal wavefront: cell (i, j) of sweep s is updated at time (i-1)+(j-1)+2s, so
// every sweep sees its up/left neighbours already updated and its down/right
// neighbours not yet, exactly as the sequential loop does, and all sweeps are in
// flight at once. An edge cell is read only by its inner neighbour, so the thread that
// updates that neighbour also rewrites the edge (the fill the host solver does after
// every sweep); corners are never read by a sweep and are averaged once at the end.
// The splat keeps the host solver's order of additions to every cell: a cell receives
// its contributions in the raster order of their source cells. When no source moves
// more than kGatherMaxD cells, each target cell gathers them itself, scanning the
// sources around it in raster order (many CTAs); otherwise the whole CTA computes the
// targets and weights of a chunk of source cells and one thread applies them in order.
//
// A step is four launches on the solver's pitched fields (element (i, j) at i*P + j):
//   1. 3 CTAs: add sources + diffuse d | copy u, add sources, diffuse u, largest
//      displacement | same for v
//   2. project u, v (CTA 0) | splat d by the step's initial velocity into a scratch
//      field: one CTA in order (CTA 1) or one CTA per 1024 target cells (CTAs 2..)
//   3. copy u, v and advect both by the copies (CTA 0) | the splat result and the
//      host solver's fill into d (CTA 1)
//   4. 1 CTA : project u, v
// Every operation uses explicitly rounded single-precision intrinsics so that no
// contraction changes a result; the outputs are bit-identical to the host solver's.

#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/fluid2d_gb300.h"
#include "fs_internal.cuh"

namespace fs {
namespace {

constexpr int kGsThreads = 1024;
constexpr int kGsStage = 512;   // source cells per splat chunk (in-order path)
constexpr int kGatherMaxD = 16; // largest displacement (cells) for the gathering splat

struct GsStageEntry {
    int i0, j0;
    float w[4];  // contributions to (i0,j0), (i0+1,j0), (i0,j0+1), (i0+1,j0+1)
};

// set_boundary_* of the host solver (fluid_solver_cpu.cpp:33-83) on an n x n field of
// row stride `ld`: edges from their inner neighbours with the mode's signs, then the
// corners averaged from their two edge neighbours. Ends with a block barrier.
__device__ void cpu_fill(float* g, int n, int ld, int mode) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const float s_lr = mode == BND_OPP_H ? -1.f : 1.f, s_tb = mode == BND_OPP_V ? -1.f : 1.f;
    for (int k = 1 + tid; k < n - 1; k += nt) {
        g[k * ld] = s_lr * g[k * ld + 1];
        g[k * ld + n - 1] = s_lr * g[k * ld + n - 2];
        g[k] = s_tb * g[ld + k];
        g[(n - 1) * ld + k] = s_tb * g[(n - 2) * ld + k];
    }
    __syncthreads();
    if (tid == 0) {
        const int b = (n - 1) * ld, c = n - 1;
        g[0] = __fmul_rn(0.5f, __fadd_rn(g[1], g[ld]));
        g[c] = __fmul_rn(0.5f, __fadd_rn(g[c - 1], g[ld + c]));
        g[b] = __fmul_rn(0.5f, __fadd_rn(g[b + 1], g[b - ld]));
        g[b + c] = __fmul_rn(0.5f, __fadd_rn(g[b + c - 1], g[b - ld + c]));
    }
    __syncthreads();
}

// Pipelined lexicographic Gauss-Seidel on x (shared, n x n dense, in place):
//   DIFF: x = (c + a*(U + D + L + R)) / den          (fluid_solver_cpu.cpp:105-110)
//   else: x = (c + R + L + D + U) / 4                (fluid_solver_cpu.cpp:197-202)
// with c read from `cst` (global, row stride P): x0 for diffusion, div for pressure.
template <bool DIFF>
__device__ void gs_wavefront(float* x, const float* cst, int n, int P, int iters, int mode, float a, float den) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const float s_lr = mode == BND_OPP_H ? -1.f : 1.f, s_tb = mode == BND_OPP_V ? -1.f : 1.f;
    const int m = n - 2, dmax = 2 * m - 2;
    const int last_t = dmax + 2 * (iters - 1);
    for (int t = 0; t <= last_t; ++t) {
        // sweeps with a diagonal d = t - 2s in [0, dmax]
        const int s_lo = t > dmax ? (t - dmax + 1) / 2 : 0;
        const int s_hi = min(iters - 1, t / 2);
        const int work = (s_hi - s_lo + 1) * m;
        for (int e = tid; e < work; e += nt) {
            const int s = s_lo + e / m, q = e % m, d = t - 2 * s;
            if (q < d - (m - 1) || q > d) continue;
            const int i = 1 + q, j = 1 + d - q;
            const int o = i * n + j;
            float val;
            if (DIFF) {
                float sum = __fadd_rn(x[o - n], x[o + n]);
                sum = __fadd_rn(sum, x[o - 1]);
                sum = __fadd_rn(sum, x[o + 1]);
                val = __fdiv_rn(__fadd_rn(cst[i * P + j], __fmul_rn(a, sum)), den);
            } else {
                float sum = __fadd_rn(cst[i * P + j], x[o + 1]);
                sum = __fadd_rn(sum, x[o - 1]);
                sum = __fadd_rn(sum, x[o + n]);
                sum = __fadd_rn(sum, x[o - n]);
                val = __fdiv_rn(sum, 4.0f);
            }
            x[o] = val;
            // the host solver's fill after this sweep, for the edges next to (i, j)
            if (j == 1) x[o - 1] = s_lr * val;
            if (j == n - 2) x[o + 1] = s_lr * val;
            if (i == 1) x[o - n] = s_tb * val;
            if (i == n - 2) x[o + n] = s_tb * val;
        }
        __syncthreads();
    }
}

struct GsArgs {
    float* f[3];         // d, u, v (state)
    const float* src[3]; // ds, us, vs
    float* su;           // scratch: copy of u
    float* sv;           // scratch: copy of v
    float* dv;           // scratch: divergence
    float* acc;          // scratch: splat result (interior)
    float* dmax;         // scratch: largest |dt0 u| and |dt0 v| of the step's initial velocity
    int n, P, kd, kp;
    float a[3], den[3];  // diffusion constants per field
    float dt, dt0, h;
};

__device__ void copy_field(float* dst, const float* src, int n, int P) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) dst[(e / n) * P + e % n] = src[(e / n) * P + e % n];
}

// add_source then diffuse (fluid_solver_cpu.cpp:85-114) of field k.
__device__ void gs_diffuse(const GsArgs& A, int k, float* x) {
    const int n = A.n, P = A.P;
    const int mode = k == 0 ? BND_CONT : (k == 1 ? BND_OPP_H : BND_OPP_V);
    float* g = A.f[k];
    const float* s = A.src[k];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e % n, o = i * P + j;
        float val = g[o];
        if (i > 0 && i < n - 1 && j > 0 && j < n - 1) {
            val = __fadd_rn(val, __fmul_rn(A.dt, s[o]));
            g[o] = val;  // the diffusion's x0
        }
        x[e] = val;
    }
    __syncthreads();
    if (A.kd > 0) {
        gs_wavefront<true>(x, g, n, P, A.kd, mode, A.a[k], A.den[k]);
        cpu_fill(x, n, n, mode);
    }
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) g[(e / n) * P + e % n] = x[e];
}

// advect(trace=true) (fluid_solver_cpu.cpp:127-152) of d by (su, sv), accumulating in
// shared memory, then the host solver's continuous fill.
__device__ void gs_splat(const GsArgs& A, float* acc, GsStageEntry* stage) {
    const int n = A.n, P = A.P, m = n - 2;
    const float* d0 = A.f[0];
    const float hi = (float)n - 1.5f;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) acc[e] = 0.f;
    for (int base = 0; base < m * m; base += kGsStage) {
        const int cnt = min(kGsStage, m * m - base);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
            const int c = base + k, i = 1 + c / m, j = 1 + c % m, o = i * P + j;
            const float x = __fadd_rn((float)j, __fmul_rn(A.dt0, A.su[o]));
            const float y = __fadd_rn((float)i, __fmul_rn(A.dt0, A.sv[o]));
            GsStageEntry en;
            if (!(x >= 0.5f && x <= hi && y >= 0.5f && y <= hi)) {  // NaN-safe form of the skip test
                en.i0 = -1;
                en.j0 = 0;
                en.w[0] = en.w[1] = en.w[2] = en.w[3] = 0.f;
            } else {
                const int j0 = (int)x, i0 = (int)y;
                const float s0 = __fsub_rn(x, (float)j0), s1 = __fsub_rn(1.f, s0);
                const float s2 = __fsub_rn(y, (float)i0), s3 = __fsub_rn(1.f, s2);
                const float w = d0[o];
                en.i0 = i0;
                en.j0 = j0;
                en.w[0] = __fmul_rn(__fmul_rn(s1, s3), w);
                en.w[1] = __fmul_rn(__fmul_rn(s1, s2), w);
                en.w[2] = __fmul_rn(__fmul_rn(s0, s3), w);
                en.w[3] = __fmul_rn(__fmul_rn(s0, s2), w);
            }
            stage[k] = en;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int k = 0; k < cnt; ++k) {
                const GsStageEntry en = stage[k];
                if (en.i0 < 0) continue;
                const int t = en.i0 * n + en.j0;
                acc[t] = __fadd_rn(acc[t], en.w[0]);
                acc[t + n] = __fadd_rn(acc[t + n], en.w[1]);
                acc[t + 1] = __fadd_rn(acc[t + 1], en.w[2]);
                acc[t + n + 1] = __fadd_rn(acc[t + n + 1], en.w[3]);
            }
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
        const int i = 1 + e / m, j = 1 + e % m;
        A.acc[i * P + j] = acc[i * n + j];
    }
}

// The same splat gathered by target: thread t of target block b owns interior cell
// T = b*blockDim + t and adds, in the raster order of the sources, the contribution of
// every source within W = D + 2 cells (D = the largest displacement, so every source
// that can reach T is scanned); each source reaches T through at most one corner.
__device__ void gs_splat_gather(const GsArgs& A, int b, int D) {
    const int n = A.n, P = A.P, m = n - 2;
    const int e = b * blockDim.x + threadIdx.x;
    if (e >= m * m) return;
    const int ti = 1 + e / m, tj = 1 + e % m;
    const float hi = (float)n - 1.5f;
    const float* d0 = A.f[0];
    const int W = D + 2;
    const int i_lo = max(1, ti - W), i_hi = min(n - 2, ti + W), j_lo = max(1, tj - W), j_hi = min(n - 2, tj + W);
    float acc = 0.f;
    for (int i = i_lo; i <= i_hi; ++i)
        for (int j = j_lo; j <= j_hi; ++j) {
            const int o = i * P + j;
            const float x = __fadd_rn((float)j, __fmul_rn(A.dt0, A.su[o]));
            const float y = __fadd_rn((float)i, __fmul_rn(A.dt0, A.sv[o]));
            if (!(x >= 0.5f && x <= hi && y >= 0.5f && y <= hi)) continue;
            const int j0 = (int)x, i0 = (int)y;
            const int di = ti - i0, dj = tj - j0;  // which corner of the source's cell T is
            if ((unsigned)di > 1u || (unsigned)dj > 1u) continue;
            const float s0 = __fsub_rn(x, (float)j0), s1 = __fsub_rn(1.f, s0);
            const float s2 = __fsub_rn(y, (float)i0), s3 = __fsub_rn(1.f, s2);
            const float wy = di ? s2 : s3, wx = dj ? s0 : s1;
            acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(wx, wy), d0[o]));
        }
    A.acc[ti * P + tj] = acc;
}

// project (fluid_solver_cpu.cpp:179-215) of (u, v), pressure from zero in shared memory.
__device__ void gs_project(const GsArgs& A, float* p) {
    const int n = A.n, P = A.P, m = n - 2;
    float* u = A.f[1];
    float* v = A.f[2];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) p[e] = 0.f;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
        const int o = (1 + e / m) * P + 1 + e % m;
        float s = __fsub_rn(u[o + 1], u[o - 1]);
        s = __fadd_rn(s, v[o + P]);
        s = __fsub_rn(s, v[o - P]);
        A.dv[o] = __fmul_rn(__fmul_rn(-0.5f, A.h), s);
    }
    __syncthreads();
    if (A.kp > 0) {
        gs_wavefront<false>(p, A.dv, n, P, A.kp, BND_CONT, 0.f, 0.f);
        cpu_fill(p, n, n, BND_CONT);
    }
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
        const int i = 1 + e / m, j = 1 + e % m, o = i * P + j, q = i * n + j;
        u[o] = __fsub_rn(u[o], __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(p[q + 1], p[q - 1])), A.h));
        v[o] = __fsub_rn(v[o], __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(p[q + n], p[q - n])), A.h));
    }
    __syncthreads();
    cpu_fill(u, n, P, BND_OPP_H);
    cpu_fill(v, n, P, BND_OPP_V);
}

// advect(trace=false) (fluid_solver_cpu.cpp:154-173) of u and v by the copies (su, sv).
__device__ void gs_gather(const GsArgs& A) {
    const int n = A.n, P = A.P, m = n - 2;
    copy_field(A.su, A.f[1], n, P);
    copy_field(A.sv, A.f[2], n, P);
    __syncthreads();
    const float hi = (float)n - 1.5f;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
        const int i = 1 + e / m, j = 1 + e % m, o = i * P + j;
        float x = __fsub_rn((float)j, __fmul_rn(A.dt0, A.su[o]));
        float y = __fsub_rn((float)i, __fmul_rn(A.dt0, A.sv[o]));
        x = (x < hi) ? x : hi;
        x = (1.5f < x) ? x : 1.5f;
        y = (y < hi) ? y : hi;
        y = (1.5f < y) ? y : 1.5f;
        const int j0 = (int)x, i0 = (int)y;
        const float s0 = __fsub_rn(x, (float)j0), s1 = __fsub_rn(1.f, s0);
        const float s2 = __fsub_rn(y, (float)i0), s3 = __fsub_rn(1.f, s2);
        const int a = i0 * P + j0;
        for (int k = 0; k < 2; ++k) {
            const float* g0 = k == 0 ? A.su : A.sv;
            const float top = __fadd_rn(__fmul_rn(s1, g0[a]), __fmul_rn(s0, g0[a + 1]));
            const float bot = __fadd_rn(__fmul_rn(s1, g0[a + P]), __fmul_rn(s0, g0[a + P + 1]));
            A.f[1 + k][o] = __fadd_rn(__fmul_rn(s3, top), __fmul_rn(s2, bot));
        }
    }
    __syncthreads();
    cpu_fill(A.f[1], n, P, BND_OPP_H);
    cpu_fill(A.f[2], n, P, BND_OPP_V);
}

__global__ void __launch_bounds__(kGsThreads) gs_diffuse_kernel(const __grid_constant__ GsArgs A) {
    extern __shared__ float4 gs_smem[];
    float* x = reinterpret_cast<float*>(gs_smem);
    const int k = blockIdx.x;
    if (k > 0) {  // keep the step's initial velocity for the density splat
        float* dst = k == 1 ? A.su : A.sv;
        const float* src = A.f[k];
        const int n = A.n, P = A.P, m = n - 2;
        copy_field(dst, src, n, P);
        // largest interior displacement |dt0 * velocity| (non-finite counts as huge)
        float dm = 0.f;
        for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
            float a = fabsf(__fmul_rn(A.dt0, src[(1 + e / m) * P + 1 + e % m]));
            if (!(a <= 1e30f)) a = 1e30f;
            dm = fmaxf(dm, a);
        }
        __shared__ float red[32];
        for (int o = 16; o > 0; o >>= 1) dm = fmaxf(dm, __shfl_xor_sync(0xffffffffu, dm, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dm;
        __syncthreads();
        if (threadIdx.x == 0) {
            float t = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmaxf(t, red[w]);
            A.dmax[k - 1] = t;
        }
        __syncthreads();
    }
    gs_diffuse(A, k, x);
}

__global__ void __launch_bounds__(kGsThreads) gs_splat_project_kernel(const __grid_constant__ GsArgs A) {
    extern __shared__ float4 gs_smem[];
    float* f = reinterpret_cast<float*>(gs_smem);
    // every CTA reads the same two values (written by the previous launch)
    const float dm = fmaxf(__ldcg(A.dmax), __ldcg(A.dmax + 1));
    const bool gather = dm <= (float)kGatherMaxD;
    if (blockIdx.x == 0)
        gs_project(A, f);
    else if (blockIdx.x == 1) {
        if (!gather) gs_splat(A, f, reinterpret_cast<GsStageEntry*>(f + A.n * A.n));
    } else if (gather) {
        gs_splat_gather(A, blockIdx.x - 2, (int)ceilf(dm));
    }
}

// CTA 0: advect u, v; CTA 1: density = the splat result with the host solver's fill.
__global__ void __launch_bounds__(kGsThreads) gs_gather_kernel(const __grid_constant__ GsArgs A) {
    if (blockIdx.x == 0) {
        gs_gather(A);
        return;
    }
    const int n = A.n, P = A.P, m = n - 2;
    float* d = A.f[0];
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
        const int o = (1 + e / m) * P + 1 + e % m;
        d[o] = A.acc[o];
    }
    __syncthreads();
    cpu_fill(d, n, P, BND_CONT);
}

__global__ void __launch_bounds__(kGsThreads) gs_project_kernel(const __grid_constant__ GsArgs A) {
    extern __shared__ float4 gs_smem[];
    gs_project(A, reinterpret_cast<float*>(gs_smem));
}

size_t gs_smem_bytes(int n) {
    return ((size_t)n * n * sizeof(float) + 15) / 16 * 16 + kGsStage * sizeof(GsStageEntry);
}

// ---------------------------------------------------------------------------
// Tiled form for grids larger than one SM's shared memory.
//
// Each in-place solve runs as one cooperative launch over kTile x kTile tiles of the
// interior, with the field in global memory. Tile (I, J) of sweep s is processed at
// wavefront time t = I + J + 2s, all tiles of one time in parallel, a grid barrier
// between times. This keeps every dependency of the sequential loop: the tiles above
// and to the left finished sweep s at time t - 1 (their new values), the tiles below
// and to the right finished sweep s - 1 at t - 1 and start sweep s only at t + 1 (their
// old values), and no two tiles of one time are neighbours. Inside a tile the cells are
// updated by the same anti-diagonal wavefront as the one-CTA form, from a shared copy
// of the tile and its one-cell halo, and an update next to a domain edge rewrites that
// edge cell (the host solver's fill after each sweep, which only that cell reads).
// Grid barriers wait a bounded number of polls; a CTA that gives up sets ctrl->error
// and the solve ends early (FS_ERR_TIMEOUT on the host).
constexpr int kTile = 64;
constexpr int kTileThreads = 64;
constexpr unsigned kGsBarrierPolls = 1u << 24;

struct GsTiled {
    float* x;        // field, in place (row stride P)
    const float* c;  // constant term: x0 (diffusion) or div (pressure)
    int n, P, iters, mode;
    float a, den;    // diffusion
    SolveCtrl* ctrl;
    const unsigned* poll_limit;
};

__device__ bool gs_grid_barrier(SolveCtrl* ctrl, unsigned nblocks, unsigned limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = &ctrl->bar_gen;
        volatile int* err = &ctrl->error;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(&ctrl->bar_count, 1u) == nblocks - 1) {
            atomicExch(&ctrl->bar_count, 0u);
            __threadfence();
            atomicAdd(&ctrl->bar_gen, 1u);
        } else {
            unsigned spins = 0;
            while (*gen == g && *err == 0) {
                if (++spins > limit) {
                    atomicExch(&ctrl->error, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = (*err == 0);
    }
    __syncthreads();
    return s_ok != 0;
}

template <bool DIFF>
__device__ void gs_tile(const GsTiled& S, int I, int J, float* xs, float* cs) {
    constexpr int LD = kTile + 2;
    const int n = S.n, P = S.P, tid = threadIdx.x, nt = blockDim.x;
    const float s_lr = S.mode == BND_OPP_H ? -1.f : 1.f, s_tb = S.mode == BND_OPP_V ? -1.f : 1.f;
    const int i0 = 1 + I * kTile, j0 = 1 + J * kTile;
    const int th = min(kTile, n - 1 - i0), tw = min(kTile, n - 1 - j0);
    for (int e = tid; e < (th + 2) * (tw + 2); e += nt) {
        const int r = e / (tw + 2), q = e - r * (tw + 2);
        xs[r * LD + q] = __ldcg(S.x + (size_t)(i0 - 1 + r) * P + (j0 - 1 + q));
    }
    for (int e = tid; e < th * tw; e += nt) {
        const int r = e / tw, q = e - r * tw;
        cs[r * kTile + q] = __ldcg(S.c + (size_t)(i0 + r) * P + (j0 + q));
    }
    __syncthreads();
    for (int dg = 0; dg < th + tw - 1; ++dg) {
        for (int r = tid; r < th; r += nt) {
            const int q = dg - r;
            if (q < 0 || q >= tw) continue;
            const int o = (r + 1) * LD + q + 1;
            float val;
            if (DIFF) {  // (x0 + a*(U + D + L + R)) / (1 + 4a), fluid_solver_cpu.cpp:107-108
                float sum = __fadd_rn(xs[o - LD], xs[o + LD]);
                sum = __fadd_rn(sum, xs[o - 1]);
                sum = __fadd_rn(sum, xs[o + 1]);
                val = __fdiv_rn(__fadd_rn(cs[r * kTile + q], __fmul_rn(S.a, sum)), S.den);
            } else {     // (div + R + L + D + U) / 4, fluid_solver_cpu.cpp:199-200
                float sum = __fadd_rn(cs[r * kTile + q], xs[o + 1]);
                sum = __fadd_rn(sum, xs[o - 1]);
                sum = __fadd_rn(sum, xs[o + LD]);
                sum = __fadd_rn(sum, xs[o - LD]);
                val = __fdiv_rn(sum, 4.0f);
            }
            xs[o] = val;
            const int gi = i0 + r, gj = j0 + q;
            if (gj == 1) xs[o - 1] = s_lr * val;
            if (gj == n - 2) xs[o + 1] = s_lr * val;
            if (gi == 1) xs[o - LD] = s_tb * val;
            if (gi == n - 2) xs[o + LD] = s_tb * val;
        }
        __syncthreads();
    }
    // the tile, and the domain-edge cells next to it (the other halo cells belong to
    // other tiles)
    for (int e = tid; e < th * tw; e += nt) {
        const int r = e / tw, q = e - r * tw;
        S.x[(size_t)(i0 + r) * P + (j0 + q)] = xs[(r + 1) * LD + q + 1];
    }
    for (int q = tid; q < tw; q += nt) {
        if (i0 == 1) S.x[j0 + q] = xs[q + 1];
        if (i0 + th == n - 1) S.x[(size_t)(n - 1) * P + j0 + q] = xs[(th + 1) * LD + q + 1];
    }
    for (int r = tid; r < th; r += nt) {
        if (j0 == 1) S.x[(size_t)(i0 + r) * P] = xs[(r + 1) * LD];
        if (j0 + tw == n - 1) S.x[(size_t)(i0 + r) * P + n - 1] = xs[(r + 1) * LD + tw + 1];
    }
    __syncthreads();  // xs is reused by this CTA's next tile
}

template <bool DIFF>
__global__ void __launch_bounds__(kTileThreads) gs_tiled_kernel(const __grid_constant__ GsTiled S) {
    __shared__ float xs[(kTile + 2) * (kTile + 2)];
    __shared__ float cs[kTile * kTile];
    const int m = S.n - 2, NT = (m + kTile - 1) / kTile, K = S.iters;
    const unsigned G = gridDim.x;
    const unsigned lim_set = S.poll_limit ? __ldcg(S.poll_limit) : 0u;
    const unsigned limit = lim_set ? lim_set : kGsBarrierPolls;
    const int last_t = 2 * (NT - 1) + 2 * (K - 1);
    for (int t = 0; t <= last_t; ++t) {
        int base = 0;
        for (int s = max(0, (t - 2 * (NT - 1) + 1) / 2); s <= min(K - 1, t / 2); ++s) {
            const int d = t - 2 * s;
            const int ilo = max(0, d - NT + 1), ihi = min(NT - 1, d);
            for (int k = 0; k <= ihi - ilo; ++k)
                if ((unsigned)(base + k) % G == blockIdx.x) gs_tile<DIFF>(S, ilo + k, d - ilo - k, xs, cs);
            base += max(0, ihi - ilo + 1);
        }
        if (t < last_t && !gs_grid_barrier(S.ctrl, G, limit)) return;
    }
}

// The host solver's fill (cpu_fill) on a field in global memory, one CTA.
__global__ void __launch_bounds__(kGsThreads) gs_fill_kernel(float* g, int n, int P, int mode) { cpu_fill(g, n, P, mode); }

// x += dt*s on the interior and x0 = x (the diffusion's constant term).
__global__ void gs_add_copy_kernel(float* x, const float* __restrict__ src, float* __restrict__ x0, int n, int P,
                                   float dt) {
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < (long)n * n; e += (long)gridDim.x * blockDim.x) {
        const int i = (int)(e / n), j = (int)(e % n);
        const size_t o = (size_t)i * P + j;
        float val = x[o];
        if (i > 0 && i < n - 1 && j > 0 && j < n - 1) {
            val = __fadd_rn(val, __fmul_rn(dt, src[o]));
            x[o] = val;
        }
        x0[o] = val;
    }
}

// su = u, sv = v and the largest interior displacement |dt0 * velocity| into dmax[0..1]
// (float bits, non-negative, so an integer maximum orders them; zeroed before).
__global__ void gs_copy_vel_kernel(const GsArgs A) {
    const int n = A.n, P = A.P;
    float dm = 0.f;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < (long)n * n; e += (long)gridDim.x * blockDim.x) {
        const int i = (int)(e / n), j = (int)(e % n);
        const size_t o = (size_t)i * P + j;
        const float u = A.f[1][o], v = A.f[2][o];
        A.su[o] = u;
        A.sv[o] = v;
        if (i > 0 && i < n - 1 && j > 0 && j < n - 1) {
            float a = fmaxf(fabsf(__fmul_rn(A.dt0, u)), fabsf(__fmul_rn(A.dt0, v)));
            if (!(a <= 1e30f)) a = 1e30f;
            dm = fmaxf(dm, a);
        }
    }
    for (int o = 16; o > 0; o >>= 1) dm = fmaxf(dm, __shfl_xor_sync(0xffffffffu, dm, o));
    if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int*>(A.dmax), __float_as_int(dm));
}

// Divergence (fluid_solver_cpu.cpp:186-191) into dv and p = 0.
__global__ void gs_div_kernel(const GsArgs A, float* p) {
    const int n = A.n, P = A.P;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < (long)n * n; e += (long)gridDim.x * blockDim.x) {
        const int i = (int)(e / n), j = (int)(e % n);
        const size_t o = (size_t)i * P + j;
        p[o] = 0.f;
        if (i > 0 && i < n - 1 && j > 0 && j < n - 1) {
            const float* u = A.f[1];
            const float* v = A.f[2];
            float s = __fsub_rn(u[o + 1], u[o - 1]);
            s = __fadd_rn(s, v[o + P]);
            s = __fsub_rn(s, v[o - P]);
            A.dv[o] = __fmul_rn(__fmul_rn(-0.5f, A.h), s);
        }
    }
}

// remove_p (fluid_solver_cpu.cpp:205-210) on the interior.
__global__ void gs_remove_p_kernel(const GsArgs A, const float* __restrict__ p) {
    const int n = A.n, P = A.P, m = n - 2;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < (long)m * m; e += (long)gridDim.x * blockDim.x) {
        const size_t o = (size_t)(1 + e / m) * P + 1 + e % m;
        float* u = A.f[1];
        float* v = A.f[2];
        u[o] = __fsub_rn(u[o], __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(p[o + 1], p[o - 1])), A.h));
        v[o] = __fsub_rn(v[o], __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(p[o + P], p[o - P])), A.h));
    }
}

// advect(trace=false) of u and v by the copies (su, sv) on the interior
// (fluid_solver_cpu.cpp:154-173).
__global__ void gs_gather_grid_kernel(const GsArgs A) {
    const int n = A.n, P = A.P, m = n - 2;
    const float hi = (float)n - 1.5f;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < (long)m * m; e += (long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(e / m), j = 1 + (int)(e % m);
        const size_t o = (size_t)i * P + j;
        float x = __fsub_rn((float)j, __fmul_rn(A.dt0, A.su[o]));
        float y = __fsub_rn((float)i, __fmul_rn(A.dt0, A.sv[o]));
        x = (x < hi) ? x : hi;
        x = (1.5f < x) ? x : 1.5f;
        y = (y < hi) ? y : hi;
        y = (1.5f < y) ? y : 1.5f;
        const int j0 = (int)x, i0 = (int)y;
        const float s0 = __fsub_rn(x, (float)j0), s1 = __fsub_rn(1.f, s0);
        const float s2 = __fsub_rn(y, (float)i0), s3 = __fsub_rn(1.f, s2);
        const size_t a = (size_t)i0 * P + j0;
        for (int k = 0; k < 2; ++k) {
            const float* g0 = k == 0 ? A.su : A.sv;
            const float top = __fadd_rn(__fmul_rn(s1, g0[a]), __fmul_rn(s0, g0[a + 1]));
            const float bot = __fadd_rn(__fmul_rn(s1, g0[a + P]), __fmul_rn(s0, g0[a + P + 1]));
            A.f[1 + k][o] = __fadd_rn(__fmul_rn(s3, top), __fmul_rn(s2, bot));
        }
    }
}

// The splat by target (gs_splat_gather) over every target block; when some source
// moves more than kGatherMaxDTiled cells, one CTA applies the contributions in the raster
// order of their sources into the global accumulator instead.
constexpr int kGatherMaxDTiled = 40;
__global__ void __launch_bounds__(kGsThreads) gs_splat_grid_kernel(const GsArgs A) {
    const float dm = fmaxf(__ldcg(A.dmax), __ldcg(A.dmax + 1));
    if (dm <= (float)kGatherMaxDTiled) {
        gs_splat_gather(A, blockIdx.x, (int)ceilf(dm));
        return;
    }
    if (blockIdx.x != 0) return;
    const int n = A.n, P = A.P, m = n - 2;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) A.acc[(size_t)(1 + e / m) * P + 1 + e % m] = 0.f;
    __syncthreads();
    if (threadIdx.x != 0) return;
    const float hi = (float)n - 1.5f;
    for (int i = 1; i < n - 1; ++i)
        for (int j = 1; j < n - 1; ++j) {
            const size_t o = (size_t)i * P + j;
            const float x = __fadd_rn((float)j, __fmul_rn(A.dt0, A.su[o]));
            const float y = __fadd_rn((float)i, __fmul_rn(A.dt0, A.sv[o]));
            if (!(x >= 0.5f && x <= hi && y >= 0.5f && y <= hi)) continue;
            const int j0 = (int)x, i0 = (int)y;
            const float s0 = __fsub_rn(x, (float)j0), s1 = __fsub_rn(1.f, s0);
            const float s2 = __fsub_rn(y, (float)i0), s3 = __fsub_rn(1.f, s2);
            const float w = A.f[0][o];
            float* t = A.acc + (size_t)i0 * P + j0;
            // the accumulator's edge cells are never read back (the density takes its
            // interior, then the fill), so every target can be added to
            t[0] = __fadd_rn(t[0], __fmul_rn(__fmul_rn(s1, s3), w));
            t[P] = __fadd_rn(t[P], __fmul_rn(__fmul_rn(s1, s2), w));
            t[1] = __fadd_rn(t[1], __fmul_rn(__fmul_rn(s0, s3), w));
            t[P + 1] = __fadd_rn(t[P + 1], __fmul_rn(__fmul_rn(s0, s2), w));
        }
}

// d = the splat result on the interior (the fill follows).
__global__ void gs_take_acc_kernel(const GsArgs A) {
    const int n = A.n, P = A.P, m = n - 2;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < (long)m * m; e += (long)gridDim.x * blockDim.x) {
        const size_t o = (size_t)(1 + e / m) * P + 1 + e % m;
        A.f[0][o] = A.acc[o];
    }
}

int g_tiled_blocks[64] = {};  // co-resident CTAs of gs_tiled_kernel per device (set-up)

cudaError_t gs_solve_tiled(const GsTiled& S, bool diff, cudaStream_t st) {
    if (S.iters <= 0) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int m = S.n - 2, NT = (m + kTile - 1) / kTile;
    const int want = NT * std::min(NT, S.iters);  // most tiles of one wavefront time
    const int blocks = std::max(1, std::min(g_tiled_blocks[dev & 63], want));
    e = cudaMemsetAsync(S.ctrl, 0, sizeof(SolveCtrl), st);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kTileThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return diff ? cudaLaunchKernelEx(&cfg, gs_tiled_kernel<true>, S) : cudaLaunchKernelEx(&cfg, gs_tiled_kernel<false>, S);
}

int grid_blocks(long work, int threads) { return (int)std::max<long>(1, std::min<long>((work + threads - 1) / threads, 4096)); }

// A step of the host solver's method on a grid too large for the one-CTA form: the
// same order of operations (fluid_solver_cpu.cpp:6-31), each solve a tiled cooperative
// launch, the rest grid-wide kernels.
cudaError_t gs_step_tiled(const GsFields& F, const GsArgs& A, cudaStream_t st) {
    const int n = A.n, P = A.P;
    const long cells = (long)n * n;
    const int B = grid_blocks(cells, 256);
    const int modes[3] = {BND_CONT, BND_OPP_H, BND_OPP_V};
    float* x0 = F.scratch[2];  // the divergence's buffer doubles as the diffusion's x0
    float* p = F.scratch[4];
    cudaError_t e = cudaMemsetAsync(A.dmax, 0, 2 * sizeof(float), st);
    if (e != cudaSuccess) return e;
    gs_copy_vel_kernel<<<B, 256, 0, st>>>(A);
    auto diffuse = [&](int k) -> cudaError_t {
        gs_add_copy_kernel<<<B, 256, 0, st>>>(A.f[k], A.src[k], x0, n, P, A.dt);
        GsTiled S{A.f[k], x0, n, P, A.kd, modes[k], A.a[k], A.den[k], F.ctrl, F.poll_limit};
        cudaError_t r = gs_solve_tiled(S, true, st);
        if (r == cudaSuccess && A.kd > 0) gs_fill_kernel<<<1, kGsThreads, 0, st>>>(A.f[k], n, P, modes[k]);
        return r == cudaSuccess ? cudaGetLastError() : r;
    };
    auto project = [&]() -> cudaError_t {
        gs_div_kernel<<<B, 256, 0, st>>>(A, p);
        GsTiled S{p, A.dv, n, P, A.kp, BND_CONT, 0.f, 0.f, F.ctrl, F.poll_limit};
        cudaError_t r = gs_solve_tiled(S, false, st);
        if (r != cudaSuccess) return r;
        if (A.kp > 0) gs_fill_kernel<<<1, kGsThreads, 0, st>>>(p, n, P, BND_CONT);
        gs_remove_p_kernel<<<B, 256, 0, st>>>(A, p);
        gs_fill_kernel<<<1, kGsThreads, 0, st>>>(A.f[1], n, P, BND_OPP_H);
        gs_fill_kernel<<<1, kGsThreads, 0, st>>>(A.f[2], n, P, BND_OPP_V);
        return cudaGetLastError();
    };
    if ((e = diffuse(0)) != cudaSuccess) return e;
    const int target_blocks = (int)(((long)(n - 2) * (n - 2) + kGsThreads - 1) / kGsThreads);
    gs_splat_grid_kernel<<<target_blocks, kGsThreads, 0, st>>>(A);
    gs_take_acc_kernel<<<B, 256, 0, st>>>(A);
    gs_fill_kernel<<<1, kGsThreads, 0, st>>>(A.f[0], n, P, BND_CONT);
    if ((e = diffuse(1)) != cudaSuccess) return e;
    if ((e = diffuse(2)) != cudaSuccess) return e;
    if ((e = project()) != cudaSuccess) return e;
    gs_copy_vel_kernel<<<B, 256, 0, st>>>(A);  // copies for the velocity advection
    gs_gather_grid_kernel<<<B, 256, 0, st>>>(A);
    gs_fill_kernel<<<1, kGsThreads, 0, st>>>(A.f[1], n, P, BND_OPP_H);
    gs_fill_kernel<<<1, kGsThreads, 0, st>>>(A.f[2], n, P, BND_OPP_V);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return project();
}

}  // namespace

int gs_max_size() {
    int dev = 0, smem = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
    int n = 3;
    while (gs_smem_bytes(n + 1) <= (size_t)smem) ++n;
    return n;
}

int gs_tiled_max_size() { return 16384; }

cudaError_t gs_prepare() {
    // the largest size, so that handles of different sizes share one setting
    const int n = gs_max_size();
    if (n < 3) return cudaErrorNoDevice;
    {
        int dev = 0, sms = 0, per = 0;
        cudaError_t r = cudaGetDevice(&dev);
        if (r == cudaSuccess) r = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (r == cudaSuccess)
            r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, gs_tiled_kernel<true>, kTileThreads, 0);
        int per2 = 0;
        if (r == cudaSuccess)
            r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, gs_tiled_kernel<false>, kTileThreads, 0);
        if (r != cudaSuccess) return r;
        g_tiled_blocks[dev & 63] = std::min(per, per2) * sms;
    }
    const int bytes = (int)gs_smem_bytes(n);
    cudaError_t e = cudaFuncSetAttribute(gs_diffuse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(gs_splat_project_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(gs_project_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e;
}

cudaError_t gs_step(const GsFields& F, int n, int pitch, int kd, int kp, float diff, float visc, float dt,
                    cudaStream_t st, int* launches) {
    GsArgs A;
    A.f[0] = F.d;
    A.f[1] = F.u;
    A.f[2] = F.v;
    A.src[0] = F.ds;
    A.src[1] = F.us;
    A.src[2] = F.vs;
    A.su = F.scratch[0];
    A.sv = F.scratch[1];
    A.dv = F.scratch[2];
    A.acc = F.scratch[3];
    A.dmax = F.aux;
    A.n = n;
    A.P = pitch;
    A.kd = kd;
    A.kp = kp;
    // constants as the host solver computes them, in float (fluid_solver_cpu.cpp:97-98,
    // 119, 181): a = dt * (rows*cols) * rate, den = 1 + 4a, dt0 = sqrt(rows*cols) * dt
    const float cells = (float)((size_t)n * (size_t)n);
    const float rates[3] = {diff, visc, visc};
    for (int k = 0; k < 3; ++k) {
        A.a[k] = dt * cells * rates[k];
        A.den[k] = 1.f + 4.f * A.a[k];  // 4a is exact, so a fused form rounds the same
    }
    A.dt = dt;
    A.dt0 = sqrtf(cells) * dt;
    A.h = 1.0f / sqrtf(cells);
    if (n > gs_max_size()) {
        *launches = 29;
        return gs_step_tiled(F, A, st);
    }
    *launches = 4;
    const size_t smem = gs_smem_bytes(n);
    gs_diffuse_kernel<<<3, kGsThreads, smem, st>>>(A);
    const int target_blocks = ((n - 2) * (n - 2) + kGsThreads - 1) / kGsThreads;
    gs_splat_project_kernel<<<2 + target_blocks, kGsThreads, smem, st>>>(A);
    gs_gather_kernel<<<2, kGsThreads, 0, st>>>(A);
    gs_project_kernel<<<1, kGsThreads, smem, st>>>(A);
    return cudaGetLastError();
}

}  // namespace fs
