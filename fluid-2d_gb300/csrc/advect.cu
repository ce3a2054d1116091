// Semi-Lagrangian advection kernels.
//
// Reference behaviour (mworchel/fluid-2d src/fluid_solver_gpu.cu):
//   density  advect(trace=true) 325-356: D2D copy, memset, advect_trace_kernel
//            131-162 (forward bilinear splat with fp32 atomicAdd), Neumann fill,
//            then smooth 314-323 (D2D copy + smooth_kernel 87-97, no fill);
//   velocity two advect(trace=false) calls 248-251 on copies u0, v0 with
//            advect_kernel 99-129 (backtrace, clamp, bilinear gather), each followed
//            by its reflecting fill.
// Here the density path is three launches with no copies: a memset of the
// accumulator, the splat, and one "finish" kernel that applies the Neumann fill and
// the smoothing together. The velocity path is one kernel that backtraces once per
// cell and gathers u and v together, writing the reflecting edges directly.
//
// Operand order and rounding follow the reference expressions as its compiled kernels
// evaluate them: explicit _rn intrinsics, with a fused multiply-add exactly where nvcc
// fuses the reference source (the positions j +- dt0*u and, in the gather, the bilinear
// sum as s3*fma(s0, B, s1*A) + s2*fma(s0, D, s1*C), fused at the first product). These
// fusions were found by comparing the reference's compiled kernels with candidate
// restatements bit for bit. The splat order of the atomics is unspecified, as in the
// reference.

#include <algorithm>

#include "fs_internal.cuh"

namespace fs {
namespace {

// Forward splat of interior source cell (i, j), advect_trace_kernel
// (fluid_solver_gpu.cu:141-159).
__device__ __forceinline__ void splat_cell(const float* __restrict__ d0, const float* __restrict__ u,
                                           const float* __restrict__ v, float* __restrict__ acc, const AdvectArgs& A,
                                           int i, int j) {
    const size_t P = (size_t)A.pitch;
    const size_t o = (size_t)i * P + j;
    const float x = __fmaf_rn(A.dt0, __ldg(u + o), (float)j);
    const float y = __fmaf_rn(A.dt0, __ldg(v + o), (float)i);
    // skipped unless inside [0.5, n-1.5] (fluid_solver_gpu.cu:144); NaN is skipped too
    if (!(x >= 0.5f && x <= A.xmax && y >= 0.5f && y <= A.ymax)) return;
    const int j0 = (int)x, i0 = (int)y;
    const float s0 = __fsub_rn(x, (float)j0), s1 = __fsub_rn(1.f, s0);
    const float s2 = __fsub_rn(y, (float)i0), s3 = __fsub_rn(1.f, s2);
    const float d = __ldg(d0 + o);
    float* t = acc + (size_t)i0 * P + j0;
    atomicAdd(t, __fmul_rn(__fmul_rn(s1, s3), d));
    atomicAdd(t + P, __fmul_rn(__fmul_rn(s1, s2), d));
    atomicAdd(t + 1, __fmul_rn(__fmul_rn(s0, s3), d));
    atomicAdd(t + P + 1, __fmul_rn(__fmul_rn(s0, s2), d));
}

// Value of the accumulator after set_boundary_continuous (fluid_solver_gpu.cu:11-24):
// edges read their inner neighbour, corners and the interior read themselves.
__device__ __forceinline__ float filled(const float* __restrict__ acc, int r, int c, const AdvectArgs& A) {
    const bool ri = r >= 1 && r <= A.rows - 2, ci = c >= 1 && c <= A.cols - 2;
    if (ri && !ci) c = (c == 0) ? 1 : A.cols - 2;
    else if (ci && !ri) r = (r == 0) ? 1 : A.rows - 2;
    return __ldg(acc + (size_t)r * A.pitch + c);
}

// Neumann fill of the splat result plus smooth_kernel (fluid_solver_gpu.cu:94) for
// cell (i, j); returns 1 if the value is not finite.
__device__ __forceinline__ int finish_cell(const float* __restrict__ acc, float* __restrict__ d, int smooth,
                                           const AdvectArgs& A, int i, int j) {
    float out = filled(acc, i, j, A);
    if (smooth && i >= 1 && i <= A.rows - 2 && j >= 1 && j <= A.cols - 2) {
        // 0.2f * (c + l + r + u + d)
        float s = __fadd_rn(out, filled(acc, i, j - 1, A));
        s = __fadd_rn(s, filled(acc, i, j + 1, A));
        s = __fadd_rn(s, filled(acc, i - 1, j, A));
        s = __fadd_rn(s, filled(acc, i + 1, j, A));
        out = __fmul_rn(0.2f, s);
    }
    d[(size_t)i * A.pitch + j] = out;
    return !isfinite(out);
}

// Backtrace advection of u and v for cell (i, j), advect_kernel
// (fluid_solver_gpu.cu:111-126), with the reflecting fills for edge cells.
__device__ __forceinline__ void advect_cell(const float* __restrict__ u0, const float* __restrict__ v0,
                                            float* __restrict__ u, float* __restrict__ v, const AdvectArgs& A, int i,
                                            int j) {
    const size_t P = (size_t)A.pitch;
    const bool ri = i >= 1 && i <= A.rows - 2, ci = j >= 1 && j <= A.cols - 2;
    const size_t o = (size_t)i * P + j;
    if (!ri && !ci) {  // corners are never written by the reference
        u[o] = __ldg(u0 + o);
        v[o] = __ldg(v0 + o);
        return;
    }
    // Edge cells copy the advected inner neighbour: u is negated on the left/right
    // edges, v on the top/bottom edges (fluid_solver_gpu.cu:26-54).
    int si = i, sj = j;
    float su = 1.f, sv = 1.f;
    if (!ci) {
        sj = (j == 0) ? 1 : A.cols - 2;
        su = -1.f;
    } else if (!ri) {
        si = (i == 0) ? 1 : A.rows - 2;
        sv = -1.f;
    }
    const size_t so = (size_t)si * P + sj;
    float x = __fmaf_rn(-A.dt0, __ldg(u0 + so), (float)sj);
    float y = __fmaf_rn(-A.dt0, __ldg(v0 + so), (float)si);
    x = fmaxf(1.5f, fminf(A.xmax, x));
    y = fmaxf(1.5f, fminf(A.ymax, y));
    const int j0 = (int)x, i0 = (int)y;
    const float s0 = __fsub_rn(x, (float)j0), s1 = __fsub_rn(1.f, s0);
    const float s2 = __fsub_rn(y, (float)i0), s3 = __fsub_rn(1.f, s2);
    const size_t q = (size_t)i0 * P + j0;
    const float ua = __ldg(u0 + q), ub = __ldg(u0 + q + 1), uc = __ldg(u0 + q + P), ud = __ldg(u0 + q + P + 1);
    const float va = __ldg(v0 + q), vb = __ldg(v0 + q + 1), vc = __ldg(v0 + q + P), vd = __ldg(v0 + q + P + 1);
    const float ut = __fmaf_rn(s0, ub, __fmul_rn(s1, ua));
    const float ubm = __fmaf_rn(s0, ud, __fmul_rn(s1, uc));
    const float vt = __fmaf_rn(s0, vb, __fmul_rn(s1, va));
    const float vbm = __fmaf_rn(s0, vd, __fmul_rn(s1, vc));
    u[o] = su * __fmaf_rn(s3, ut, __fmul_rn(s2, ubm));
    v[o] = sv * __fmaf_rn(s3, vt, __fmul_rn(s2, vbm));
}

__global__ void __launch_bounds__(256) splat_kernel(const float* __restrict__ d0, const float* __restrict__ u,
                                                    const float* __restrict__ v, float* __restrict__ acc,
                                                    const AdvectArgs A) {
    for (int i = blockIdx.y * blockDim.y + threadIdx.y + 1; i < A.rows - 1; i += blockDim.y * gridDim.y)
        for (int j = blockIdx.x * blockDim.x + threadIdx.x + 1; j < A.cols - 1; j += blockDim.x * gridDim.x)
            splat_cell(d0, u, v, acc, A, i, j);
}

__global__ void __launch_bounds__(256) density_finish_kernel(const float* __restrict__ acc, float* __restrict__ d,
                                                             int smooth, const AdvectArgs A, int* nonfinite) {
    int bad = 0;
    for (int i = blockIdx.y * blockDim.y + threadIdx.y; i < A.rows; i += blockDim.y * gridDim.y)
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < A.cols; j += blockDim.x * gridDim.x)
            bad |= finish_cell(acc, d, smooth, A, i, j);
    if (bad && nonfinite) atomicOr(nonfinite, 1);
}

__global__ void __launch_bounds__(256) advect_velocity_kernel(const float* __restrict__ u0,
                                                              const float* __restrict__ v0, float* __restrict__ u,
                                                              float* __restrict__ v, const AdvectArgs A) {
    for (int i = blockIdx.y * blockDim.y + threadIdx.y; i < A.rows; i += blockDim.y * gridDim.y)
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < A.cols; j += blockDim.x * gridDim.x)
            advect_cell(u0, v0, u, v, A, i, j);
}

// ----------------------------------------------------------------- batched
// One launch covers every grid of a batch: blocks of 32x8 threads each cover 32x32
// cells (four rows per thread, so a large grid needs a quarter of the blocks one cell
// per thread would), numbered grid by grid (prefix[g] = first block of grid g,
// block_job[b] = grid of block b).
constexpr int kBatchRows = 32;

template <int OP>
__global__ void __launch_bounds__(256) advect_batch_kernel(const AdvectJob* __restrict__ jobs,
                                                           const int* __restrict__ prefix,
                                                           const int* __restrict__ block_job, int* nonfinite) {
    const int b = blockIdx.x;
    const int g = __ldg(block_job + b);
    const AdvectJob& J = jobs[g];
    const int lb = b - __ldg(prefix + g);
    const int bx = (J.A.cols + 31) / 32;
    const int j = (lb % bx) * 32 + threadIdx.x;
    int bad = 0;
#pragma unroll
    for (int r = 0; r < kBatchRows; r += 8) {
        const int i = (lb / bx) * kBatchRows + r + threadIdx.y;
        if (OP == 0) {
            if (i >= 1 && i < J.A.rows - 1 && j >= 1 && j < J.A.cols - 1)
                splat_cell(J.in0, J.in1, J.in2, J.out0, J.A, i, j);
        } else if (OP == 1) {
            if (i < J.A.rows && j < J.A.cols) bad |= finish_cell(J.in0, J.out0, J.smooth, J.A, i, j);
        } else {
            if (i < J.A.rows && j < J.A.cols) advect_cell(J.in0, J.in1, J.out0, J.out1, J.A, i, j);
        }
    }
    if (bad && nonfinite) atomicOr(nonfinite, 1);
}

dim3 grid_for(int rows, int cols) {
    const int gx = (cols + 31) / 32;
    int gy = (rows + 7) / 8;
    // cap the grid (grid-stride loops) at a few waves of 152 SMs x 8 CTAs
    const long cap = 152L * 8 * 8;
    if ((long)gx * gy > cap) gy = (int)((cap + gx - 1) / gx);
    if (gy < 1) gy = 1;
    return dim3(gx, gy);
}

}  // namespace

cudaError_t launch_splat(const float* d0, const float* u, const float* v, float* acc, const AdvectArgs& A,
                         cudaStream_t st) {
    splat_kernel<<<grid_for(A.rows, A.cols), dim3(32, 8), 0, st>>>(d0, u, v, acc, A);
    return cudaGetLastError();
}

cudaError_t launch_density_finish(const float* acc, float* d, int smooth, const AdvectArgs& A, int* nonfinite,
                                  cudaStream_t st) {
    density_finish_kernel<<<grid_for(A.rows, A.cols), dim3(32, 8), 0, st>>>(acc, d, smooth, A, nonfinite);
    return cudaGetLastError();
}

cudaError_t launch_advect_velocity(const float* u0, const float* v0, float* u, float* v, const AdvectArgs& A,
                                   cudaStream_t st) {
    advect_velocity_kernel<<<grid_for(A.rows, A.cols), dim3(32, 8), 0, st>>>(u0, v0, u, v, A);
    return cudaGetLastError();
}

int advect_batch_blocks(int rows, int cols) { return ((cols + 31) / 32) * ((rows + kBatchRows - 1) / kBatchRows); }

cudaError_t launch_advect_batch(int op, const AdvectJob* jobs, const int* prefix, const int* block_job, int nblocks,
                                int* nonfinite, cudaStream_t st) {
    if (nblocks <= 0) return cudaSuccess;
    if (op == 0)
        advect_batch_kernel<0><<<nblocks, dim3(32, 8), 0, st>>>(jobs, prefix, block_job, nonfinite);
    else if (op == 1)
        advect_batch_kernel<1><<<nblocks, dim3(32, 8), 0, st>>>(jobs, prefix, block_job, nonfinite);
    else
        advect_batch_kernel<2><<<nblocks, dim3(32, 8), 0, st>>>(jobs, prefix, block_job, nonfinite);
    return cudaGetLastError();
}

}  // namespace fs
