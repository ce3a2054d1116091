// Elementwise, pooling, gradient and optimizer kernels of the learned pressure warm
// start, and the fine <-> coarse transfers that connect it to the pressure solve.
//
// The network runs on a coarse grid (G x G cells, G = FS_NET_GRID): each coarse cell
// covers an R x R block of the fine interior (R = N / G). Its input is the block sum of
// the Poisson residual of the current pressure; its output is the block mean of the
// correction that solves the residual equation, L_c e_c = block sums of r, so a network
// trained at one fine size applies to others and to any starting pressure. Activations are NHWC with 32 channels; gradients are FP32.
//
// No counterpart in the reference (it has no learned component).

#include <cuda_bf16.h>
#include <algorithm>
#include <cuda_runtime.h>

#include "../../include/fluid2d_gb300.h"
#include "fs_internal.cuh"

namespace fs {
namespace {

constexpr int kC = 32;

inline int blocks_for(long n, int t) { return (int)((n + t - 1) / t); }

// ---------------------------------------------------------------- pooling
// 2x2 average pool, BF16 NHWC: out rows = rows/2, cols = W/2.
__global__ void avgpool2_kernel(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ y, int rows_out,
                                int w_out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;  // (pixel, channel)
    if (i >= (long)rows_out * w_out * kC) return;
    const int c = (int)(i % kC);
    const long p = i / kC;
    const int Y = (int)(p / w_out), X = (int)(p % w_out);
    const int W = 2 * w_out;
    const long a = ((long)(2 * Y) * W + 2 * X) * kC + c;
    const float s = __bfloat162float(x[a]) + __bfloat162float(x[a + kC]) + __bfloat162float(x[a + (long)W * kC]) +
                    __bfloat162float(x[a + (long)W * kC + kC]);
    y[i] = __float2bfloat16_rn(0.25f * s);
}

// Backward of the 2x2 average pool: dx[y][x] = dy[y/2][x/2] / 4 (FP32).
__global__ void avgpool2_bwd_kernel(const float* __restrict__ dy, float* __restrict__ dx, int rows_in, int w_in) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)rows_in * w_in * kC) return;
    const int c = (int)(i % kC);
    const long p = i / kC;
    const int y = (int)(p / w_in), x = (int)(p % w_in);
    dx[i] = 0.25f * dy[((long)(y >> 1) * (w_in >> 1) + (x >> 1)) * kC + c];
}

// Backward of the nearest 2x upsample: dlow[Y][X] = sum of dup over its 2x2 block.
__global__ void upsample2_bwd_kernel(const float* __restrict__ dup, float* __restrict__ dlow, int rows_low,
                                     int w_low) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)rows_low * w_low * kC) return;
    const int c = (int)(i % kC);
    const long p = i / kC;
    const int Y = (int)(p / w_low), X = (int)(p % w_low);
    const int W = 2 * w_low;
    const long a = ((long)(2 * Y) * W + 2 * X) * kC + c;
    dlow[i] = dup[a] + dup[a + kC] + dup[a + (long)W * kC] + dup[a + (long)W * kC + kC];
}

// dz = da * (a > 0) (ReLU backward through the layer output a), plus an optional
// extra gradient (skip branch) added first; writes FP32 and a BF16 copy.
__global__ void relu_bwd_kernel(const float* __restrict__ da, const float* __restrict__ da2,
                                const __nv_bfloat16* __restrict__ a, float* __restrict__ dz,
                                __nv_bfloat16* __restrict__ dzb, long n, int relu) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g = da[i] + (da2 ? da2[i] : 0.f);
    if (relu && !(__bfloat162float(a[i]) > 0.f)) g = 0.f;
    dz[i] = g;
    dzb[i] = __float2bfloat16_rn(g);
}

// ------------------------------------------------------------- weight gradient
// dW[co][t][ci] += sum_p dz[p][co] * x(p, tap t)[ci]; db[co] += sum_p dz[p][co].
// CUDA cores: a CTA stages 64 pixels' dz rows and im2col rows in shared memory and
// each of 256 threads accumulates 36 weights (one co, 36 consecutive k) in registers,
// then adds them to the FP32 gradient with atomics once per CTA.
constexpr int kWgPix = 64;
__global__ void __launch_bounds__(256) weight_grad_kernel(const float* __restrict__ dz,
                                                          const __nv_bfloat16* __restrict__ x, float* __restrict__ dw,
                                                          float* __restrict__ db, int H, int W, int img_h, int up,
                                                          int pix_per_cta) {
    __shared__ float zs[kWgPix][kC];
    __shared__ __nv_bfloat16 xs[kWgPix][9 * kC + 8];
    const int tid = threadIdx.x;
    const int co = tid >> 3, k0 = (tid & 7) * 36;
    float acc[36];
#pragma unroll
    for (int j = 0; j < 36; ++j) acc[j] = 0.f;
    float bacc = 0.f;
    const long npix = (long)H * W;
    const long pbeg = (long)blockIdx.x * pix_per_cta;
    const long pend = min(npix, pbeg + pix_per_cta);
    for (long c0 = pbeg; c0 < pend; c0 += kWgPix) {
        __syncthreads();
        for (int e = tid; e < kWgPix * kC; e += 256) {
            const int m = e / kC, c = e % kC;
            const long p = c0 + m;
            zs[m][c] = p < pend ? dz[p * kC + c] : 0.f;
        }
        for (int e = tid; e < kWgPix * 9 * kC; e += 256) {
            const int m = e / (9 * kC), k = e % (9 * kC);
            const int t = k / kC, ci = k % kC;
            const long p = c0 + m;
            __nv_bfloat16 v = __float2bfloat16_rn(0.f);
            if (p < pend) {
                const int y = (int)(p / W), xx = (int)(p % W);
                const int ly = y % img_h + t / 3 - 1, ix = xx + t % 3 - 1;
                if (ly >= 0 && ly < img_h && ix >= 0 && ix < W) {
                    const int iy = y + t / 3 - 1;
                    const long src = up ? (long)(iy >> 1) * (W >> 1) + (ix >> 1) : (long)iy * W + ix;
                    v = x[src * kC + ci];
                }
            }
            xs[m][k] = v;
        }
        __syncthreads();
        for (int m = 0; m < kWgPix; ++m) {
            const float z = zs[m][co];
            if ((tid & 7) == 0) bacc += z;
#pragma unroll
            for (int j = 0; j < 36; ++j) acc[j] = fmaf(z, __bfloat162float(xs[m][k0 + j]), acc[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < 36; ++j) atomicAdd(dw + co * 9 * kC + k0 + j, acc[j]);
    if ((tid & 7) == 0 && db) atomicAdd(db + co, bacc);
}

// Weights of the backward-data convolution: w'[ci][t][co] = w[co][8 - t][ci].
__global__ void flip_weights_kernel(const float* __restrict__ w, float* __restrict__ wt) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kC * 9 * kC) return;
    const int co = e / (9 * kC), t = (e / kC) % 9, ci = e % kC;
    wt[(ci * 9 + (8 - t)) * kC + co] = w[e];
}

// ------------------------------------------------------------------ loss
// Mean squared error on channel 0 against a target (n pixels): dy = 2 (y - t) / n on
// channel 0, zero elsewhere; the per-CTA partial sums of (y - t)^2 go to loss_part.
__global__ void mse_kernel(const float* __restrict__ y, const float* __restrict__ target, float* __restrict__ dy,
                           float* __restrict__ loss_part, long n) {
    __shared__ float red[256];
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    float e2 = 0.f;
    if (p < n) {
        const float e = y[p * kC] - target[p];
        e2 = e * e;
        dy[p * kC] = 2.f * e / (float)n;
#pragma unroll
        for (int c = 1; c < kC; ++c) dy[p * kC + c] = 0.f;
    }
    red[threadIdx.x] = e2;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0];
}

// ------------------------------------------------------------------ Adam
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, long n, float lr, float b1, float b2, float eps, float c1,
                            float c2, const unsigned char* __restrict__ frozen) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (frozen && frozen[i]) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// ------------------------------------------------------- fine <-> coarse
// Block sums of the Poisson residual r = div + sum(nbrs p) - 4p of a starting pressure
// p (pitched, edges filled; null = zero, r = div) over the fine interior 1..N: coarse
// cell (I, J) of the G x G grid covers an R x R block. One CTA per coarse cell writes
// the FP32 sum to bs[cell] and, when pc is given, the block MEAN of p to pc[cell].
// The coarse correction that makes p exact solves L_c e_c = bs, so the residual alone
// carries what the network needs from the divergence and the starting pressure.
__global__ void restrict_kernel(const float* __restrict__ div, const float* __restrict__ p, int pitch, int R, int G,
                                float* __restrict__ bs, float* __restrict__ pc, const int* __restrict__ skip_if) {
    if (skip_if && __ldcg(skip_if)) return;
    const int cell = blockIdx.x;
    const int I = cell / G, J = cell % G;
    float sr = 0.f, sp = 0.f;
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
        const int i = 1 + I * R + e / R, j = 1 + J * R + e % R;
        const size_t o = (size_t)i * pitch + j;
        float r = div[o];
        if (p) {
            const float c = p[o];
            r += (p[o - 1] + p[o + 1]) + (p[o - pitch] + p[o + pitch]) - 4.f * c;
            sp += c;
        }
        sr += r;
    }
    __shared__ float a[256], b[256];
    a[threadIdx.x] = sr;
    b[threadIdx.x] = sp;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            a[threadIdx.x] += a[threadIdx.x + s];
            b[threadIdx.x] += b[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        bs[cell] = a[0];
        if (pc) pc[cell] = b[0] / (float)(R * R);
    }
}

// Network input from the block sums (one CTA): scale = RMS of bs with a floor,
// channel 0 = bs / scale, channels 1..31 = 0 (xin nullable); *norm2 = sum of bs^2
// (nullable).
__global__ void coarse_input_kernel(const float* __restrict__ bs, int G, float* __restrict__ scale_out,
                                    __nv_bfloat16* __restrict__ xin, double* __restrict__ norm2,
                                    const int* __restrict__ skip_if) {
    if (skip_if && __ldcg(skip_if)) return;
    __shared__ double red[1024];
    __shared__ float s_scale;
    double acc = 0.0;
    for (int c = threadIdx.x; c < G * G; c += blockDim.x) acc += (double)bs[c] * bs[c];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        s_scale = (float)fmax(sqrt(red[0] / (double)(G * G)), 1e-30);
        if (scale_out) *scale_out = s_scale;
        if (norm2) *norm2 = red[0];
    }
    __syncthreads();
    if (!xin) return;
    const float inv = 1.f / s_scale;
    for (int e = threadIdx.x; e < G * G * kC; e += blockDim.x)
        xin[e] = __float2bfloat16_rn((e % kC) == 0 ? bs[e / kC] * inv : 0.f);
}

// Coarse post-smoothing of a coarse correction (one CTA, G*G <= 4096): e = y_in[.,0] *
// scale * kappa (y_in null: e = 0), then nu sweeps of e_I <- (1-w) e_I + w (bs_I + sum
// of the four neighbours) / 4, a missing neighbour reflecting e_I (Neumann), w = 0.8;
// the mean is removed (the coarse problem's null space) and y_out[.,0] = e / (scale *
// kappa) written (y_out may equal y_in). Applied to the network's output it removes the
// cell-to-cell error that the fine sweeps would otherwise damp slowly; applied to zero it
// is the classical coarse correction the network has to beat.
constexpr int kCoarseMax = 64;
constexpr int kSmoothThreads = 1024;
constexpr int kSmoothCells = kCoarseMax * kCoarseMax / kSmoothThreads;  // cells per thread
// One CTA per candidate (blockIdx.x selects a or b): nu weighted-Jacobi sweeps of the
// coarse equation in shared memory. Each thread keeps its cells' right-hand sides and
// neighbour offsets in registers (the edges reflect: a missing neighbour is the cell
// itself), so a sweep is five shared loads, the update and one store per cell.
__global__ void __launch_bounds__(kSmoothThreads) coarse_smooth_kernel(const float* y_in_a, float* y_out_a,
                                                                       const float* y_in_b, float* y_out_b,
                                                                       const float* __restrict__ bs,
                                                                       const float* __restrict__ scale_ptr,
                                                                       float kappa, int G, int nu,
                                                                       const int* __restrict__ skip_if) {
    if (skip_if && __ldcg(skip_if)) return;
    const float* y_in = blockIdx.x ? y_in_b : y_in_a;
    float* y_out = blockIdx.x ? y_out_b : y_out_a;
    if (!y_out) return;
    __shared__ float e[2][kCoarseMax * kCoarseMax];
    __shared__ double red[kSmoothThreads];
    const int tid = threadIdx.x, n = G * G;
    const float unit = (*scale_ptr) * kappa;
    for (int c = tid; c < n; c += kSmoothThreads) e[0][c] = y_in ? y_in[(size_t)c * kC] * unit : 0.f;
    float b[kSmoothCells];
    int up[kSmoothCells], dn[kSmoothCells], lf[kSmoothCells], rt[kSmoothCells];
#pragma unroll
    for (int k = 0; k < kSmoothCells; ++k) {
        const int c = tid + k * kSmoothThreads;
        const int I = c / G, J = c - (c / G) * G;
        const bool in = c < n;
        b[k] = in ? bs[c] : 0.f;
        up[k] = in && I > 0 ? c - G : c;
        dn[k] = in && I < G - 1 ? c + G : c;
        lf[k] = in && J > 0 ? c - 1 : c;
        rt[k] = in && J < G - 1 ? c + 1 : c;
    }
    __syncthreads();
    const float w = 0.8f;
    int cur = 0;
    for (int it = 0; it < nu; ++it) {
        const float* src = e[cur];
        float* dst = e[cur ^ 1];
#pragma unroll
        for (int k = 0; k < kSmoothCells; ++k) {
            const int c = tid + k * kSmoothThreads;
            if (c < n) {
                const float x = src[c];
                dst[c] = (1.f - w) * x + w * 0.25f * (b[k] + src[up[k]] + src[dn[k]] + src[lf[k]] + src[rt[k]]);
            }
        }
        __syncthreads();
        cur ^= 1;
    }
    double acc = 0.0;
    for (int c = tid; c < n; c += kSmoothThreads) acc += e[cur][c];
    red[tid] = acc;
    __syncthreads();
    for (int s = kSmoothThreads / 2; s > 0; s >>= 1) {
        if (tid < s) red[tid] += red[tid + s];
        __syncthreads();
    }
    const float mean = (float)(red[0] / (double)n);
    for (int c = tid; c < n; c += kSmoothThreads) y_out[(size_t)c * kC] = (e[cur][c] - mean) / unit;
}

// Fine warm start: p_out = p_prev + bilinear interpolation of the coarse correction
// (network channel 0 times scale * kappa) at fine cell centres, over the interior;
// edges take their inner neighbour (Neumann fill), corners keep p_prev.
__global__ void prolong_kernel(const float* __restrict__ y, const float* __restrict__ p_prev, float* __restrict__ p_out,
                               int rows, int cols, int pitch, int R, int G, const float* __restrict__ scale_ptr,
                               float kappa, const int* __restrict__ skip_if) {
    if (skip_if && __ldcg(skip_if)) return;
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)rows * cols) return;
    const int i = (int)(e / cols), j = (int)(e % cols);
    const bool ri = i >= 1 && i <= rows - 2, ci = j >= 1 && j <= cols - 2;
    int si = i, sj = j;
    if (ri && !ci) sj = (j == 0) ? 1 : cols - 2;
    else if (ci && !ri) si = (i == 0) ? 1 : rows - 2;
    else if (!ri && !ci) {
        p_out[(size_t)i * pitch + j] = p_prev ? p_prev[(size_t)i * pitch + j] : 0.f;
        return;
    }
    // coarse coordinate of fine interior cell (si, sj): centres at (I + 0.5) * R
    const float fy = ((si - 1) + 0.5f) / R - 0.5f, fx = ((sj - 1) + 0.5f) / R - 0.5f;
    const int y0 = max(0, min(G - 1, (int)floorf(fy))), x0 = max(0, min(G - 1, (int)floorf(fx)));
    const int y1 = min(G - 1, y0 + 1), x1 = min(G - 1, x0 + 1);
    const float wy = fminf(fmaxf(fy - y0, 0.f), 1.f), wx = fminf(fmaxf(fx - x0, 0.f), 1.f);
    const float c00 = y[((size_t)y0 * G + x0) * kC], c01 = y[((size_t)y0 * G + x1) * kC];
    const float c10 = y[((size_t)y1 * G + x0) * kC], c11 = y[((size_t)y1 * G + x1) * kC];
    const float corr = (1.f - wy) * ((1.f - wx) * c00 + wx * c01) + wy * ((1.f - wx) * c10 + wx * c11);
    const float base = p_prev ? p_prev[(size_t)si * pitch + sj] : 0.f;
    p_out[(size_t)i * pitch + j] = base + corr * (*scale_ptr) * kappa;
}


// Energy-norm gain of a candidate pressure p_try over p_cur: with c = p_try - p_cur and
// the residual r = div + sum(nbrs p_cur) - 4 p_cur, the error e = A^-1 r (A the Neumann
// 5-point operator, symmetric) changes by ||e - c||_A^2 = ||e||_A^2 - (2 c.r - c.Ac), so
// gain = 2 c.r - c.Ac (interior sums, FP64 partials) is exactly how much closer p_try is
// to the solution than p_cur in the norm the Jacobi iteration contracts. Accumulated
// into *out (zeroed before).
__global__ void energy_gain_kernel(const float* __restrict__ div, const float* __restrict__ p_cur,
                                   const float* __restrict__ p_try, int rows, int cols, int pitch,
                                   double* __restrict__ out, const int* __restrict__ skip_if) {
    if (skip_if && __ldcg(skip_if)) return;
    __shared__ double red[256];
    float g = 0.f;  // a thread's few cells; the CTA and grid sums are in FP64
    const int j = blockIdx.x * 256 + threadIdx.x;
    if (j >= 1 && j <= cols - 2) {
        for (int i = 1 + blockIdx.y; i <= rows - 2; i += gridDim.y) {
            const size_t o = (size_t)i * pitch + j;
            const float pc = p_cur[o];
            const float r = div[o] + (p_cur[o - 1] + p_cur[o + 1]) + (p_cur[o - pitch] + p_cur[o + pitch]) - 4.f * pc;
            const float c = p_try[o] - pc;
            const float cl = p_try[o - 1] - p_cur[o - 1], cr = p_try[o + 1] - p_cur[o + 1];
            const float cu = p_try[o - pitch] - p_cur[o - pitch], cd = p_try[o + pitch] - p_cur[o + pitch];
            const float ac = 4.f * c - ((cl + cr) + (cu + cd));
            g += 2.f * c * r - c * ac;
        }
    }
    red[threadIdx.x] = g;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(out, red[0]);
}

// One damped Jacobi step, p_out = p + (J(p) - p) / 2 with J(p) = (div + sum(nbrs p)) / 4,
// on the interior, edges from their inner neighbour's new value (Neumann fill), corners
// copied. Plain Jacobi never damps the checkerboard mode (its amplification is -1 on a
// Neumann grid), so rounding noise in that mode piles up over thousands of sweeps and
// sets a floor on the relative residual once the divergence is small; this step removes
// the mode exactly and reduces every other error mode in the A-norm.
__device__ __forceinline__ float damped_cell(const float* __restrict__ div, const float* __restrict__ p, size_t o,
                                             int pitch) {
    const float j = 0.25f * (div[o] + (p[o - 1] + p[o + 1]) + (p[o - pitch] + p[o + pitch]));
    return 0.5f * (p[o] + j);
}

__global__ void damp_kernel(const float* __restrict__ div, const float* __restrict__ p, float* __restrict__ out,
                            int rows, int cols, int pitch, const int* __restrict__ skip_if) {
    if (skip_if && __ldcg(skip_if)) return;
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)rows * cols) return;
    const int i = (int)(e / cols), j = (int)(e % cols);
    const bool ri = i >= 1 && i <= rows - 2, ci = j >= 1 && j <= cols - 2;
    const size_t o = (size_t)i * pitch + j;
    if (!ri && !ci) {
        out[o] = p[o];
        return;
    }
    const int si = ri ? i : (i == 0 ? 1 : rows - 2), sj = ci ? j : (j == 0 ? 1 : cols - 2);
    out[o] = damped_cell(div, p, (size_t)si * pitch + sj, pitch);
}

// Block sums on a G x G grid from those on the 2G x 2G grid (sum of the four children).
__global__ void coarse_sum2x2_kernel(const float* __restrict__ fine, float* __restrict__ coarse, int G,
                                     const int* __restrict__ skip_if) {
    if (skip_if && __ldcg(skip_if)) return;
    const int G2 = 2 * G;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < G * G; c += gridDim.x * blockDim.x) {
        const int I = c / G, J = c % G;
        const float* f = fine + (size_t)(2 * I) * G2 + 2 * J;
        coarse[c] = (f[0] + f[1]) + (f[G2] + f[G2 + 1]);
    }
}

// A coarse correction on the G x G grid (channel 0 of y, times scale * kappa) carried
// to the 2G x 2G grid by bilinear interpolation at the finer cell centres, in absolute
// units, into channel 0 of e (stride 32, the layout the smoothing and prolongation use).
__global__ void coarse_interp_kernel(const float* __restrict__ y, float* __restrict__ e, int G,
                                     const float* __restrict__ scale_ptr, float kappa,
                                     const int* __restrict__ skip_if) {
    if (skip_if && __ldcg(skip_if)) return;
    const int G2 = 2 * G;
    const float unit = (*scale_ptr) * kappa;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < G2 * G2; c += gridDim.x * blockDim.x) {
        const int I = c / G2, J = c % G2;
        const float fy = (I + 0.5f) * 0.5f - 0.5f, fx = (J + 0.5f) * 0.5f - 0.5f;
        const int y0 = max(0, min(G - 1, (int)floorf(fy))), x0 = max(0, min(G - 1, (int)floorf(fx)));
        const int y1 = min(G - 1, y0 + 1), x1 = min(G - 1, x0 + 1);
        const float wy = fminf(fmaxf(fy - y0, 0.f), 1.f), wx = fminf(fmaxf(fx - x0, 0.f), 1.f);
        const float c00 = y[((size_t)y0 * G + x0) * kC], c01 = y[((size_t)y0 * G + x1) * kC];
        const float c10 = y[((size_t)y1 * G + x0) * kC], c11 = y[((size_t)y1 * G + x1) * kC];
        const float v = (1.f - wy) * ((1.f - wx) * c00 + wx * c01) + wy * ((1.f - wx) * c10 + wx * c11);
        e[(size_t)c * kC] = v * unit;
    }
}

// Keep the candidate with the largest positive energy gain (see launch_accept_best).
__global__ void accept_best_kernel(float* __restrict__ p_cur, const float* __restrict__ pa,
                                   const float* __restrict__ pb, long n4, const double* __restrict__ gain,
                                   const int* __restrict__ converged, unsigned long long* __restrict__ counters) {
    if (converged && __ldcg(converged)) return;
    int pick = 0;
    double best = 0.0;
    if (gain[0] > best) {
        pick = 1;
        best = gain[0];
    }
    if (gain[1] > best) pick = 2;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + (pick == 1 ? 0 : 1), 1ull);
    if (pick == 0) return;
    const float4* src = reinterpret_cast<const float4*>(pick == 1 ? pa : pb);
    float4* dst = reinterpret_cast<float4*>(p_cur);
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n4; e += (long)gridDim.x * blockDim.x)
        dst[e] = src[e];
}

// ------------------------------------------------------- defect correction
// Mixed-precision defect correction of a residual-driven projection. The pressure is
// kept as an unevaluated sum p_hi + p_lo of two FP32 fields; each cycle forms the
// residual of that sum in FP64, solves the correction e in FP32 (network + Jacobi, from
// e = 0) and adds it back exactly. The FP32 iteration alone stalls once the residual
// nears its rounding floor (about 4 eps |p| per cell, far above 1e-4 ||div|| when the
// divergence is smooth); the correction's own floor is relative to |e|, so each cycle
// gains a further factor.
//
// r = div + sum(nbrs (p_hi + p_lo)) - 4 (p_hi + p_lo) on the interior in FP64, stored in
// FP32 (edges 0); sums[0] += ||r||^2, sums[1] += ||div||^2 (FP64, zeroed before).
// Double-float arithmetic on the FP32 pipe (GB300's FP64 rate is a small fraction of its
// FP32 rate): two_sum is the error-free transformation a + b = s + e (Knuth, TAOCP vol. 2,
// 4.2.2; Moller 1965); sum2 accumulates terms with their rounding errors (Ogita, Rump,
// Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26(6), 2005), so a sum comes
// out as if computed in twice the working precision.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Rows per CTA row-slab of the row-wise kernels below (blockIdx.x: 256-column slice).
inline dim3 row_grid(int rows, int cols) {
    const int gx = (cols + 255) / 256;
    const int gy = std::max(1, std::min(rows, 2048 / gx));
    return dim3(gx, gy);
}

// r = div + sum(nbrs of p) - 4p for p = p_hi + p_lo, to about twice FP32 precision: the
// FP32 heads (and div, and -4*p_hi, which is exact) are summed with their rounding errors
// (sum2), the tails, which are ~2^-24 of the heads, in FP32; zero on the boundary.
// sums[0] += ||r||^2 and sums[1] += ||div||^2 over the interior.
__global__ void residual_df_kernel(const float* __restrict__ div, const float* __restrict__ ph,
                                   const float* __restrict__ pl, float* __restrict__ r, int rows, int cols, int pitch,
                                   double* __restrict__ sums) {
    __shared__ double red[2][256];
    float rr = 0.f, dd = 0.f;
    const int j = blockIdx.x * 256 + threadIdx.x;
    if (j < cols) {
        for (int i = blockIdx.y; i < rows; i += gridDim.y) {
            const size_t o = (size_t)i * pitch + j;
            if (i < 1 || i > rows - 2 || j < 1 || j > cols - 2) {
                r[o] = 0.f;
                continue;
            }
            const float dv = div[o];
            const float t[5] = {ph[o - 1], ph[o + 1], ph[o - pitch], ph[o + pitch], __fmul_rn(-4.f, ph[o])};
            float sh = dv, sl = 0.f;
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                float e;
                two_sum(sh, t[k], sh, e);
                sl = __fadd_rn(sl, e);
            }
            const float lo = __fsub_rn(__fadd_rn(__fadd_rn(pl[o - 1], pl[o + 1]), __fadd_rn(pl[o - pitch], pl[o + pitch])),
                                       __fmul_rn(4.f, pl[o]));
            const float res = __fadd_rn(sh, __fadd_rn(sl, lo));
            r[o] = res;
            rr = fmaf(res, res, rr);
            dd = fmaf(dv, dv, dd);
        }
    }
    red[0][threadIdx.x] = rr;
    red[1][threadIdx.x] = dd;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) {
            red[0][threadIdx.x] += red[0][threadIdx.x + k];
            red[1][threadIdx.x] += red[1][threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(sums, red[0][0]);
        atomicAdd(sums + 1, red[1][0]);
    }
}
// (p_hi, p_lo) += e as a double-float sum: two_sum of the heads, the error folded into
// the tail, renormalised (fast two_sum: the new head dominates).
__global__ void accumulate_df_kernel(float* __restrict__ ph, float* __restrict__ pl, const float* __restrict__ e,
                                     long n) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        float s, err;
        two_sum(ph[k], e[k], s, err);
        const float lo = __fadd_rn(pl[k], err);
        const float hi = __fadd_rn(s, lo);
        ph[k] = hi;
        pl[k] = __fsub_rn(lo, __fsub_rn(hi, s));
    }
}

}  // namespace

cudaError_t launch_coarse_residual(const float* div, const float* p, int rows, int cols, int pitch, int G, float* bs,
                                   double* norm2, float* scale, void* xin, const int* skip_if, cudaStream_t st) {
    const int R = (rows - 2) / G;
    restrict_kernel<<<G * G, 256, 0, st>>>(div, p, pitch, R, G, bs, nullptr, skip_if);
    coarse_input_kernel<<<1, 1024, 0, st>>>(bs, G, scale, (__nv_bfloat16*)xin, norm2, skip_if);
    return cudaGetLastError();
}

cudaError_t launch_coarse_input(const float* bs, int G, float* scale, void* xin, double* norm2, const int* skip_if,
                                cudaStream_t st) {
    coarse_input_kernel<<<1, 1024, 0, st>>>(bs, G, scale, (__nv_bfloat16*)xin, norm2, skip_if);
    return cudaGetLastError();
}

cudaError_t launch_coarse_sum2x2(const float* fine, float* coarse, int G, const int* skip_if, cudaStream_t st) {
    coarse_sum2x2_kernel<<<(G * G + 255) / 256, 256, 0, st>>>(fine, coarse, G, skip_if);
    return cudaGetLastError();
}

cudaError_t launch_coarse_interp(const float* y, float* e, int G, const float* scale, float kappa,
                                 const int* skip_if, cudaStream_t st) {
    coarse_interp_kernel<<<(4 * G * G + 255) / 256, 256, 0, st>>>(y, e, G, scale, kappa, skip_if);
    return cudaGetLastError();
}

cudaError_t launch_coarse_smooth(const float* y_in, float* y_out, const float* bs, const float* scale, float kappa,
                                 int G, int nu, const int* skip_if, cudaStream_t st) {
    if (G > kCoarseMax) return cudaErrorInvalidValue;
    coarse_smooth_kernel<<<1, kSmoothThreads, 0, st>>>(y_in, y_out, nullptr, nullptr, bs, scale, kappa, G, nu,
                                                       skip_if);
    return cudaGetLastError();
}

cudaError_t launch_coarse_smooth_pair(const float* y_in_a, float* y_out_a, const float* y_in_b, float* y_out_b,
                                      const float* bs, const float* scale, float kappa, int G, int nu,
                                      const int* skip_if, cudaStream_t st) {
    if (G > kCoarseMax) return cudaErrorInvalidValue;
    coarse_smooth_kernel<<<2, kSmoothThreads, 0, st>>>(y_in_a, y_out_a, y_in_b, y_out_b, bs, scale, kappa, G, nu,
                                                       skip_if);
    return cudaGetLastError();
}

cudaError_t launch_prolong(const float* y, const float* p_prev, float* p_out, int rows, int cols, int pitch, int G,
                           const float* scale, float kappa, const int* skip_if, cudaStream_t st) {
    const long n = (long)rows * cols;
    prolong_kernel<<<blocks_for(n, 256), 256, 0, st>>>(y, p_prev, p_out, rows, cols, pitch, (rows - 2) / G, G, scale,
                                                       kappa, skip_if);
    return cudaGetLastError();
}

cudaError_t launch_damp(const float* div, const float* p, float* out, int rows, int cols, int pitch,
                        const int* skip_if, cudaStream_t st) {
    const long n = (long)rows * cols;
    damp_kernel<<<blocks_for(n, 256), 256, 0, st>>>(div, p, out, rows, cols, pitch, skip_if);
    return cudaGetLastError();
}

cudaError_t launch_energy_gain(const float* div, const float* p_cur, const float* p_try, int rows, int cols,
                               int pitch, double* out, const int* skip_if, cudaStream_t st) {
    energy_gain_kernel<<<row_grid(rows, cols), 256, 0, st>>>(div, p_cur, p_try, rows, cols, pitch, out, skip_if);
    return cudaGetLastError();
}

cudaError_t launch_accept_best(float* p_cur, const float* pa, const float* pb, long n_floats, const double* gain,
                               const int* converged, unsigned long long* counters, cudaStream_t st) {
    accept_best_kernel<<<152 * 4, 256, 0, st>>>(p_cur, pa, pb, n_floats / 4, gain, converged, counters);
    return cudaGetLastError();
}

cudaError_t launch_residual_df(const float* div, const float* p_hi, const float* p_lo, float* r, int rows, int cols,
                               int pitch, double* sums, cudaStream_t st) {
    residual_df_kernel<<<row_grid(rows, cols), 256, 0, st>>>(div, p_hi, p_lo, r, rows, cols, pitch, sums);
    return cudaGetLastError();
}

cudaError_t launch_accumulate_df(float* p_hi, float* p_lo, const float* e, long n_floats, cudaStream_t st) {
    const int blocks = (int)std::min<long>((n_floats + 255) / 256, 8192);
    accumulate_df_kernel<<<blocks, 256, 0, st>>>(p_hi, p_lo, e, n_floats);
    return cudaGetLastError();
}

}  // namespace fs

using namespace fs;

namespace {
int launched(const char* what) {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FS_OK : record_error(FS_ERR_CUDA, what);
}
}  // namespace

extern "C" {

int fs_net_avgpool2(const void* x, void* y, int rows_out, int w_out, void* stream) {
    const long n = (long)rows_out * w_out * kC;
    avgpool2_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16*)x, (__nv_bfloat16*)y, rows_out, w_out);
    return launched("fs_net_avgpool2");
}

int fs_net_avgpool2_bwd(const float* dy, float* dx, int rows_in, int w_in, void* stream) {
    const long n = (long)rows_in * w_in * kC;
    avgpool2_bwd_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(dy, dx, rows_in, w_in);
    return launched("fs_net_avgpool2_bwd");
}

int fs_net_upsample2_bwd(const float* dup, float* dlow, int rows_low, int w_low, void* stream) {
    const long n = (long)rows_low * w_low * kC;
    upsample2_bwd_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(dup, dlow, rows_low, w_low);
    return launched("fs_net_upsample2_bwd");
}

int fs_net_relu_bwd(const float* da, const float* da2, const void* a, float* dz, void* dzb, long long n, int relu,
                    void* stream) {
    relu_bwd_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(da, da2, (const __nv_bfloat16*)a, dz,
                                                                           (__nv_bfloat16*)dzb, n, relu);
    return launched("fs_net_relu_bwd");
}

int fs_net_weight_grad(const float* dz, const void* x, float* dw, float* db, int H, int W, int img_h, int up,
                       void* stream) {
    const long npix = (long)H * W;
    if (img_h <= 0) img_h = H;
    const int per = 1024;
    weight_grad_kernel<<<blocks_for(npix, per), 256, 0, (cudaStream_t)stream>>>(dz, (const __nv_bfloat16*)x, dw, db, H,
                                                                                 W, img_h, up, per);
    return launched("fs_net_weight_grad");
}

int fs_net_flip_weights(const float* w, float* wt, void* stream) {
    flip_weights_kernel<<<blocks_for(kC * 9 * kC, 256), 256, 0, (cudaStream_t)stream>>>(w, wt);
    return launched("fs_net_flip_weights");
}

int fs_net_mse(const float* y, const float* target, float* dy, float* loss_part, long long n, void* stream) {
    mse_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(y, target, dy, loss_part, n);
    return launched("fs_net_mse");
}

int fs_net_adam(float* w, const float* g, float* m, float* v, long long n, float lr, float b1, float b2, float eps,
                int step, const unsigned char* frozen, void* stream) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    adam_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2, frozen);
    return launched("fs_net_adam");
}

int fs_net_restrict(const float* div, const float* p_prev, int rows, int cols, int pitch, int G, float* work,
                    float* scale, void* xin, float* pc, void* stream) {
    const int N = rows - 2;
    if (rows != cols || N % G != 0 || !work) return record_error(FS_ERR_ARG, "fs_net_restrict: N must be a multiple of G");
    const int R = N / G;
    cudaStream_t st = (cudaStream_t)stream;
    restrict_kernel<<<G * G, 256, 0, st>>>(div, p_prev, pitch, R, G, work, pc, nullptr);
    coarse_input_kernel<<<1, 1024, 0, st>>>(work, G, scale, (__nv_bfloat16*)xin, nullptr, nullptr);
    return launched("fs_net_restrict");
}

int fs_net_prolong(const float* y, const float* p_prev, float* p_out, int rows, int cols, int pitch, int G,
                   const float* scale, float kappa, void* stream) {
    const int N = rows - 2;
    if (rows != cols || N % G != 0) return record_error(FS_ERR_ARG, "fs_net_prolong: N must be a multiple of G");
    const long n = (long)rows * cols;
    prolong_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(y, p_prev, p_out, rows, cols, pitch, N / G,
                                                                         G, scale, kappa, nullptr);
    return launched("fs_net_prolong");
}

}  // extern "C"
