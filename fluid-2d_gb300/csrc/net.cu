// Elementwise, pooling, gradient and optimizer kernels of the learned pressure warm
// start, and the fine <-> coarse transfers that connect it to the pressure solve.
//
// The network runs on a fixed coarse grid (G x G cells, G = FS_NET_GRID): each coarse
// cell covers an R x R block of the fine interior (R = N / G). The coarse problem is
// L_c p_c = sum of the fine divergence over the block, whose solution approximates the
// block mean of the fine pressure, so a network trained at one fine size applies to
// others. Activations are NHWC with 32 channels; gradients are FP32.
//
// No counterpart in the reference (it has no learned component).

#include <cuda_bf16.h>
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
// Network input from the fine interior (pitched fields, rows x pitch, interior
// 1..N): coarse cell (I, J) of a G x G grid covers an R x R block. Channel 0 = block
// SUM of div divided by `scale`, channel 1 = block MEAN of p_prev divided by
// (scale * kappa), channels 2..31 = 0. Also writes the FP32 coarse p_prev mean.
__global__ void restrict_kernel(const float* __restrict__ div, const float* __restrict__ p, int pitch, int R, int G,
                                const float* __restrict__ scale_ptr, float kappa, __nv_bfloat16* __restrict__ xin,
                                float* __restrict__ pc) {
    const int cell = blockIdx.x;  // one CTA per coarse cell
    const int I = cell / G, J = cell % G;
    float sd = 0.f, sp = 0.f;
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
        const int i = 1 + I * R + e / R, j = 1 + J * R + e % R;
        sd += div[(size_t)i * pitch + j];
        sp += p ? p[(size_t)i * pitch + j] : 0.f;
    }
    __shared__ float a[256], b[256];
    a[threadIdx.x] = sd;
    b[threadIdx.x] = sp;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            a[threadIdx.x] += a[threadIdx.x + s];
            b[threadIdx.x] += b[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x < kC) {
        const float scale = *scale_ptr;
        const float mean_p = b[0] / (float)(R * R);
        float v = 0.f;
        if (threadIdx.x == 0) v = a[0] / scale;
        if (threadIdx.x == 1) v = mean_p / (scale * kappa);
        xin[(size_t)cell * kC + threadIdx.x] = __float2bfloat16_rn(v);
        if (threadIdx.x == 0 && pc) pc[cell] = mean_p;
    }
}

// RMS of the block sums of div over the coarse grid (one CTA), with a floor; the
// network's input scale.
__global__ void coarse_scale_kernel(const float* __restrict__ div, int pitch, int R, int G, float* __restrict__ out) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int cell = threadIdx.x; cell < G * G; cell += blockDim.x) {
        const int I = cell / G, J = cell % G;
        float s = 0.f;
        for (int e = 0; e < R * R; ++e) s += div[(size_t)(1 + I * R + e / R) * pitch + 1 + J * R + e % R];
        acc += (double)s * s;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = (float)fmax(sqrt(red[0] / (double)(G * G)), 1e-30);
}

// Fine warm start: p_out = p_prev + bilinear interpolation of the coarse correction
// (network channel 0 times scale * kappa) at fine cell centres, over the interior;
// edges take their inner neighbour (Neumann fill), corners keep p_prev.
__global__ void prolong_kernel(const float* __restrict__ y, const float* __restrict__ p_prev, float* __restrict__ p_out,
                               int rows, int cols, int pitch, int R, int G, const float* __restrict__ scale_ptr,
                               float kappa) {
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

// Squared Poisson residuals ||div + sum(nbrs) - 4p||^2 of two pressures over the
// interior (pb may be null = zero), accumulated into out[0], out[1] (zeroed before).
__global__ void residual_pair_kernel(const float* __restrict__ div, const float* __restrict__ pa,
                                     const float* __restrict__ pb, int rows, int cols, int pitch,
                                     double* __restrict__ out) {
    __shared__ double ra[256], rb[256];
    double a = 0.0, b = 0.0;
    const long n = (long)(rows - 2) * (cols - 2);
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(e / (cols - 2)), j = 1 + (int)(e % (cols - 2));
        const size_t o = (size_t)i * pitch + j;
        const float d = div[o];
        const float s1 = d + pa[o - 1] + pa[o + 1] + pa[o - pitch] + pa[o + pitch] - 4.f * pa[o];
        a += (double)s1 * s1;
        float s2 = d;
        if (pb) s2 += pb[o - 1] + pb[o + 1] + pb[o - pitch] + pb[o + pitch] - 4.f * pb[o];
        b += (double)s2 * s2;
    }
    ra[threadIdx.x] = a;
    rb[threadIdx.x] = b;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            ra[threadIdx.x] += ra[threadIdx.x + s];
            rb[threadIdx.x] += rb[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(out, ra[0]);
        atomicAdd(out + 1, rb[0]);
    }
}

// Keep the network's guess when its residual is not larger than the previous
// pressure's; otherwise overwrite the guess with the previous pressure (or zero).
// counters[0] counts guesses used, counters[1] fallbacks.
__global__ void select_guess_kernel(float* __restrict__ guess, const float* __restrict__ prev, long n_floats,
                                    const double* __restrict__ res, unsigned long long* __restrict__ counters) {
    const bool fallback = res[0] > res[1];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + (fallback ? 1 : 0), 1ull);
    if (!fallback) return;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n_floats; e += (long)gridDim.x * blockDim.x)
        guess[e] = prev ? prev[e] : 0.f;
}

}  // namespace

cudaError_t launch_learned_select(const float* div, float* guess, const float* prev, int rows, int cols, int pitch,
                                  double* res2, unsigned long long* counters, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(res2, 0, 2 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    residual_pair_kernel<<<152 * 4, 256, 0, st>>>(div, guess, prev, rows, cols, pitch, res2);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    select_guess_kernel<<<152 * 4, 256, 0, st>>>(guess, prev, (long)rows * pitch, res2, counters);
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

int fs_net_restrict(const float* div, const float* p_prev, int rows, int cols, int pitch, int G, float kappa,
                    float* scale, void* xin, float* pc, void* stream) {
    const int N = rows - 2;
    if (rows != cols || N % G != 0) return record_error(FS_ERR_ARG, "fs_net_restrict: N must be a multiple of G");
    const int R = N / G;
    cudaStream_t st = (cudaStream_t)stream;
    coarse_scale_kernel<<<1, 256, 0, st>>>(div, pitch, R, G, scale);
    restrict_kernel<<<G * G, 256, 0, st>>>(div, p_prev, pitch, R, G, scale, kappa, (__nv_bfloat16*)xin, pc);
    return launched("fs_net_restrict");
}

int fs_net_prolong(const float* y, const float* p_prev, float* p_out, int rows, int cols, int pitch, int G,
                   const float* scale, float kappa, void* stream) {
    const int N = rows - 2;
    if (rows != cols || N % G != 0) return record_error(FS_ERR_ARG, "fs_net_prolong: N must be a multiple of G");
    const long n = (long)rows * cols;
    prolong_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(y, p_prev, p_out, rows, cols, pitch, N / G,
                                                                         G, scale, kappa);
    return launched("fs_net_prolong");
}

}  // extern "C"
