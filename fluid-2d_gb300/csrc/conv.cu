// 3x3 convolutions for the learned pressure warm start (BF16 operands, FP32
// accumulation), NHWC activations with 32 channels.
//
// conv3x3_tc_kernel is an implicit GEMM on the tcgen05 tensor cores: one CTA computes
// 128 output pixels x 32 output channels, D[128x32] = A[128x288] * B[32x288]^T with
// K = 9 taps x 32 input channels. A (the im2col rows of the 128 pixels, zero-filled
// outside the image) and B (the packed weights) are staged in shared memory in the
// no-swizzle K-major core-matrix layout by 16-byte cp.async copies; one thread issues
// the 18 K=16 MMAs into a 32-column FP32 accumulator in tensor memory and commits them
// to an mbarrier; each warp then reads its 32 rows back with tcgen05.ld and applies
// bias, the optional skip input, ReLU and the BF16 store.
//
// Layout of both operands in shared memory: element (row r, k) of a [R x 288] operand
// lives at byte ((r/8)*36 + k/8)*128 + (r%8)*16 + (k%8)*2, i.e. core matrices of 8 rows
// x 8 BF16 values, 128 contiguous bytes each; adjacent along K: +128 B (LBO), adjacent
// along rows: +36*128 B (SBO).
//
// conv3x3_ref_kernel computes the same thing on CUDA cores, one output value per
// thread; it is the checked reference for the tensor-core kernel and a fallback for
// debugging only.
//
// No counterpart in the reference (it has no learned component).

#include <cuda_bf16.h>
#include <algorithm>
#include <cuda_runtime.h>

#include "../../include/fluid2d_gb300.h"
#include "fs_internal.cuh"
#include "tc.cuh"

namespace fs {
namespace {

constexpr int kC = 32;             // channels
constexpr int kK = 9 * kC;         // GEMM K = 288
constexpr int kKC = kK / 8;        // core matrices along K = 36
constexpr int kTileM = 128;        // pixels per CTA
constexpr int kAbytes = kTileM * kK * 2;  // 73728
constexpr int kBbytes = kC * kK * 2;      // 18432
constexpr int kConvSmem = kAbytes + kBbytes + 64;
constexpr uint32_t kWaitLimit = 1u << 22;

struct ConvArgs {
    const __nv_bfloat16* x;    // input NHWC, 32 channels: (H x W), or (H/2 x W/2) when up
    const __nv_bfloat16* wpk;  // packed weights, 32 x 288 in the core-matrix layout
    const float* bias;         // 32 (nullable)
    const __nv_bfloat16* skip; // NHWC H x W x 32 added before the activation (nullable)
    __nv_bfloat16* y;          // output NHWC H x W x 32 (nullable)
    float* yf;                 // output FP32 H x W x 32 (nullable)
    int H, W;                  // output size (H = images x img_h rows)
    int img_h;                 // rows per image: zero padding applies at image borders
    int up;                    // 1: the input is nearest-upsampled by 2 on the fly
    int relu;
    int* err;                  // set to 1 if an mbarrier wait gave up
    const int* skip_if;        // nullable: when *skip_if != 0 the launch does nothing
};

// Source pixel of tap (dy, dx) for output pixel (y, x), or -1 outside its image.
// Images of img_h rows are stacked along y; with `up` the input has img_h/2 rows per
// image and W/2 columns, so the source row (y+dy)/2 stays inside the same image.
__device__ __forceinline__ long tap_source(const ConvArgs& P, int y, int x, int dy, int dx) {
    const int ly = y % P.img_h + dy, ix = x + dx;
    if (ly < 0 || ly >= P.img_h || ix < 0 || ix >= P.W) return -1;
    const int iy = y + dy;
    if (P.up) return (long)(iy >> 1) * (P.W >> 1) + (ix >> 1);
    return (long)iy * P.W + ix;
}

__device__ __forceinline__ void epilogue_store(const ConvArgs& P, long p, float (&v)[32]) {
    if (P.bias) {
#pragma unroll
        for (int c = 0; c < kC; ++c) v[c] += __ldg(P.bias + c);
    }
    if (P.skip) {
        const uint4* s = reinterpret_cast<const uint4*>(P.skip + p * kC);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint4 w = __ldg(s + q);
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&w);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                float2 f = __bfloat1622float2(h[e]);
                v[q * 8 + 2 * e] += f.x;
                v[q * 8 + 2 * e + 1] += f.y;
            }
        }
    }
    if (P.relu) {
#pragma unroll
        for (int c = 0; c < kC; ++c) v[c] = fmaxf(v[c], 0.f);
    }
    if (P.y) {
        uint4* o = reinterpret_cast<uint4*>(P.y + p * kC);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint4 w;
            __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&w);
#pragma unroll
            for (int e = 0; e < 4; ++e) h[e] = __floats2bfloat162_rn(v[q * 8 + 2 * e], v[q * 8 + 2 * e + 1]);
            o[q] = w;
        }
    }
    if (P.yf) {
        float4* o = reinterpret_cast<float4*>(P.yf + p * kC);
#pragma unroll
        for (int q = 0; q < 8; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
}

__global__ void __launch_bounds__(128) conv3x3_tc_kernel(const ConvArgs P) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* As = sm;
    uint8_t* Bs = sm + kAbytes;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kAbytes + kBbytes);
    uint32_t* s_taddr = reinterpret_cast<uint32_t*>(sm + kAbytes + kBbytes + 16);
    if (P.skip_if && __ldcg(P.skip_if)) return;  // uniform across the CTA, before any TMEM use
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long npix = (long)P.H * P.W;
    const long p0 = (long)blockIdx.x * kTileM;

    if (warp == 0) {
        tc::tmem_alloc(s_taddr, 32);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(bar, 1);

    // B: 32 rows x 36 core-matrix columns, already packed in this layout
    for (int c = tid; c < kC * kKC; c += 128) tc::cp_async16(Bs + c * 16, P.wpk + c * 8, 16);
    // A: im2col of 128 pixels; chunk q = (pixel m, core column kc = tap*4 + channel group)
    for (int q = tid; q < kTileM * kKC; q += 128) {
        const int m = q / kKC, kc = q - m * kKC;
        const int t = kc >> 2, g = kc & 3;
        const long p = p0 + m;
        long src = -1;
        if (p < npix) {
            const int y = (int)(p / P.W), x = (int)(p - (long)y * P.W);
            src = tap_source(P, y, x, t / 3 - 1, t % 3 - 1);
        }
        uint8_t* dst = As + ((m >> 3) * kKC + kc) * 128 + (m & 7) * 16;
        const __nv_bfloat16* s = P.x + (src < 0 ? 0 : src * kC + g * 8);
        tc::cp_async16(dst, s, src < 0 ? 0u : 16u);
    }
    tc::cp_async_wait_all();
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = *s_taddr;

    if (tid == 0) {
        const uint32_t a0 = tc::smem_u32(As), b0 = tc::smem_u32(Bs);
        constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 32);
#pragma unroll
        for (int kk = 0; kk < kK / 16; ++kk) {
            const uint64_t ad = tc::smem_desc(a0 + kk * 256, 128, kKC * 128);
            const uint64_t bd = tc::smem_desc(b0 + kk * 256, 128, kKC * 128);
            tc::mma_bf16(taddr, ad, bd, idesc, kk > 0);
        }
        tc::commit_to(bar);
    }
    // Bounded wait for the MMAs. Tensor memory is read and freed only after the commit
    // has arrived, since an MMA still in flight writes it (and reads the shared-memory
    // operands). If the first bound runs out the CTA flags the error, skips the
    // epilogue, and waits once more with the same bound before freeing; a CTA whose
    // warp 0 never sees the arrival leaves the allocation in place rather than free
    // columns an MMA may still write (the host treats the flagged error as fatal for
    // the network).
    auto wait_commit = [&]() {
        uint32_t spins = 0;
        while (!tc::mbar_try_wait(bar, 0))
            if (++spins > kWaitLimit) return false;
        return true;
    };
    bool arrived = wait_commit();
    if (!arrived && P.err) atomicOr(P.err, 1);
    tc::fence_after_sync();
    if (__all_sync(0xffffffffu, arrived)) {
        float v[32];
        tc::tmem_ld_32x32(taddr + ((uint32_t)(warp * 32) << 16), v);
        const long p = p0 + warp * 32 + lane;
        if (p < npix) epilogue_store(P, p, v);
    } else {
        arrived = wait_commit();
    }
    const bool free_ok = __all_sync(0xffffffffu, arrived);

    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0 && free_ok) tc::tmem_dealloc(taddr, 32);
}

// Reference: one thread per (pixel, output channel), FP32 accumulation of BF16 values.
__global__ void __launch_bounds__(256) conv3x3_ref_kernel(const ConvArgs P, const float* __restrict__ w32) {
    if (P.skip_if && __ldcg(P.skip_if)) return;
    const long npix = (long)P.H * P.W;
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    const int y = (int)(i / P.W), x = (int)(i - (long)y * P.W);
    float v[32];
    for (int co = 0; co < kC; ++co) {
        float acc = 0.f;
        for (int t = 0; t < 9; ++t) {
            const long src = tap_source(P, y, x, t / 3 - 1, t % 3 - 1);
            if (src < 0) continue;
            for (int ci = 0; ci < kC; ++ci) {
                const float a = __bfloat162float(P.x[src * kC + ci]);
                const float b = __bfloat162float(__float2bfloat16_rn(w32[(co * 9 + t) * kC + ci]));
                acc = fmaf(a, b, acc);
            }
        }
        v[co] = acc;
    }
    epilogue_store(P, i, v);
}

// ------------------------------------------------------------- weight gradient
// wgrad_tc_kernel: dW[co][t][ci] = sum_p dz[p][co] * x(p, tap t)[ci] and db[co] =
// sum_p dz[p][co] as one implicit GEMM on the tensor cores with the pixels as the
// reduction dimension: D[f][co] = sum_p A[f][p] * B[co][p], f = t*32 + ci (288 rows)
// plus f = 288, a row of ones, whose result is db. The 289 rows are three M = 128
// tiles (rows 289..383 are zero), N = 32, three 32-column FP32 accumulators in tensor
// memory. Each CTA reduces a contiguous range of pixels in chunks of 64 (K = 64, four
// K = 16 MMAs per tile), double-buffered: the threads stage chunk s + 1 while the
// MMAs of chunk s run. Both operands are pixel-contiguous in the K-major core-matrix
// layout (element (row, k) of a buffer at ((row/8)*8 + k/8)*128 + (row%8)*16 +
// (k%8)*2), so the NHWC activations (channel-contiguous) are transposed on the way in:
// a thread loads eight pixels' 16-byte channel groups and writes one 128-byte core
// matrix (8 channels x 8 pixels) with byte permutes. The CTA writes its 289 x 32
// partial sums to a workspace and wgrad_reduce_kernel adds the CTAs' partials in a
// fixed order, so the gradient is deterministic.
constexpr int kWgK = 64;                   // pixels per chunk
constexpr int kWgRows = 384;               // 3 M tiles
constexpr int kWgAbytes = kWgRows * kWgK * 2;  // 49152
constexpr int kWgBbytes = kC * kWgK * 2;       // 4096
constexpr int kWgStage = kWgAbytes + kWgBbytes;
constexpr int kWgSmem = 2 * kWgStage + 64;
constexpr int kWgOut = 289;                // rows of the partial result (288 weights + bias)
constexpr int kWgThreads = 256;            // 8 warps; two CTAs per SM (shared memory and TMEM allow it)

struct WgradArgs {
    const __nv_bfloat16* x;   // layer input NHWC (as in ConvArgs, `up` for nearest-upsampled)
    const __nv_bfloat16* dz;  // BF16 gradient at the layer output, NHWC H x W x 32
    float* work;              // [gridDim.x][289][32] partial sums
    int H, W, img_h, up;
    int per;                  // pixels per CTA (a multiple of kWgK)
    int* err;
};

// 8 x 8 transpose of BF16 values: in[j] holds 8 channels of pixel j, out[i] gets
// channel i of the 8 pixels.
__device__ __forceinline__ void transpose8x8_b16(const uint4 (&in)[8], uint4 (&out)[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t sel = (i & 1) ? 0x7632u : 0x5410u;
        uint32_t w[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint4 a = in[2 * k], b = in[2 * k + 1];
            const uint32_t av = (i >> 1) == 0 ? a.x : (i >> 1) == 1 ? a.y : (i >> 1) == 2 ? a.z : a.w;
            const uint32_t bv = (i >> 1) == 0 ? b.x : (i >> 1) == 1 ? b.y : (i >> 1) == 2 ? b.z : b.w;
            w[k] = __byte_perm(av, bv, sel);
        }
        out[i] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

__global__ void __launch_bounds__(kWgThreads) wgrad_tc_kernel(const WgradArgs P) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 2 * kWgStage);  // one per buffer
    uint32_t* s_taddr = reinterpret_cast<uint32_t*>(sm + 2 * kWgStage + 32);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long npix = (long)P.H * P.W;
    const long pbeg = (long)blockIdx.x * P.per;
    const long pend = min(npix, pbeg + (long)P.per);
    const int nchunks = pbeg < pend ? (int)((pend - pbeg + kWgK - 1) / kWgK) : 0;

    if (warp == 0) {
        tc::tmem_alloc(s_taddr, 128);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(bar, 1);
        tc::mbar_init(bar + 1, 1);
    }
    // rows 288..383 of both A buffers: row 288 all ones (its product row is db), the
    // rest zero; the staging below never writes them
    for (int b = 0; b < 2; ++b) {
        uint4* z = reinterpret_cast<uint4*>(sm + b * kWgStage + 36 * 8 * 128);
        for (int e = tid; e < 12 * 8 * 8; e += kWgThreads) {
            const bool ones = e < 8 * 8 && (e & 7) == 0;  // core matrices (36, pg), row 0
            z[e] = ones ? make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u) : make_uint4(0, 0, 0, 0);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = *s_taddr;

    auto wait_bar = [&](uint64_t* b, uint32_t parity) {
        uint32_t spins = 0;
        while (!tc::mbar_try_wait(b, parity))
            if (++spins > kWaitLimit) return false;
        return true;
    };
    bool ok = true;
    int last_issued = -1;  // last chunk whose MMAs were committed
    for (int s = 0; s < nchunks && ok; ++s) {
        const int buf = s & 1;
        uint8_t* As = sm + buf * kWgStage;
        uint8_t* Bs = As + kWgAbytes;
        if (s >= 2) {  // the MMAs of chunk s - 2 read this buffer
            const bool got = wait_bar(bar + buf, (uint32_t)((s - 2) >> 1) & 1u);
            ok = __syncthreads_and(got) != 0;
            if (!ok) break;
        }
        const long c0 = pbeg + (long)s * kWgK;
        // items: 288 of A (tap t, channel group cg, pixel group pg), 32 of B (cg, pg)
        for (int q = tid; q < 320; q += kWgThreads) {
            uint4 in[8], out[8];
            uint8_t* dst;
            if (q < 288) {
                const int t = q >> 5, cg = (q >> 3) & 3, pg = q & 7;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const long p = c0 + pg * 8 + j;
                    long src = -1;
                    if (p < pend) {
                        const int y = (int)(p / P.W), xx = (int)(p - (long)y * P.W);
                        const int ly = y % P.img_h + t / 3 - 1, ix = xx + t % 3 - 1;
                        if (ly >= 0 && ly < P.img_h && ix >= 0 && ix < P.W) {
                            const int iy = y + t / 3 - 1;
                            src = P.up ? (long)(iy >> 1) * (P.W >> 1) + (ix >> 1) : (long)iy * P.W + ix;
                        }
                    }
                    in[j] = src < 0 ? make_uint4(0, 0, 0, 0)
                                    : __ldg(reinterpret_cast<const uint4*>(P.x + src * kC + cg * 8));
                }
                dst = As + ((t * 4 + cg) * 8 + pg) * 128;
            } else {
                const int cg = (q - 288) >> 3, pg = q & 7;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const long p = c0 + pg * 8 + j;
                    in[j] = p < pend ? __ldg(reinterpret_cast<const uint4*>(P.dz + p * kC + cg * 8))
                                     : make_uint4(0, 0, 0, 0);
                }
                dst = Bs + (cg * 8 + pg) * 128;
            }
            transpose8x8_b16(in, out);
#pragma unroll
            for (int i = 0; i < 8; ++i) *reinterpret_cast<uint4*>(dst + i * 16) = out[i];
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 32);
            const uint32_t a0 = tc::smem_u32(As), b0 = tc::smem_u32(Bs);
#pragma unroll
            for (int g = 0; g < 3; ++g)
#pragma unroll
                for (int kk = 0; kk < kWgK / 16; ++kk) {
                    const uint64_t ad = tc::smem_desc(a0 + g * 16 * 8 * 128 + kk * 256, 128, 8 * 128);
                    const uint64_t bd = tc::smem_desc(b0 + kk * 256, 128, 8 * 128);
                    tc::mma_bf16(taddr + g * 32, ad, bd, idesc, s > 0 || kk > 0);
                }
            tc::commit_to(bar + buf);
        }
        last_issued = s;
    }
    // The last commit covers every MMA this CTA issued. Tensor memory is read and freed
    // only after it has arrived; a CTA that gives up waiting (here, or for a buffer in
    // the loop) flags the error, skips the epilogue, and keeps its allocation unless
    // the last commit arrives after all, rather than free columns an MMA may still write.
    bool arrived = true;
    if (last_issued >= 0) arrived = wait_bar(bar + (last_issued & 1), (uint32_t)(last_issued >> 1) & 1u);
    const bool all_arrived = __syncthreads_and(arrived) != 0;
    if ((!ok || !all_arrived) && tid == 0 && P.err) atomicOr(P.err, 1);
    tc::fence_after_sync();
    if (ok && all_arrived) {
        float* out = P.work + (size_t)blockIdx.x * kWgOut * kC;
        // warp w reads tensor-memory lanes 32*(w%4).. of the tiles g = w/4, w/4 + 2
#pragma unroll 1
        for (int g = warp >> 2; g < 3; g += kWgThreads / 128) {
            const int f = g * 128 + (warp & 3) * 32 + lane;
            float v[32];
            if (nchunks > 0) {
                tc::tmem_ld_32x32(taddr + ((uint32_t)((warp & 3) * 32) << 16) + g * 32, v);
            } else {
#pragma unroll
                for (int c = 0; c < 32; ++c) v[c] = 0.f;
            }
            if (f < kWgOut) {
                float4* o = reinterpret_cast<float4*>(out + (size_t)f * kC);
#pragma unroll
                for (int q = 0; q < 8; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0 && all_arrived) tc::tmem_dealloc(taddr, 128);
}

// dw[co][f] += sum over CTAs of work[cta][f][co] (f < 288); db[co] += the f = 288 row.
__global__ void wgrad_reduce_kernel(const float* __restrict__ work, int nblocks, float* __restrict__ dw,
                                    float* __restrict__ db) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kWgOut * kC) return;
    const int f = e / kC, co = e - f * kC;
    float s = 0.f;
    for (int b = 0; b < nblocks; ++b) s += __ldcg(work + (size_t)b * kWgOut * kC + e);
    if (f < kK)
        dw[co * kK + f] += s;
    else if (db)
        db[co] += s;
}

// ------------------------------------------------------------- fused inference
// net_infer32_kernel: the whole 8-layer network on one 32 x 32 grid in one CTA (one CTA
// per image of a batch): e1 = conv(x0) -> pool -> e2, e3 (16 x 16) -> pool -> b1, b2
// (8 x 8) -> d1 = conv(up b2) + e3 -> d2 = conv(up d1) + e1 -> out = conv(d2), the same
// layer sequence and arithmetic as the per-layer launches of conv3x3_tc_kernel.
//
// Activations stay in shared memory, one buffer per level, in a zero-padded layout
// that makes every 3x3 tap a plain shifted operand, so no im2col copy is made: the
// (g+2) x (g+2) padded pixels of a level are numbered m = py*(g+2) + px, preceded by
// g+3 and followed by enough zero slots that every shifted read stays inside, and
// channel group c/8 of slot k lives at plane (c/8) * PL + k*16 bytes (PL = plane
// stride). Rows m..m+127 of the A operand for tap (dy, dx) are then slots m + dy*(g+2)
// + dx onward: one K-major no-swizzle descriptor with 16-byte rows (SBO = 128 B between
// 8-row groups, LBO = PL between channel groups). The GEMM runs over all padded pixels
// (border outputs are computed and dropped), 18 MMAs (9 taps x K = 32) per 128-pixel
// tile, every tile of a layer in its own 32 columns of tensor memory (10 tiles = 320
// columns at 32 x 32). All MMAs of a layer complete before its epilogue writes, so each
// layer writes its output over its input; the skip of layer 5 (e3) is kept in a
// separate shared buffer and that of layer 6 (e1) in global memory. Pooling and
// upsampling move data between the level buffers; only interior pixels are written,
// so the borders stay zero.
constexpr int kInfG = 32;
constexpr int kInfThreads = 256;
struct InfLevel {
    int g, P, npad, tiles, guard, slots, PL, bytes;
};
__host__ __device__ constexpr InfLevel inf_level(int g) {
    return InfLevel{g,
                    g + 2,
                    (g + 2) * (g + 2),
                    ((g + 2) * (g + 2) + 127) / 128,
                    g + 3,
                    (g + 3) + ((g + 2) * (g + 2) + 127) / 128 * 128 + (g + 3),
                    16 * ((g + 3) + ((g + 2) * (g + 2) + 127) / 128 * 128 + (g + 3)),
                    4 * 16 * ((g + 3) + ((g + 2) * (g + 2) + 127) / 128 * 128 + (g + 3))};
}
constexpr InfLevel kL0 = inf_level(kInfG), kL1 = inf_level(kInfG / 2), kL2 = inf_level(kInfG / 4);
constexpr int kInfWOff = 0;                           // packed weights of the current layer
constexpr int kInfB0 = kInfWOff + kBbytes;            // level buffers
constexpr int kInfB1 = kInfB0 + kL0.bytes;
constexpr int kInfB2 = kInfB1 + kL1.bytes;
constexpr int kInfE3 = kInfB2 + kL2.bytes;            // e3, NHWC 16 x 16 x 32
constexpr int kInfBar = kInfE3 + (kInfG / 2) * (kInfG / 2) * kC * 2;
constexpr int kInfSmem = kInfBar + 64;
static_assert(kL0.tiles * 32 <= 512, "tensor memory holds every tile of a layer");
static_assert(kInfSmem <= 227 * 1024, "fits one CTA's shared memory");
static_assert(kL0.PL % 16 == 0 && kL1.PL % 16 == 0 && kL2.PL % 16 == 0, "16-byte planes");

struct InferArgs {
    const __nv_bfloat16* x0;  // network input, B images of 32 x 32 x 32 (NHWC)
    const __nv_bfloat16* wpk; // 8 layers x 9216 packed weights
    const float* params;      // FP32 parameters, layer li's bias at li*9248 + 9216
    __nv_bfloat16* e1;        // scratch, B x 32 x 32 x 32: the skip of layer 6
    float* y;                 // output, B x 32 x 32 x 32 FP32
    int* err;
    const int* skip_if;
};

// 16 bytes (8 channels) of slot k, channel group cg, in a level buffer
__device__ __forceinline__ uint4* inf_slot(uint8_t* buf, const InfLevel L, int k, int cg) {
    return reinterpret_cast<uint4*>(buf + cg * L.PL + k * 16);
}
__device__ __forceinline__ int inf_interior(const InfLevel L, int y, int x) {
    return L.guard + (y + 1) * L.P + (x + 1);
}

__global__ void __launch_bounds__(kInfThreads) net_infer32_kernel(const InferArgs A) {
    extern __shared__ __align__(1024) uint8_t sm[];
    if (A.skip_if && __ldcg(A.skip_if)) return;  // uniform, before any tensor-memory use
    uint8_t* Ws = sm + kInfWOff;
    uint8_t* B0 = sm + kInfB0;
    uint8_t* B1 = sm + kInfB1;
    uint8_t* B2 = sm + kInfB2;
    uint8_t* E3 = sm + kInfE3;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kInfBar);
    uint32_t* s_taddr = reinterpret_cast<uint32_t*>(sm + kInfBar + 16);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int img = blockIdx.x;
    constexpr int G = kInfG;
    const __nv_bfloat16* x0 = A.x0 + (size_t)img * G * G * kC;
    __nv_bfloat16* e1g = A.e1 + (size_t)img * G * G * kC;
    float* yout = A.y + (size_t)img * G * G * kC;

    if (warp == 0) {
        tc::tmem_alloc(s_taddr, 512);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(bar, 1);
    // zero the level buffers (borders and guards stay zero), then the input's interior
    for (int e = tid; e < (kL0.bytes + kL1.bytes + kL2.bytes) / 16; e += kInfThreads)
        reinterpret_cast<uint4*>(B0)[e] = make_uint4(0, 0, 0, 0);
    __syncthreads();
    for (int e = tid; e < G * G * 4; e += kInfThreads) {
        const int p = e >> 2, cg = e & 3;
        *inf_slot(B0, kL0, inf_interior(kL0, p / G, p % G), cg) =
            __ldg(reinterpret_cast<const uint4*>(x0 + (size_t)p * kC + cg * 8));
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = *s_taddr;

    auto pool = [&](uint8_t* src, const InfLevel Ls, uint8_t* dst, const InfLevel Ld) {
        // 2x2 average (avgpool2_kernel's order and rounding) into the next level
        for (int e = tid; e < Ld.g * Ld.g * kC; e += kInfThreads) {
            const int c = e % kC, p = e / kC, Y = p / Ld.g, X = p % Ld.g;
            const int cg = c >> 3, ci = c & 7;
            auto at = [&](int y, int x) {
                const __nv_bfloat16* q = reinterpret_cast<const __nv_bfloat16*>(
                    inf_slot(src, Ls, inf_interior(Ls, y, x), cg));
                return __bfloat162float(q[ci]);
            };
            const float sum = __fadd_rn(__fadd_rn(__fadd_rn(at(2 * Y, 2 * X), at(2 * Y, 2 * X + 1)),
                                                  at(2 * Y + 1, 2 * X)),
                                        at(2 * Y + 1, 2 * X + 1));
            reinterpret_cast<__nv_bfloat16*>(inf_slot(dst, Ld, inf_interior(Ld, Y, X), cg))[ci] =
                __float2bfloat16_rn(__fmul_rn(0.25f, sum));
        }
    };
    auto upsample = [&](uint8_t* src, const InfLevel Ls, uint8_t* dst, const InfLevel Ld) {
        // nearest x2 into the interior of the finer level
        for (int e = tid; e < Ld.g * Ld.g * 4; e += kInfThreads) {
            const int p = e >> 2, cg = e & 3, y = p / Ld.g, x = p % Ld.g;
            *inf_slot(dst, Ld, inf_interior(Ld, y, x), cg) = *inf_slot(src, Ls, inf_interior(Ls, y >> 1, x >> 1), cg);
        }
    };

    bool ok = true;
    // layer li on the level buffer `buf` (input, overwritten by the output), with the
    // given skip source; out_kind 0: BF16 in place, 1: also e1 to global, 2: also e3 to
    // the skip buffer, 3: FP32 to the output (no ReLU)
    auto layer = [&](int li, uint8_t* buf, const InfLevel L, int skip_kind, int out_kind) {
        if (!ok) return;
        // the layer's weights (the previous layer's MMAs are complete)
        const __nv_bfloat16* wsrc = A.wpk + (size_t)li * (kC * kK);
        for (int c = tid; c < kC * kKC; c += kInfThreads) tc::cp_async16(Ws + c * 16, wsrc + c * 8, 16);
        tc::cp_async_wait_all();
        tc::fence_proxy_async_smem();  // weights and the activations written by this CTA
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 32);
            const uint32_t a0 = tc::smem_u32(buf), w0 = tc::smem_u32(Ws);
            for (int T = 0; T < L.tiles; ++T) {
#pragma unroll
                for (int t = 0; t < 9; ++t) {
                    const int shift = (t / 3 - 1) * L.P + (t % 3 - 1);
                    const uint32_t row0 = (uint32_t)(L.guard + T * 128 + shift) * 16u;
#pragma unroll
                    for (int kk = 0; kk < 2; ++kk) {
                        const uint64_t ad = tc::smem_desc(a0 + (uint32_t)(2 * kk * L.PL) + row0, L.PL, 128);
                        const uint64_t bd = tc::smem_desc(w0 + (uint32_t)(t * 2 + kk) * 256, 128, kKC * 128);
                        tc::mma_bf16(taddr + T * 32, ad, bd, idesc, t > 0 || kk > 0);
                    }
                }
            }
            tc::commit_to(bar);
        }
        uint32_t spins = 0;
        bool got = true;
        while (!tc::mbar_try_wait(bar, (uint32_t)(li & 1)))
            if (++spins > kWaitLimit) {
                got = false;
                break;
            }
        ok = __syncthreads_and(got) != 0;
        tc::fence_after_sync();
        if (!ok) return;
        const float* bias = A.params + (size_t)li * (kC * kK + kC) + kC * kK;
        // warp w reads tensor-memory lanes 32*(w%4).. of the tiles T = w/4, w/4 + 2, ...
        for (int T = warp >> 2; T < L.tiles; T += kInfThreads / 128) {
            float v[32];
            tc::tmem_ld_32x32(taddr + ((uint32_t)((warp & 3) * 32) << 16) + T * 32, v);
            const int m = T * 128 + (warp & 3) * 32 + lane;
            const int py = m / L.P, px = m - py * L.P;
            if (m >= L.npad || py < 1 || py > L.g || px < 1 || px > L.g) continue;
            const int y = py - 1, x = px - 1, k = L.guard + m;
#pragma unroll
            for (int c = 0; c < kC; ++c) v[c] += __ldg(bias + c);
            if (skip_kind) {
                const uint4* sp = skip_kind == 1 ? reinterpret_cast<const uint4*>(e1g + (size_t)(y * G + x) * kC)
                                                 : reinterpret_cast<const uint4*>(E3 + (y * (G / 2) + x) * kC * 2);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    uint4 w = skip_kind == 1 ? __ldcg(sp + q) : sp[q];
                    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&w);
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float2 f = __bfloat1622float2(h[e]);
                        v[q * 8 + 2 * e] += f.x;
                        v[q * 8 + 2 * e + 1] += f.y;
                    }
                }
            }
            if (out_kind == 3) {
                float4* o = reinterpret_cast<float4*>(yout + (size_t)(y * G + x) * kC);
#pragma unroll
                for (int q = 0; q < 8; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                continue;
            }
#pragma unroll
            for (int c = 0; c < kC; ++c) v[c] = fmaxf(v[c], 0.f);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint4 w;
                __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&w);
#pragma unroll
                for (int e = 0; e < 4; ++e) h[e] = __floats2bfloat162_rn(v[q * 8 + 2 * e], v[q * 8 + 2 * e + 1]);
                *inf_slot(buf, L, k, q) = w;
                if (out_kind == 1) reinterpret_cast<uint4*>(e1g + (size_t)(y * G + x) * kC)[q] = w;
                if (out_kind == 2) reinterpret_cast<uint4*>(E3 + (y * (G / 2) + x) * kC * 2)[q] = w;
            }
        }
        tc::fence_before_sync();
        __syncthreads();
    };

    layer(0, B0, kL0, 0, 1);  // e1
    if (ok) {
        pool(B0, kL0, B1, kL1);  // pool1
        __syncthreads();
    }
    layer(1, B1, kL1, 0, 0);  // e2
    layer(2, B1, kL1, 0, 2);  // e3 (+ skip copy)
    if (ok) {
        pool(B1, kL1, B2, kL2);  // pool2
        __syncthreads();
    }
    layer(3, B2, kL2, 0, 0);  // b1
    layer(4, B2, kL2, 0, 0);  // b2
    if (ok) {
        upsample(B2, kL2, B1, kL1);
        __syncthreads();
    }
    layer(5, B1, kL1, 2, 0);  // d1 = relu(conv(up b2) + b + e3)
    if (ok) {
        __threadfence_block();  // e1 stores to global by this CTA, read back in layer 6
        upsample(B1, kL1, B0, kL0);
        __syncthreads();
    }
    layer(6, B0, kL0, 1, 0);  // d2 = relu(conv(up d1) + b + e1)
    layer(7, B0, kL0, 0, 3);  // out
    if (!ok && tid == 0 && A.err) atomicOr(A.err, 1);
    // every MMA was waited for, unless a wait gave up: then keep the allocation rather
    // than free columns an MMA may still write
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0 && ok) tc::tmem_dealloc(taddr, 512);
}

// FP32 weights [co][tap][ci] (32 x 9 x 32) -> BF16 B operand in the core-matrix layout.
__global__ void pack_weights_kernel(const float* __restrict__ w32, __nv_bfloat16* __restrict__ wpk) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;  // one element
    if (e >= kC * kK) return;
    const int n = e / kK, k = e - n * kK;
    const int off = ((n >> 3) * kKC + (k >> 3)) * 64 + (n & 7) * 8 + (k & 7);  // in BF16 elements
    wpk[off] = __float2bfloat16_rn(w32[e]);
}

}  // namespace
}  // namespace fs

using namespace fs;

// Opt the tensor-core kernels into their dynamic shared memory on the current device.
cudaError_t fs::conv_prepare() {
    cudaError_t e = cudaFuncSetAttribute(conv3x3_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(net_infer32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kInfSmem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(wgrad_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kWgSmem);
}

int fs::net_infer32_launch(const void* x0, const void* wpk, const float* params, void* e1, float* y, int images,
                           int* err, const int* skip_if, void* stream) {
    if (!x0 || !wpk || !params || !e1 || !y || images < 1)
        return record_error(FS_ERR_ARG, "fs_net_infer32: bad argument");
    int dev = 0;
    cudaGetDevice(&dev);
    static unsigned long long configured = 0;
    if (!(configured & (1ull << (dev & 63)))) {
        if (cudaFuncSetAttribute(net_infer32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kInfSmem) !=
            cudaSuccess)
            return record_error(FS_ERR_CUDA, "fs_net_infer32: smem attribute");
        configured |= 1ull << (dev & 63);
    }
    InferArgs A;
    A.x0 = static_cast<const __nv_bfloat16*>(x0);
    A.wpk = static_cast<const __nv_bfloat16*>(wpk);
    A.params = params;
    A.e1 = static_cast<__nv_bfloat16*>(e1);
    A.y = y;
    A.err = err;
    A.skip_if = skip_if;
    net_infer32_kernel<<<images, kInfThreads, kInfSmem, (cudaStream_t)stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? FS_OK : record_error(FS_ERR_CUDA, "fs_net_infer32: launch failed");
}

extern "C" int fs_net_infer32(const void* x0, const void* wpk, const float* params, void* e1, float* y, int images,
                              int* err, void* stream) {
    return fs::net_infer32_launch(x0, wpk, params, e1, y, images, err, nullptr, stream);
}

extern "C" long long fs_net_weight_grad_tc_work_floats(int H, int W) {
    (void)H;
    (void)W;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    return 2LL * sms * kWgOut * kC;
}

extern "C" int fs_net_weight_grad_tc(const void* dzb, const void* x, float* dw, float* db, float* work,
                                     long long work_floats, int H, int W, int img_h, int up, int* err, void* stream) {
    if (!dzb || !x || !dw || !work || H < 1 || W < 1) return record_error(FS_ERR_ARG, "fs_net_weight_grad_tc: bad argument");
    if (img_h <= 0) img_h = H;
    if (H % img_h != 0) return record_error(FS_ERR_ARG, "fs_net_weight_grad_tc: H must be a multiple of img_h");
    if (up && ((img_h & 1) || (W & 1)))
        return record_error(FS_ERR_ARG, "fs_net_weight_grad_tc: upsampled output must be even");
    const long long per_block = (long long)kWgOut * kC;
    const long long max_blocks = work_floats / per_block;
    // two CTAs per SM
    if (max_blocks < 1) return record_error(FS_ERR_ARG, "fs_net_weight_grad_tc: workspace too small");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    static unsigned long long configured = 0;
    if (!(configured & (1ull << (dev & 63)))) {
        if (cudaFuncSetAttribute(wgrad_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kWgSmem) != cudaSuccess)
            return record_error(FS_ERR_CUDA, "fs_net_weight_grad_tc: smem attribute");
        configured |= 1ull << (dev & 63);
    }
    // two CTAs per SM at most, each over a whole number of 64-pixel chunks
    const long npix = (long)H * W;
    const long chunks = (npix + kWgK - 1) / kWgK;
    long nb = std::min<long>({2L * sms, chunks, (long)max_blocks});
    const long per = ((chunks + nb - 1) / nb) * kWgK;
    nb = (npix + per - 1) / per;
    WgradArgs P;
    P.x = static_cast<const __nv_bfloat16*>(x);
    P.dz = static_cast<const __nv_bfloat16*>(dzb);
    P.work = work;
    P.H = H;
    P.W = W;
    P.img_h = img_h;
    P.up = up;
    P.per = (int)per;
    P.err = err;
    cudaStream_t st = (cudaStream_t)stream;
    wgrad_tc_kernel<<<(unsigned)nb, kWgThreads, kWgSmem, st>>>(P);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return record_error(FS_ERR_CUDA, "fs_net_weight_grad_tc: launch failed");
    wgrad_reduce_kernel<<<(kWgOut * kC + 255) / 256, 256, 0, st>>>(work, (int)nb, dw, db);
    e = cudaGetLastError();
    return e == cudaSuccess ? FS_OK : record_error(FS_ERR_CUDA, "fs_net_weight_grad_tc: reduce launch failed");
}

extern "C" int fs_conv_pack_weights(const float* w32, void* wpk, void* stream) {
    if (!w32 || !wpk) return record_error(FS_ERR_ARG, "fs_conv_pack_weights: null pointer");
    pack_weights_kernel<<<(kC * kK + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        w32, static_cast<__nv_bfloat16*>(wpk));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FS_OK : record_error(FS_ERR_CUDA, "fs_conv_pack_weights: launch failed");
}

extern "C" int fs_conv3x3(const void* x, const void* wpk, const float* w32, const float* bias, const void* skip,
                          void* y, float* yf, int H, int W, int img_h, int up, int relu, int use_tensor_cores,
                          int* err, void* stream) {
    return fs::conv3x3_launch(x, wpk, w32, bias, skip, y, yf, H, W, img_h, up, relu, use_tensor_cores, err, nullptr,
                              stream);
}

int fs::conv3x3_launch(const void* x, const void* wpk, const float* w32, const float* bias, const void* skip, void* y,
                       float* yf, int H, int W, int img_h, int up, int relu, int use_tensor_cores, int* err,
                       const int* skip_if, void* stream) {
    if (!x || H < 1 || W < 1 || (!y && !yf)) return record_error(FS_ERR_ARG, "fs_conv3x3: bad argument");
    if (img_h <= 0) img_h = H;
    if (H % img_h != 0) return record_error(FS_ERR_ARG, "fs_conv3x3: H must be a multiple of img_h");
    if (up && ((img_h & 1) || (W & 1))) return record_error(FS_ERR_ARG, "fs_conv3x3: upsampled output must be even");
    ConvArgs P;
    P.x = static_cast<const __nv_bfloat16*>(x);
    P.wpk = static_cast<const __nv_bfloat16*>(wpk);
    P.bias = bias;
    P.skip = static_cast<const __nv_bfloat16*>(skip);
    P.y = static_cast<__nv_bfloat16*>(y);
    P.yf = yf;
    P.H = H;
    P.W = W;
    P.img_h = img_h;
    P.up = up;
    P.relu = relu;
    P.err = err;
    P.skip_if = skip_if;
    cudaStream_t st = (cudaStream_t)stream;
    const long npix = (long)H * W;
    if (use_tensor_cores) {
        if (!wpk) return record_error(FS_ERR_ARG, "fs_conv3x3: packed weights required");
        static unsigned long long configured = 0;
        int dev = 0;
        cudaGetDevice(&dev);
        if (!(configured & (1ull << (dev & 63)))) {
            cudaError_t e = cudaFuncSetAttribute(conv3x3_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 kConvSmem);
            if (e != cudaSuccess) return record_error(FS_ERR_CUDA, "fs_conv3x3: smem attribute");
            configured |= 1ull << (dev & 63);
        }
        conv3x3_tc_kernel<<<(unsigned)((npix + kTileM - 1) / kTileM), 128, kConvSmem, st>>>(P);
    } else {
        if (!w32) return record_error(FS_ERR_ARG, "fs_conv3x3: FP32 weights required");
        conv3x3_ref_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(P, w32);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FS_OK : record_error(FS_ERR_CUDA, "fs_conv3x3: launch failed");
}
