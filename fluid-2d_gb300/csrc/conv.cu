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

// Opt the tensor-core conv into its dynamic shared memory on the current device.
cudaError_t fs::conv_prepare() {
    return cudaFuncSetAttribute(conv3x3_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmem);
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
