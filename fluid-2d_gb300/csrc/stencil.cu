// Temporally blocked 5-point Jacobi passes for diffusion and pressure.
//
// Reference behaviour (mworchel/fluid-2d src/fluid_solver_gpu.cu):
//   diffuse 290-312 + diffuse_iteration_kernel 69-85: per sweep, a D2D copy of the
//     field, one Jacobi kernel, a device sync, one boundary kernel, a device sync;
//   project 358-404 + kernels 164-206: clear div and p, divergence, Neumann fill,
//     Kp x (copy, Jacobi, fill), gradient subtract, two reflecting fills.
// That is ~20 B/cell of HBM traffic and two launches per sweep. Here one launch runs
// `sweeps` sweeps of one or more fields: each CTA loads a 128-column region (its
// output tile grown by a halo H >= sweeps), iterates on chip with the
// boundary fill's effect reproduced exactly after every sweep, and writes only its
// output tile back. The first pass of a solve fuses what precedes it
// (add_sources for diffusion, the divergence for pressure) and the last pressure
// pass fuses the gradient subtract and the two reflecting fills.
//
// The sweeps are register-blocked (run_sweeps): each thread holds an 8 x 4 block of
// the field in registers, exchanges block edges with its neighbours by warp shuffles
// and a small shared-memory row exchange, and reads its constant terms (x0 or div) from
// shared memory, one barrier per sweep. Interior tiles of the diffusion passes and the
// middle pressure passes load and store the block layout straight from global memory
// (16-byte accesses); edge tiles and the first and last pressure passes stage the
// region in shared memory in a one-column-per-thread layout, where the masked loads,
// the fused divergence and the gradient epilogue run. The
// reference's per-sweep boundary fill is folded into the sweep (the cells next to a
// domain edge read what the fill would have stored there) and applied for real once,
// after the last sweep. Arithmetic follows the reference's operand order with explicit
// round-to-nearest intrinsics and a fused multiply-add exactly where the reference's
// compiled kernels fuse one (add_sources x + dt*s and the diffusion numerator
// x0 + a*sum). The reference divides by (1.0 + 4.0*a) in
// double; FP64 is slow on GB300, so the quotient is formed as
//   q = num*rf;  e = fma(-q, dh, num);  e = fma(-q, dl, e);  q = fma(e, rf, q)
// with dh + dl = 1 + 4a split into two floats and rf = (float)(1/(1 + 4a)). This
// Newton-corrected quotient agrees with (float)((double)num / (1.0 + 4.0*a)) except
// where the reference's double rounding lands exactly on a float tie (about one
// value in 10^8 in random testing).

#include <algorithm>

#include "fs_internal.cuh"

namespace fs {
namespace {

// ---------------------------------------------------------------------------
// Register-blocked sweeps.
//
// The region's RH x 128 cells are split among the CTA's NW warps: warp w owns rows
// [8w, 8w + 8) and lane l of a warp owns the four columns 4l .. 4l+3 of those rows, so
// each thread holds an 8 x 4 block of the field in registers for the whole pass, as
// float2 row pairs P[j][q] = (row j, row j + 4) of column q (j = 0..3). One packed
// FP32 instruction (FADD2 / FMUL2 / FFMA2, each lane rounding exactly as the scalar
// form) then updates two cells. Per sweep and row pair:
//   left / right neighbours: the thread's own columns, except the left one of column 0
//     and the right one of column 3, which come from the adjacent lanes by shuffles;
//   up / down neighbours: the thread's own rows, except above row 0 and below row 7,
//     which come from the adjacent warps through a small double-buffered exchange area
//     in shared memory (each warp publishes its rows 0 and 7 as float4);
//   constant term (x0 or div): shared memory, in a layout where one float4 holds the
//     row pair's values of two columns (kidx).
// The new values go to a second register block (the sweep loop alternates the two), so
// no register is copied. Per 128 cell updates of a warp: 8 FP instructions per cell pair
// (diffusion) or 5 (pressure), 2 shuffles, 4 wavefronts of constant loads and 4 of row
// exchange, and one barrier per sweep.
// Cells at the region border read clamped or wrapped neighbours and compute values that
// nothing stored depends on (the halo is at least the number of sweeps).
//
// Domain edges. The reference fills the edge cells after every sweep with their inner
// neighbour's new value times a sign (set_boundary_*, fluid_solver_gpu.cu:11-54), corners
// excepted. Here every cell of the block is updated by the stencil (edge, corner and
// outside cells compute values nothing uses), and from the second sweep on, before the
// sweep reads them, the edge cells the interior reads are filled exactly as the
// reference fills them: in the thread itself where edge and inner cell share a thread,
// and otherwise in the value received from the neighbour (the shuffled column or the
// exchanged row is replaced by sign x the interior cell's own value, the float the fill
// would have stored there). After the last sweep fill_edges applies the fill for the
// stores, and the corners get their loaded values back (restore_corners).

struct Coef2 {
    float2 a, ndh, ndl, rf;  // diffusion: a, -dh, -dl and rf of the quotient (head of this file)
};

template <bool DIFF>
__device__ __forceinline__ float2 update2(float2 k, float2 L, float2 R, float2 U, float2 D, const Coef2& c) {
    if (DIFF) {
        // (x0 + a*(L + R + U + D)) / (1 + 4a), fluid_solver_gpu.cu:81-82: the numerator
        // fused as in the compiled reference, the quotient Newton-corrected in FP32 (see
        // the head of this file)
        float2 s = __fadd2_rn(L, R);
        s = __fadd2_rn(s, U);
        s = __fadd2_rn(s, D);
        const float2 num = __ffma2_rn(c.a, s, k);
        const float2 q = __fmul2_rn(num, c.rf);
        float2 e = __ffma2_rn(q, c.ndh, num);
        e = __ffma2_rn(q, c.ndl, e);
        return __ffma2_rn(e, c.rf, q);
    } else {
        // (div + R + L + D + U) / 4, fluid_solver_gpu.cu:187-188
        float2 s = __fadd2_rn(k, R);
        s = __fadd2_rn(s, L);
        s = __fadd2_rn(s, D);
        s = __fadd2_rn(s, U);
        return __fmul2_rn(s, make_float2(0.25f, 0.25f));
    }
}

// Offset of the constant term of region cell (r, c) in its shared buffer: per warp
// block of 8 rows, row pair j = r & 3, plane (c & 2) (columns 0-1 or 2-3 of a lane),
// lane c / 4, then (column c & 1, row half (r >> 2) & 1) — so that a lane's float4 at
// (j, plane) is (k[j][q], k[j+4][q], k[j][q+1], k[j+4][q+1]) and a warp's float4 loads
// of one plane are 512 contiguous bytes.
__device__ __forceinline__ int kidx(int r, int c) {
    return (r >> 3) * (8 * kRegionW) + (r & 3) * (2 * kRegionW) + ((c >> 1) & 1) * kRegionW + (c >> 2) * 4 +
           (c & 1) * 2 + ((r >> 2) & 1);
}

// x / b correctly rounded, for b > 0 with y = RN(1/b): Markstein's correction step
// (P. Markstein, "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990): q0 = RN(x*y), r = x - q0*b (exact with one
// FMA), RN(q0 + r*y) = RN(x/b) while x, the quotient and r stay in the normal range.
// Zero (x / b = x for b > 0), very small or large and non-finite x take the IEEE
// division. Used for the gradient subtract's division by h.
__device__ __noinline__ float ieee_div(float x, float b) { return __fdiv_rn(x, b); }

__device__ __forceinline__ float div_by(float x, float b, float y) {
    const float ax = fabsf(x);
    if (ax > 0x1p-100f && ax < 0x1p100f) {
        const float q0 = __fmul_rn(x, y);
        const float r = __fmaf_rn(-q0, b, x);
        return __fmaf_rn(r, y, q0);
    }
    return ax == 0.f ? x : ieee_div(x, b);  // out of line: rare, and keeps the epilogue small
}

struct EdgeGeom {
    int i1, i2;  // block row of grid row 1 / rows - 2 (out of 0..7: none)
    int q1, q2;  // block column of grid column 1 / cols - 2 (out of 0..3: none)
    float s_lr, s_tb;
};

template <int I> __device__ __forceinline__ float& rowref(float2 (&X)[4][4], int q) {
    return (I >> 2) ? X[I & 3][q].y : X[I & 3][q].x;
}
template <int DST, int SRC> __device__ __forceinline__ void fill_row(float2 (&X)[4][4], float sg) {
#pragma unroll
    for (int q = 0; q < 4; ++q) rowref<DST>(X, q) = __fmul_rn(sg, rowref<SRC>(X, q));
}
template <int DST, int SRC> __device__ __forceinline__ void fill_col(float2 (&X)[4][4], float sg) {
#pragma unroll
    for (int j = 0; j < 4; ++j) X[j][DST] = make_float2(__fmul_rn(sg, X[j][SRC].x), __fmul_rn(sg, X[j][SRC].y));
}

// The in-thread part of the reference's edge fill on the previous sweep's values:
// left/right edge columns from their inner column, top/bottom edge rows from their
// inner row, where both lie in this thread's block. Corner and outside cells this also
// writes are never read by interior cells.
__device__ __forceinline__ void fill_in_thread(float2 (&X)[4][4], const EdgeGeom& g) {
    switch (g.q1) {  // grid column 0 = block column q1 - 1
        case 1: fill_col<0, 1>(X, g.s_lr); break;
        case 2: fill_col<1, 2>(X, g.s_lr); break;
        case 3: fill_col<2, 3>(X, g.s_lr); break;
        default: break;
    }
    switch (g.q2) {  // grid column cols - 1 = block column q2 + 1
        case 0: fill_col<1, 0>(X, g.s_lr); break;
        case 1: fill_col<2, 1>(X, g.s_lr); break;
        case 2: fill_col<3, 2>(X, g.s_lr); break;
        default: break;
    }
    switch (g.i1) {  // grid row 0 = block row i1 - 1
        case 1: fill_row<0, 1>(X, g.s_tb); break;
        case 2: fill_row<1, 2>(X, g.s_tb); break;
        case 3: fill_row<2, 3>(X, g.s_tb); break;
        case 4: fill_row<3, 4>(X, g.s_tb); break;
        case 5: fill_row<4, 5>(X, g.s_tb); break;
        case 6: fill_row<5, 6>(X, g.s_tb); break;
        case 7: fill_row<6, 7>(X, g.s_tb); break;
        default: break;
    }
    switch (g.i2) {  // grid row rows - 1 = block row i2 + 1
        case 0: fill_row<1, 0>(X, g.s_tb); break;
        case 1: fill_row<2, 1>(X, g.s_tb); break;
        case 2: fill_row<3, 2>(X, g.s_tb); break;
        case 3: fill_row<4, 3>(X, g.s_tb); break;
        case 4: fill_row<5, 4>(X, g.s_tb); break;
        case 5: fill_row<6, 5>(X, g.s_tb); break;
        case 6: fill_row<7, 6>(X, g.s_tb); break;
        default: break;
    }
}

// One sweep X -> Y. K: this thread's constant terms (kidx layout, warp block base +
// 4 * lane); E: the exchange buffer of this sweep; my_top/my_bot/nb_up/nb_dn: offsets of
// this warp's published rows and of the neighbours' rows in it.
template <bool DIFF, bool EDGE>
__device__ __forceinline__ void sweep(float2 (&X)[4][4], float2 (&Y)[4][4], const float* __restrict__ K,
                                      float* __restrict__ E, int my_top, int my_bot, int nb_up, int nb_dn, bool fold,
                                      const EdgeGeom& g, const Coef2& c) {
    constexpr int RW = kRegionW;
    constexpr unsigned FULL = 0xffffffffu;
    if (EDGE && fold) fill_in_thread(X, g);
    *reinterpret_cast<float4*>(E + my_top) = make_float4(X[0][0].x, X[0][1].x, X[0][2].x, X[0][3].x);
    *reinterpret_cast<float4*>(E + my_bot) = make_float4(X[3][0].y, X[3][1].y, X[3][2].y, X[3][3].y);
    __syncthreads();
    const float4 u4 = *reinterpret_cast<const float4*>(E + nb_up);
    const float4 d4 = *reinterpret_cast<const float4*>(E + nb_dn);
    float up[4] = {u4.x, u4.y, u4.z, u4.w}, dn[4] = {d4.x, d4.y, d4.z, d4.w};
    if (EDGE && fold) {
        if (g.i1 == 0) {  // grid row 0 is the row above this block
#pragma unroll
            for (int q = 0; q < 4; ++q) up[q] = __fmul_rn(g.s_tb, X[0][q].x);
        }
        if (g.i2 == 7) {  // grid row rows - 1 is the row below this block
#pragma unroll
            for (int q = 0; q < 4; ++q) dn[q] = __fmul_rn(g.s_tb, X[3][q].y);
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float2 L0 = make_float2(__shfl_up_sync(FULL, X[j][3].x, 1), __shfl_up_sync(FULL, X[j][3].y, 1));
        float2 R3 = make_float2(__shfl_down_sync(FULL, X[j][0].x, 1), __shfl_down_sync(FULL, X[j][0].y, 1));
        if (EDGE && fold) {
            if (g.q1 == 0) L0 = make_float2(__fmul_rn(g.s_lr, X[j][0].x), __fmul_rn(g.s_lr, X[j][0].y));
            if (g.q2 == 3) R3 = make_float2(__fmul_rn(g.s_lr, X[j][3].x), __fmul_rn(g.s_lr, X[j][3].y));
        }
        const float4 ka = *reinterpret_cast<const float4*>(K + j * (2 * RW));
        const float4 kb = *reinterpret_cast<const float4*>(K + j * (2 * RW) + RW);
        const float2 kk[4] = {make_float2(ka.x, ka.y), make_float2(ka.z, ka.w), make_float2(kb.x, kb.y),
                              make_float2(kb.z, kb.w)};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float2 L = q > 0 ? X[j][q - 1] : L0;
            const float2 R = q < 3 ? X[j][q + 1] : R3;
            const float2 U = j > 0 ? X[j - 1][q] : make_float2(up[q], X[3][q].x);
            const float2 D = j < 3 ? X[j + 1][q] : make_float2(X[0][q].y, dn[q]);
            Y[j][q] = update2<DIFF>(kk[q], L, R, U, D, c);
        }
    }
}

template <bool DIFF, bool EDGE, int NW>
__device__ __forceinline__ void run_sweeps(float2 (&X)[4][4], int koff, int eoff, int nsweeps, int w, int lane,
                                           const EdgeGeom& g, const Coef2& c) {
    constexpr int RW = kRegionW;
    extern __shared__ float4 smem4[];
    float* const S = reinterpret_cast<float*>(smem4);
    const float* const K = S + koff + w * (8 * RW) + 4 * lane;
    float* const E0 = S + eoff;
    float* const E1 = E0 + 2 * NW * RW;  // the second exchange buffer
    const int my_top = (2 * w) * RW + 4 * lane;
    const int my_bot = my_top + RW;
    // bottom row of warp w - 1 and top row of warp w + 1; the first and last warps read
    // their own rows instead (the region border, whose values nothing stored uses)
    const int nb_up = w > 0 ? my_top - RW : my_top;
    const int nb_dn = w < NW - 1 ? my_top + 2 * RW : my_bot;
    float2 Y[4][4];
    int s = 0;
#pragma unroll 1
    for (; s + 1 < nsweeps; s += 2) {
        sweep<DIFF, EDGE>(X, Y, K, E0, my_top, my_bot, nb_up, nb_dn, s > 0, g, c);
        sweep<DIFF, EDGE>(Y, X, K, E1, my_top, my_bot, nb_up, nb_dn, true, g, c);
    }
    if (s < nsweeps) {
        sweep<DIFF, EDGE>(X, Y, K, E0, my_top, my_bot, nb_up, nb_dn, s > 0, g, c);
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) X[j][q] = Y[j][q];
    }
}

// The reference's boundary fill applied once to the final sweep in S + co: edge cells
// (corners excepted) take their inner neighbour's value times the field's sign. Reads
// touch interior cells only and writes edge cells only, so one barrier after suffices.
template <int SR, int RH>
__device__ __forceinline__ void fill_edges(int co, int r0, int tx, int txl, int txr, int g0, int gc, int rows,
                                           int cols, float s_lr, float s_tb) {
    constexpr int RW = kRegionW;
    extern __shared__ float4 smem4[];
    float* const S = reinterpret_cast<float*>(smem4) + co;
    if (gc >= 1 && gc <= cols - 2) {
        const int it = -g0, ib = rows - 1 - g0;  // segment rows of grid rows 0 and rows - 1
        if (it >= 0 && it < SR) {
            const int r = r0 + it;
            S[r * RW + tx] = s_tb * S[min(r + 1, RH - 1) * RW + tx];
        }
        if (ib >= 0 && ib < SR) {
            const int r = r0 + ib;
            S[r * RW + tx] = s_tb * S[max(r - 1, 0) * RW + tx];
        }
    } else if (gc == 0 || gc == cols - 1) {
        const int src = gc == 0 ? txr : txl;
#pragma unroll
        for (int i = 0; i < SR; ++i) {
            const int gr = g0 + i;
            if (gr >= 1 && gr <= rows - 2) S[(r0 + i) * RW + tx] = s_lr * S[(r0 + i) * RW + src];
        }
    }
    __syncthreads();
}

// Tile b of a pass in dispatch order: the domain-edge tiles first (their sweeps carry
// the edge folding and a final fill, ~20 % more time), then the interior row by row, so
// that the last tiles a pass starts are the short ones.
__device__ __forceinline__ void tile_coords(int b, int tx_n, int ty_n, int& tyi, int& txi) {
    if (tx_n <= 2 || ty_n <= 2) {
        tyi = b / tx_n;
        txi = b - tyi * tx_n;
        return;
    }
    const int side = ty_n - 2;
    if (b < 2 * tx_n) {  // top and bottom rows
        tyi = b < tx_n ? 0 : ty_n - 1;
        txi = b < tx_n ? b : b - tx_n;
    } else if (b < 2 * tx_n + 2 * side) {  // left and right columns
        const int k = b - 2 * tx_n;
        tyi = 1 + (k < side ? k : k - side);
        txi = k < side ? 0 : tx_n - 1;
    } else {
        const int k = b - 2 * tx_n - 2 * side, w = tx_n - 2;
        tyi = 1 + k / w;
        txi = 1 + (k - (k / w) * w);
    }
}

// Interior tiles of the passes without an epilogue (diffusion passes, middle pressure
// passes) need neither the column layout nor any masking: the region lies inside the
// grid's interior, so every cell is loaded and every cell is live. There the field and
// its constant term go straight from global memory into the block layout (a lane's four
// columns of a row are one 16-byte load, a warp's row 512 contiguous bytes), and the
// final field straight back from registers, without staging the region in shared
// memory ("direct" tiles). Requires the region's first column and the row pitch to be
// multiples of four floats and the buffers 16-byte aligned (checked by the caller).
// Flags of a tile's sweep phase.
constexpr int kSwEdge = 1;    // a domain-edge tile (edge folding in the sweeps)
constexpr int kSwDirect = 2;  // a direct tile: global -> registers -> global
constexpr int kSwFirst = 4;   // direct loads: first diffusion pass (add_sources fused)
constexpr int kSwResid = 8;   // direct: residual partial sums wanted
constexpr int kSwLoad = 16;   // direct tiles: load global -> registers
constexpr int kSwDiv = 32;    // direct loads: first pressure pass (divergence of u, v from P.F)
struct SweepParams {
    int nsweeps, flags, gy0, gx0, rows, cols;
    float s_lr, s_tb, a, dh, dl, rf;
    // direct tiles only
    const float* x;  // field in
    const float* k;  // constant term in (x0 / div), or the source s of a first diffusion pass
    float* y;        // field out (output tile; may be null)
    float* kout;     // first diffusion pass: x0 out (output tile; may be null)
    int pitch, halo, halo_l, tile_h, tile_w;  // halo_l: left margin (columns)
    float dt;
    const StencilField* F;  // last pressure pass: the gradient epilogue's fields (else null)
};

// Stores the four values v of one block row (columns cb .. cb+3 of the region) where
// they fall in the output columns [c_lo, c_hi) (relative to cb).
__device__ __forceinline__ void store_row4(float* p, float4 v, int c_lo, int c_hi) {
    if (c_lo <= 0 && c_hi >= 4) {
        *reinterpret_cast<float4*>(p) = v;
    } else {
        if (c_lo <= 0 && c_hi > 0) p[0] = v.x;
        if (c_lo <= 1 && c_hi > 1) p[1] = v.y;
        if (c_lo <= 2 && c_hi > 2) p[2] = v.z;
        if (c_lo <= 3 && c_hi > 3) p[3] = v.w;
    }
}

// Gradient subtract of a direct tile of the last pressure pass (remove_p_kernel,
// fluid_solver_gpu.cu:202-203): u -= (0.5*(pR - pL))/h, v -= (0.5*(pD - pU))/h on the
// output cells, from the final pressure block in registers. Left/right neighbours of the
// block's edge columns come by shuffles, the rows above and below by one more row
// exchange, in the buffer the last sweep did not use (`eoff`). Interior tiles only: no
// reflecting fill is needed.
template <int NW>
__device__ __forceinline__ void gradient_direct(const float2 (&X)[4][4], int eoff, int w, int lane, size_t o,
                                                size_t pitch, int r_lo, int r_hi, int c_lo, int c_hi,
                                                const StencilField& F) {
    constexpr int RW = kRegionW;
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ float4 smem4[];
    float* const E = reinterpret_cast<float*>(smem4) + eoff;
    const bool out_cols = c_lo < 4 && c_hi > 0;
    auto pv = [&](int ii, int q) -> float { return (ii >> 2) ? X[ii & 3][q].y : X[ii & 3][q].x; };
    auto live = [&](int i) { return out_cols && i >= r_lo && i < r_hi; };
    // u and v of the first four rows are loaded before the exchange's barrier, so their
    // latency overlaps it; those of the last four rows are loaded together
    float4 uu[4], vv[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        uu[i] = live(i) ? __ldcg(reinterpret_cast<const float4*>(F.u_in + o + i * pitch)) : make_float4(0, 0, 0, 0);
        vv[i] = live(i) ? __ldcg(reinterpret_cast<const float4*>(F.v_in + o + i * pitch)) : make_float4(0, 0, 0, 0);
    }
    const int my_top = (2 * w) * RW + 4 * lane, my_bot = my_top + RW;
    const int nb_up = w > 0 ? my_top - RW : my_top;
    const int nb_dn = w < NW - 1 ? my_top + 2 * RW : my_bot;
    *reinterpret_cast<float4*>(E + my_top) = make_float4(X[0][0].x, X[0][1].x, X[0][2].x, X[0][3].x);
    *reinterpret_cast<float4*>(E + my_bot) = make_float4(X[3][0].y, X[3][1].y, X[3][2].y, X[3][3].y);
    __syncthreads();
    const float4 u4 = *reinterpret_cast<const float4*>(E + nb_up);
    const float4 d4 = *reinterpret_cast<const float4*>(E + nb_dn);
    const float up[4] = {u4.x, u4.y, u4.z, u4.w}, dn[4] = {d4.x, d4.y, d4.z, d4.w};
    const float h = F.h, rh = __frcp_rn(h);
    int bad = 0;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        float L0[4], R3[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = half * 4 + k;
            L0[k] = __shfl_up_sync(FULL, pv(i, 3), 1);
            R3[k] = __shfl_down_sync(FULL, pv(i, 0), 1);
        }
        float4 un4[4], vn4[4];
        if (half == 1) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int i = 4 + k;
                uu[k] = live(i) ? __ldcg(reinterpret_cast<const float4*>(F.u_in + o + i * pitch)) : make_float4(0, 0, 0, 0);
                vv[k] = live(i) ? __ldcg(reinterpret_cast<const float4*>(F.v_in + o + i * pitch)) : make_float4(0, 0, 0, 0);
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = half * 4 + k;
            const float uin[4] = {uu[k].x, uu[k].y, uu[k].z, uu[k].w}, vin[4] = {vv[k].x, vv[k].y, vv[k].z, vv[k].w};
            float un[4], vn[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float pl = q > 0 ? pv(i, q - 1) : L0[k];
                const float pr = q < 3 ? pv(i, q + 1) : R3[k];
                const float pu = i > 0 ? pv(i - 1, q) : up[q];
                const float pd = i < 7 ? pv(i + 1, q) : dn[q];
                const float gu = div_by(__fmul_rn(0.5f, __fsub_rn(pr, pl)), h, rh);
                const float gv = div_by(__fmul_rn(0.5f, __fsub_rn(pd, pu)), h, rh);
                un[q] = __fsub_rn(uin[q], gu);
                vn[q] = __fsub_rn(vin[q], gv);
                if (live(i) && q >= c_lo && q < c_hi) bad |= !(isfinite(un[q]) && isfinite(vn[q]));
            }
            un4[k] = make_float4(un[0], un[1], un[2], un[3]);
            vn4[k] = make_float4(vn[0], vn[1], vn[2], vn[3]);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = half * 4 + k;
            if (!live(i)) continue;
            store_row4(F.u_out + o + i * pitch, un4[k], c_lo, c_hi);
            store_row4(F.v_out + o + i * pitch, vn4[k], c_lo, c_hi);
        }
    }
    if (bad && F.nonfinite) atomicOr(F.nonfinite, 1);
}

// Residual partial sums of a direct tile of a residual-target pass: over the output cells,
// ||div + R + L + D + U - 4p||^2 and ||div||^2 of the final pressure block in registers,
// div read back from this thread's constant terms (K, kidx layout), the neighbours by
// shuffles and one more row exchange (in the buffer the last sweep did not use). Interior
// tiles only, so every output cell is an interior cell. Returns (rnum, rden).
template <int NW>
__device__ __forceinline__ float2 residual_direct(const float2 (&X)[4][4], int eoff, const float* __restrict__ K,
                                                  int w, int lane, int r_lo, int r_hi, int c_lo, int c_hi) {
    constexpr int RW = kRegionW;
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ float4 smem4[];
    float* const E = reinterpret_cast<float*>(smem4) + eoff;
    const int my_top = (2 * w) * RW + 4 * lane, my_bot = my_top + RW;
    const int nb_up = w > 0 ? my_top - RW : my_top;
    const int nb_dn = w < NW - 1 ? my_top + 2 * RW : my_bot;
    *reinterpret_cast<float4*>(E + my_top) = make_float4(X[0][0].x, X[0][1].x, X[0][2].x, X[0][3].x);
    *reinterpret_cast<float4*>(E + my_bot) = make_float4(X[3][0].y, X[3][1].y, X[3][2].y, X[3][3].y);
    __syncthreads();
    const float4 u4 = *reinterpret_cast<const float4*>(E + nb_up);
    const float4 d4 = *reinterpret_cast<const float4*>(E + nb_dn);
    const float up[4] = {u4.x, u4.y, u4.z, u4.w}, dn[4] = {d4.x, d4.y, d4.z, d4.w};
    auto pv = [&](int ii, int q) -> float { return (ii >> 2) ? X[ii & 3][q].y : X[ii & 3][q].x; };
    const bool out_cols = c_lo < 4 && c_hi > 0;
    float rnum = 0.f, rden = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float L0 = __shfl_up_sync(FULL, pv(i, 3), 1);
        const float R3 = __shfl_down_sync(FULL, pv(i, 0), 1);
        if (!out_cols || i < r_lo || i >= r_hi) continue;
        const int j = i & 3, hsel = i >> 2;
        const float4 ka = *reinterpret_cast<const float4*>(K + j * (2 * RW));
        const float4 kb = *reinterpret_cast<const float4*>(K + j * (2 * RW) + RW);
        const float kk[4] = {hsel ? ka.y : ka.x, hsel ? ka.w : ka.z, hsel ? kb.y : kb.x, hsel ? kb.w : kb.z};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (q < c_lo || q >= c_hi) continue;
            const float pl = q > 0 ? pv(i, q - 1) : L0;
            const float pr = q < 3 ? pv(i, q + 1) : R3;
            const float pu = i > 0 ? pv(i - 1, q) : up[q];
            const float pd = i < 7 ? pv(i + 1, q) : dn[q];
            // the staged residual's order: div + R + L + D + U - 4p
            float sres = __fadd_rn(kk[q], pr);
            sres = __fadd_rn(sres, pl);
            sres = __fadd_rn(sres, pd);
            sres = __fadd_rn(sres, pu);
            const float res = __fsub_rn(sres, __fmul_rn(4.f, pv(i, q)));
            rnum = fmaf(res, res, rnum);
            rden = fmaf(kk[q], kk[q], rden);
        }
    }
    return make_float2(rnum, rden);
}

// The sweeps of one tile in the block layout of run_sweeps. Staged tiles: the field
// comes from shared memory (row-major at xoff) and goes back there; direct tiles: from
// and to global memory, the constant terms written to shared memory here. The sweeps
// read the constant terms at koff in the kidx layout, the exchange area overlaying the
// field's buffer. Kept out of line so that the tile body's other live values are saved
// once around the call instead of competing with the register blocks, and so that
// staged and direct interior tiles share one copy of the sweep loop.
// MODE bits: 1 direct tiles, 2 the direct gradient epilogue, 4 the direct residual sums,
// 16 direct first pressure passes (the divergence formed in registers). Edge tiles are
// always staged: masked direct loads for them were measured slower, on a large grid and
// over a batch of small ones alike.
// A direct residual tile leaves its thread's partial sums (rnum, rden) in shared memory
// at resid_slot(), in the exchange buffer the last sweep used (free once every warp has
// passed the final exchange's barrier).
constexpr int kModeDirect = 1, kModeGrad = 2, kModeResid = 4, kModeDiv = 16;
template <int NW>
__device__ __forceinline__ int resid_slot(int xoff, int nsweeps, int tid) {
    return xoff + (((nsweeps & 1) ^ 1) * (2 * NW * kRegionW)) + 2 * tid;
}
template <bool DIFF, int NW, int MODE>
__device__ __noinline__ void sweep_phase(int xoff, int koff, const SweepParams P) {
    constexpr int RW = kRegionW;
    extern __shared__ float4 smem4[];
    float* const S = reinterpret_cast<float*>(smem4);
    float* const X = S + xoff;
    const int tid = threadIdx.y * RW + threadIdx.x;
    const int w = tid >> 5, lane = tid & 31;
    const int rb = w * 8, cb = 4 * lane;
    const size_t pitch = (size_t)P.pitch;
    const size_t o = (size_t)(P.gy0 + rb) * pitch + (size_t)(P.gx0 + cb);
    // direct tiles: output rows [r_lo, r_hi) and columns [c_lo, c_hi) relative to this
    // thread's block
    const int r_lo = P.halo - rb, r_hi = P.halo + P.tile_h - rb;
    const int c_lo = P.halo_l - cb, c_hi = P.halo_l + P.tile_w - cb;
    const bool out_cols = c_lo < 4 && c_hi > 0;
    float2 xb[4][4];
    if ((MODE & kModeDirect) && (P.flags & kSwLoad)) {
        float* const K = S + koff + w * (8 * RW) + 4 * lane;
        float4 t[8], kk[8];
        if ((MODE & kModeDiv) && (P.flags & kSwDiv)) {
            // divergence_kernel (fluid_solver_gpu.cu:173-174): div = cdiv*(((uR - uL) + vD) - vU)
            // on every cell of the region (a direct tile's region lies inside the grid's
            // interior); the starting pressure (zero without one). u's left/right neighbours
            // of the block's edge columns come by shuffles, v's rows above and below the block
            // straight from global memory (a region-border row or column gets a value that
            // only halo cells depend on).
            const StencilField& Fd = *P.F;
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            auto load = [&](const float* base, int i) {
                return __ldcg(reinterpret_cast<const float4*>(base + (long long)o + (long long)i * (long long)pitch));
            };
            const float cdiv = Fd.cdiv;
            float4 vu = load(Fd.x2, -1), vc = load(Fd.x2, 0);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const float4 vd = load(Fd.x2, i + 1);
                const float4 u = load(Fd.x, i);
                const float uL = __shfl_up_sync(0xffffffffu, u.w, 1), uR = __shfl_down_sync(0xffffffffu, u.x, 1);
                const float ul[4] = {uL, u.x, u.y, u.z}, ur[4] = {u.y, u.z, u.w, uR};
                const float dn[4] = {vd.x, vd.y, vd.z, vd.w}, upv[4] = {vu.x, vu.y, vu.z, vu.w};
                float dv[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    float sd = __fsub_rn(ur[q], ul[q]);
                    sd = __fadd_rn(sd, dn[q]);
                    sd = __fsub_rn(sd, upv[q]);
                    dv[q] = __fmul_rn(cdiv, sd);
                }
                kk[i] = make_float4(dv[0], dv[1], dv[2], dv[3]);
                vu = vc;
                vc = vd;
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) t[i] = Fd.cst ? load(Fd.cst, i) : z;
        } else {
#pragma unroll
            for (int i = 0; i < 8; ++i) t[i] = __ldcg(reinterpret_cast<const float4*>(P.x + o + i * pitch));
#pragma unroll
            for (int i = 0; i < 8; ++i) kk[i] = __ldcg(reinterpret_cast<const float4*>(P.k + o + i * pitch));
            if (P.flags & kSwFirst) {
                // add_sources_kernel (fluid_solver_gpu.cu:64), fused as compiled: x0 = x + dt*s
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    t[i].x = __fmaf_rn(P.dt, kk[i].x, t[i].x);
                    t[i].y = __fmaf_rn(P.dt, kk[i].y, t[i].y);
                    t[i].z = __fmaf_rn(P.dt, kk[i].z, t[i].z);
                    t[i].w = __fmaf_rn(P.dt, kk[i].w, t[i].w);
                    kk[i] = t[i];
                }
            }
        }
        if ((P.flags & (kSwFirst | kSwDiv)) && (P.flags & kSwDirect)) {
            if (P.kout != nullptr && out_cols) {
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    if (i >= r_lo && i < r_hi) store_row4(P.kout + o + i * pitch, kk[i], c_lo, c_hi);
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            xb[j][0] = make_float2(t[j].x, t[j + 4].x);
            xb[j][1] = make_float2(t[j].y, t[j + 4].y);
            xb[j][2] = make_float2(t[j].z, t[j + 4].z);
            xb[j][3] = make_float2(t[j].w, t[j + 4].w);
            // kidx layout: (row j, row j+4) of columns (0, 1), then of columns (2, 3); each
            // thread reads back only the constant terms it wrote
            *reinterpret_cast<float4*>(K + j * (2 * RW)) = make_float4(kk[j].x, kk[j + 4].x, kk[j].y, kk[j + 4].y);
            *reinterpret_cast<float4*>(K + j * (2 * RW) + RW) =
                make_float4(kk[j].z, kk[j + 4].z, kk[j].w, kk[j + 4].w);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float4 t = *reinterpret_cast<const float4*>(X + (rb + j) * RW + cb);
            const float4 b = *reinterpret_cast<const float4*>(X + (rb + j + 4) * RW + cb);
            xb[j][0] = make_float2(t.x, b.x);
            xb[j][1] = make_float2(t.y, b.y);
            xb[j][2] = make_float2(t.z, b.z);
            xb[j][3] = make_float2(t.w, b.w);
        }
        __syncthreads();  // the exchange area of the sweeps overlays the field's buffer
    }
    const Coef2 c = {make_float2(P.a, P.a), make_float2(-P.dh, -P.dh), make_float2(-P.dl, -P.dl),
                     make_float2(P.rf, P.rf)};
    if (P.flags & kSwEdge) {
        const int gyb = P.gy0 + rb, gxb = P.gx0 + cb;
        const EdgeGeom g = {1 - gyb, P.rows - 2 - gyb, 1 - gxb, P.cols - 2 - gxb, P.s_lr, P.s_tb};
        run_sweeps<DIFF, true, NW>(xb, koff, xoff, P.nsweeps, w, lane, g, c);
    } else {
        const EdgeGeom g = {-1, -1, -1, -1, P.s_lr, P.s_tb};
        run_sweeps<DIFF, false, NW>(xb, koff, xoff, P.nsweeps, w, lane, g, c);
    }
    if ((MODE & kModeDirect) && (P.flags & kSwDirect)) {
        if (P.y != nullptr && out_cols) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                if (i < r_lo || i >= r_hi) continue;
                const int j = i & 3;
                const float4 v = (i < 4) ? make_float4(xb[j][0].x, xb[j][1].x, xb[j][2].x, xb[j][3].x)
                                         : make_float4(xb[j][0].y, xb[j][1].y, xb[j][2].y, xb[j][3].y);
                store_row4(P.y + o + i * pitch, v, c_lo, c_hi);
            }
        }
        const int efin = xoff + (P.nsweeps & 1) * (2 * NW * RW);  // exchange buffer the last sweep did not use
        if ((MODE & kModeGrad) && P.F != nullptr && P.F->epilogue)
            gradient_direct<NW>(xb, efin, w, lane, o, pitch, r_lo, r_hi, c_lo, c_hi, *P.F);
        if ((MODE & kModeResid) && (P.flags & kSwResid)) {
            const float2 r =
                residual_direct<NW>(xb, efin, S + koff + w * (8 * RW) + 4 * lane, w, lane, r_lo, r_hi, c_lo, c_hi);
            *reinterpret_cast<float2*>(S + resid_slot<NW>(xoff, P.nsweeps, tid)) = r;
        }
        return;  // the next tile's first barrier orders the exchange area's reuse
    }
    __syncthreads();  // every warp has read its last exchange rows
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        *reinterpret_cast<float4*>(X + (rb + j) * RW + cb) =
            make_float4(xb[j][0].x, xb[j][1].x, xb[j][2].x, xb[j][3].x);
        *reinterpret_cast<float4*>(X + (rb + j + 4) * RW + cb) =
            make_float4(xb[j][0].y, xb[j][1].y, xb[j][2].y, xb[j][3].y);
    }
    __syncthreads();
}

// One tile of one pass: load the region (fusing add_sources or the divergence into
// the first pass), run F.sweeps sweeps (edge CTAs: with the boundary fill folded in and
// applied once at the end), store the
// output tile, then the optional gradient-subtract epilogue and the optional residual
// partial sums (for residual-driven pressure solves). xin/yout stand in for F.x/F.y so
// a persistent caller can ping-pong buffers across passes.
// MODE as for sweep_phase.
template <int TY, int SRB, bool DIFF, int MODE = kModeDirect | kModeGrad>
__device__ __forceinline__ void process_tile(const StencilField& F, int b, const float* __restrict__ xin,
                                             float* __restrict__ yout, bool resid,
                                             float& rnum, float& rden) {
    // Two thread layouts over the same region: the column layout (thread = one column,
    // SR consecutive rows; coalesced global loads and stores, the fused first-pass
    // arithmetic, the epilogues) and the block layout of run_sweeps.
    constexpr int RW = kRegionW, NW = 4 * TY, RH = NW * SRB, SR = RH / TY;
    static_assert(SR <= 32, "column-layout row masks are 32-bit");
    static_assert(SRB == 8, "run_sweeps holds 8 rows per warp");
    extern __shared__ float4 smem4[];
    float* const S = reinterpret_cast<float*>(smem4);
    constexpr int co = 0, no = RH * RW;  // S + co: the field; S + no: its constant term
    __syncthreads();  // the previous tile of this CTA may still be reading shared memory
    int tyi, txi;
    tile_coords(b, F.tiles_x, F.tiles_y, tyi, txi);
    const int H = F.halo;
    const int gy0 = tyi * F.tile_h - F.shift_y - H;
    // region start column; a realigned tiling moves it down to a multiple of four, which
    // widens the left margin to HL (the tile width leaves room on the right)
    const int gx0h = txi * F.tile_w - F.shift_x - H;
    const int gx0 = F.realign ? (gx0h & ~3) : gx0h;
    const int HL = H + (gx0h - gx0);
    const int rows = F.rows, cols = F.cols;
    const size_t pitch = (size_t)F.pitch;
    const int kind = F.kind;
    const int tx = threadIdx.x, r0 = threadIdx.y * SR;
    const int gc = gx0 + tx;
    const bool col_in = gc >= 0 && gc < cols;
    const bool col_int = gc >= 1 && gc <= cols - 2;
    const int txl = tx > 0 ? tx - 1 : 0;
    const int txr = tx < RW - 1 ? tx + 1 : RW - 1;
    const bool edge_cta = gy0 <= 0 || gy0 + RH - 1 >= rows - 1 || gx0 <= 0 || gx0 + RW - 1 >= cols - 1;

    // direct loads: a region starting on a multiple of four columns, 16-byte rows and buffers
    const bool aligned16 =
        (MODE & kModeDirect) && F.sweeps > 0 && (kind != PASS_PRESSURE_FIRST || (MODE & kModeDiv)) &&
        (((gx0 | F.pitch) & 3) == 0) &&
        ((reinterpret_cast<uintptr_t>(xin) | reinterpret_cast<uintptr_t>(F.x2) | reinterpret_cast<uintptr_t>(F.cst) |
          reinterpret_cast<uintptr_t>(yout) | reinterpret_cast<uintptr_t>(F.cst_out) |
          reinterpret_cast<uintptr_t>(F.u_in) | reinterpret_cast<uintptr_t>(F.v_in) |
          reinterpret_cast<uintptr_t>(F.u_out) | reinterpret_cast<uintptr_t>(F.v_out)) & 15) == 0;
    const bool first = kind == PASS_DIFFUSE_FIRST;
    const bool divp = kind == PASS_PRESSURE_FIRST;
    if (aligned16 && !edge_cta && (!resid || (MODE & kModeResid)) && ((MODE & kModeGrad) || !F.epilogue)) {
        SweepParams P = {F.sweeps,
                         kSwLoad | kSwDirect | (first ? kSwFirst : 0) | (divp ? kSwDiv : 0) | (resid ? kSwResid : 0),
                         gy0, gx0, rows, cols, F.s_lr, F.s_tb, F.a, F.dh, F.dl, F.rf};
        P.x = xin;
        P.k = first ? F.x2 : F.cst;
        P.y = yout;
        P.kout = (first || divp) ? F.cst_out : nullptr;
        P.pitch = F.pitch;
        P.halo = H;
        P.halo_l = HL;
        P.tile_h = F.tile_h;
        P.tile_w = F.tile_w;
        P.dt = F.dt;
        P.F = (!DIFF && (F.epilogue || divp)) ? &F : nullptr;
        sweep_phase<DIFF, NW, MODE>(0, RH * RW, P);
        if ((MODE & kModeResid) && resid) {
            const float2 r = *reinterpret_cast<const float2*>(
                S + resid_slot<NW>(0, F.sweeps, threadIdx.y * RW + threadIdx.x));
            rnum += r.x;
            rden += r.y;
        }
        return;
    }

    // kidx(r0 + i, tx) split into a per-thread base and a compile-time row offset (r0 is a
    // multiple of 8)
    const int kbase = no + kidx(r0, tx);
#define KREF(i) (S[kbase + ((i) >> 3) * (8 * RW) + ((i) & 3) * (2 * RW) + (((i) >> 2) & 1)])
#define XREF(i) (S[co + (r0 + (i)) * RW + tx])

    // Row masks of this thread's column segment (bit i = row r0 + i of the region),
    // computed once so that the unrolled row loops below test one bit per row:
    //   m_in  - the cell lies in the grid (loads);
    //   m_int - the cell is an interior cell (constant terms, add_sources, live cells);
    //   m_out - the cell is in this tile's output and in the grid (stores).
    const int g0 = gy0 + r0;  // grid row of bit 0
    auto range = [](int lo, int hi) -> unsigned {
        lo = max(lo, 0);
        hi = min(hi, SR);
        return hi > lo ? (((hi - lo) >= 32 ? ~0u : ((1u << (hi - lo)) - 1u)) << lo) : 0u;
    };
    const unsigned m_in = col_in ? range(-g0, rows - g0) : 0u;
    const unsigned m_int = col_int ? range(1 - g0, rows - 1 - g0) : 0u;
    const size_t o0 = (size_t)((long long)g0 * (long long)pitch + gc);  // offset of bit 0 (wraps if g0 < 0;
                                                                         // only masked rows are dereferenced)

    // ------------------------------------------------------------------ load
    // The field goes to S + co and its constant term to S + no, row by row.
    {
        if (kind == PASS_PRESSURE_FIRST) {
            // divergence_kernel (fluid_solver_gpu.cu:173-174) on the region, from u, v
            // staged in the two shared buffers.
#pragma unroll
            for (int i = 0; i < SR; ++i) {
                const bool in = (m_in >> i) & 1u;
                const size_t o = o0 + (size_t)i * pitch;
                S[co + (r0 + i) * RW + tx] = in ? __ldcg(xin + o) : 0.f;
                S[no + (r0 + i) * RW + tx] = in ? __ldcg(F.x2 + o) : 0.f;
            }
            __syncthreads();
            const float cdiv = F.cdiv;
            float kc[SR];
#pragma unroll
            for (int i = 0; i < SR; ++i) {
                const int r = r0 + i;
                const int ru = r > 0 ? r - 1 : 0, rd = r < RH - 1 ? r + 1 : RH - 1;
                float s = __fsub_rn(S[co + r * RW + txr], S[co + r * RW + txl]);
                s = __fadd_rn(s, S[no + rd * RW + tx]);
                s = __fsub_rn(s, S[no + ru * RW + tx]);
                kc[i] = ((m_int >> i) & 1u) ? __fmul_rn(cdiv, s) : 0.f;
            }
            __syncthreads();
            const float* __restrict__ cst = F.cst;  // starting pressure (null = zero)
#pragma unroll
            for (int i = 0; i < SR; ++i) {
                S[co + (r0 + i) * RW + tx] =
                    (cst != nullptr && ((m_in >> i) & 1u)) ? __ldcg(cst + o0 + (size_t)i * pitch) : 0.f;
                KREF(i) = kc[i];
            }
        } else if (kind == PASS_DIFFUSE_FIRST) {
            // add_sources_kernel (fluid_solver_gpu.cu:64) fused into the load
            const float dt = F.dt;
#pragma unroll 8
            for (int i = 0; i < SR; ++i) {
                const size_t o = o0 + (size_t)i * pitch;
                float x = ((m_in >> i) & 1u) ? __ldcg(xin + o) : 0.f;
                if ((m_int >> i) & 1u) x = __fmaf_rn(dt, __ldcg(F.x2 + o), x);  // fused, as compiled
                S[co + (r0 + i) * RW + tx] = x;
                KREF(i) = x;
            }
        } else {
#pragma unroll 8
            for (int i = 0; i < SR; ++i) {
                const size_t o = o0 + (size_t)i * pitch;
                S[co + (r0 + i) * RW + tx] = ((m_in >> i) & 1u) ? __ldcg(xin + o) : 0.f;
                KREF(i) = ((m_int >> i) & 1u) ? __ldcg(F.cst + o) : 0.f;
            }
        }
        __syncthreads();
    }

    // ------------------------------------------------------------------ sweeps
    if (F.sweeps > 0) {
        SweepParams P = {F.sweeps, edge_cta ? kSwEdge : 0, gy0, gx0, rows, cols, F.s_lr, F.s_tb, F.a, F.dh, F.dl, F.rf};
        P.x = xin;
        P.k = first ? F.x2 : F.cst;
        P.pitch = F.pitch;
        P.dt = F.dt;
        sweep_phase<DIFF, NW, MODE>(co, no, P);
        if (edge_cta) {
            fill_edges<SR, RH>(co, r0, tx, txl, txr, g0, gc, rows, cols, F.s_lr, F.s_tb);
            // restore_corners: the reference never writes the four corners; the sweeps
            // computed values there that nothing read, so put the pass's input back
            if (gc == 0 || gc == cols - 1) {
                const float* src = kind == PASS_PRESSURE_FIRST ? F.cst : xin;
#pragma unroll
                for (int i = 0; i < SR; ++i) {
                    const int gr = g0 + i;
                    if (gr == 0 || gr == rows - 1)
                        XREF(i) = src ? __ldcg(src + o0 + (size_t)i * pitch) : 0.f;
                }
            }
            __syncthreads();
        }
    }
    // final values of this thread's column: XREF(i) (S + co is complete after the last barrier)

    // ------------------------------------------------------------------ store
    const bool col_out = col_in && tx >= HL && tx < HL + F.tile_w;
    const unsigned m_out = col_out ? (range(H - r0, H + F.tile_h - r0) & m_in) : 0u;
    if (m_out) {
        float* __restrict__ y = yout;
        float* __restrict__ ko = F.cst_out;
        if (y) {
#pragma unroll 8
            for (int i = 0; i < SR; ++i)
                if ((m_out >> i) & 1u) y[o0 + (size_t)i * pitch] = XREF(i);
        }
        if (ko) {
#pragma unroll 8
            for (int i = 0; i < SR; ++i)
                if ((m_out >> i) & 1u) ko[o0 + (size_t)i * pitch] = KREF(i);
        }
    }
    if (F.epilogue && col_out) {

        // ---------------------------------------------- gradient subtract epilogue
        // remove_p_kernel (fluid_solver_gpu.cu:202-203) then the reflecting fills
        // set_boundary_opposite_horizontal(u) / _vertical(v) (fluid_solver_gpu.cu:402-403).
        // Edge cells take the updated value of their inner neighbour (negated for the
        // normal component), corners keep their input value.
        const float h = F.h, rh = __frcp_rn(h);  // RN(1/h) for div_by
        int bad = 0;
        const unsigned m_out_rows = range(H - r0, H + F.tile_h - r0) & m_in;
        if (!edge_cta) {
            // every output cell of an interior tile is an interior cell: batches of eight
            // rows, the batch's u and v loads in flight together, then the arithmetic in
            // the reference's order
#pragma unroll 1
            for (int i0 = 0; i0 < SR; i0 += 8) {
                float uin[8], vin[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    uin[k] = vin[k] = 0.f;
                    if ((m_out_rows >> (i0 + k)) & 1u) {
                        uin[k] = __ldcg(F.u_in + o0 + (size_t)(i0 + k) * pitch);
                        vin[k] = __ldcg(F.v_in + o0 + (size_t)(i0 + k) * pitch);
                    }
                }
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    if (!((m_out_rows >> (i0 + k)) & 1u)) continue;
                    const int r = r0 + i0 + k;
                    const float gu =
                        div_by(__fmul_rn(0.5f, __fsub_rn(S[co + r * RW + tx + 1], S[co + r * RW + tx - 1])), h, rh);
                    const float gv = div_by(
                        __fmul_rn(0.5f, __fsub_rn(S[co + (r + 1) * RW + tx], S[co + (r - 1) * RW + tx])), h, rh);
                    const float un = __fsub_rn(uin[k], gu), vn = __fsub_rn(vin[k], gv);
                    const size_t o = o0 + (size_t)(i0 + k) * pitch;
                    F.u_out[o] = un;
                    F.v_out[o] = vn;
                    bad |= !(isfinite(un) && isfinite(vn));
                }
            }
        } else {
            // Edge tiles: rows go in batches of EB: first the cell each row reads u and v
            // from (its own, or its inner neighbour's on an edge) for the whole batch, so
            // the global loads are in flight together, then the arithmetic, in the
            // reference's order.
            constexpr int EB = 8;
#pragma unroll 1
            for (int i0 = 0; i0 < SR; i0 += EB) {
                float uin[EB], vin[EB];
                unsigned live_rows = 0;
#pragma unroll
                for (int k = 0; k < EB; ++k) {
                    const int r = r0 + i0 + k, gr = gy0 + r;
                    uin[k] = vin[k] = 0.f;
                    if (r < H || r >= H + F.tile_h || gr < 0 || gr >= rows) continue;
                    const bool row_int = gr >= 1 && gr <= rows - 2;
                    int ir = gr, ic = gc;
                    if (!(col_int && row_int)) {
                        if (row_int) ic = (gc == 0) ? 1 : cols - 2;       // left / right edge
                        else if (col_int) ir = (gr == 0) ? 1 : rows - 2;  // top / bottom edge
                    }
                    const size_t oi = (size_t)ir * pitch + ic;
                    uin[k] = __ldcg(F.u_in + oi);
                    vin[k] = __ldcg(F.v_in + oi);
                    live_rows |= 1u << k;
                }
#pragma unroll
                for (int k = 0; k < EB; ++k) {
                    if (!((live_rows >> k) & 1u)) continue;
                    const int r = r0 + i0 + k, gr = gy0 + r;
                    const bool row_int = gr >= 1 && gr <= rows - 2;
                    int ir = gr, ic = gc;
                    float su = 1.f, sv = 1.f;
                    bool corner = false;
                    if (col_int && row_int) {
                    } else if (row_int) {  // left / right edge
                        ic = (gc == 0) ? 1 : cols - 2;
                        su = -1.f;
                    } else if (col_int) {  // top / bottom edge
                        ir = (gr == 0) ? 1 : rows - 2;
                        sv = -1.f;
                    } else {
                        corner = true;
                    }
                    const size_t o = (size_t)gr * pitch + gc;
                    float un, vn;
                    if (corner) {
                        un = uin[k];
                        vn = vin[k];
                    } else {
                        const int rr = min(max(ir - gy0, 0), RH - 1), rc = min(max(ic - gx0, 0), RW - 1);
                        const int rcl = rc > 0 ? rc - 1 : 0, rcr = rc < RW - 1 ? rc + 1 : RW - 1;
                        const int rru = rr > 0 ? rr - 1 : 0, rrd = rr < RH - 1 ? rr + 1 : RH - 1;
                        const float gu =
                            div_by(__fmul_rn(0.5f, __fsub_rn(S[co + rr * RW + rcr], S[co + rr * RW + rcl])), h, rh);
                        const float gv =
                            div_by(__fmul_rn(0.5f, __fsub_rn(S[co + rrd * RW + rc], S[co + rru * RW + rc])), h, rh);
                        un = su * __fsub_rn(uin[k], gu);
                        vn = sv * __fsub_rn(vin[k], gv);
                    }
                    F.u_out[o] = un;
                    F.v_out[o] = vn;
                    bad |= !(isfinite(un) && isfinite(vn));
                }
            }
        }
        if (bad && F.nonfinite) atomicOr(F.nonfinite, 1);
    }

    // ------------------------------------------------ residual partial sums
    // ||div + sum(nbrs) - 4p||^2 and ||div||^2 over this tile's interior output
    // cells, from the final p (valid one ring beyond the tile: halo = sweeps + 1).
    if (resid && col_out) {
#pragma unroll 8
        for (int i = 0; i < SR; ++i) {
            const int r = r0 + i, gr = gy0 + r;
            if (r < H || r >= H + F.tile_h || !col_int || gr < 1 || gr > rows - 2) continue;
            const int ru = r > 0 ? r - 1 : 0, rd = r < RH - 1 ? r + 1 : RH - 1;
            float sres = KREF(i) + S[co + r * RW + txr];
            sres += S[co + r * RW + txl];
            sres += S[co + rd * RW + tx];
            sres += S[co + ru * RW + tx];
            const float res = sres - 4.f * XREF(i);
            rnum = fmaf(res, res, rnum);
            rden = fmaf(KREF(i), KREF(i), rden);
        }
    }
}

#undef KREF
#undef XREF

// Gradient subtract and reflecting fills as a separate pass, from a final pressure p whose
// edge cells are already filled: remove_p_kernel (fluid_solver_gpu.cu:202-203) on interior
// cells, then set_boundary_opposite_horizontal(u) / _vertical(v) (fluid_solver_gpu.cu:
// 402-403): an edge cell takes its inner neighbour's new value, negated for the normal
// component; corners keep their input value. The same operations, in the same order, as
// the fused epilogue of the last stencil pass, one cell per thread (a bandwidth-bound
// pass: p, u, v read, u, v written).
__device__ __forceinline__ void gradient_cell(const float* __restrict__ p, const float* __restrict__ u_in,
                                              const float* __restrict__ v_in, int i, int j, int rows, int cols,
                                              size_t pitch, float h, float rh, float& un, float& vn) {
    const bool ri = i >= 1 && i <= rows - 2, ci = j >= 1 && j <= cols - 2;
    const size_t o = (size_t)i * pitch + j;
    if (!ri && !ci) {
        un = __ldg(u_in + o);
        vn = __ldg(v_in + o);
        return;
    }
    int ii = i, jj = j;
    float su = 1.f, sv = 1.f;
    if (!ci) {  // left / right edge
        jj = (j == 0) ? 1 : cols - 2;
        su = -1.f;
    } else if (!ri) {  // top / bottom edge
        ii = (i == 0) ? 1 : rows - 2;
        sv = -1.f;
    }
    const size_t q = (size_t)ii * pitch + jj;
    const float gu = div_by(__fmul_rn(0.5f, __fsub_rn(__ldg(p + q + 1), __ldg(p + q - 1))), h, rh);
    const float gv = div_by(__fmul_rn(0.5f, __fsub_rn(__ldg(p + q + pitch), __ldg(p + q - pitch))), h, rh);
    un = su * __fsub_rn(__ldg(u_in + q), gu);
    vn = sv * __fsub_rn(__ldg(v_in + q), gv);
}

// Four consecutive cells (i, j0 .. j0 + 3) of the gradient subtract: an interior group
// with 16-byte loads and stores (p's row and its rows above and below, two more p values
// at the group's ends), a group touching an edge cell per cell. Requires the rows 16-byte
// aligned (pitch a multiple of four, buffers 16-byte aligned). Returns true when an
// output is NaN or Inf.
__device__ __forceinline__ bool gradient_group(const float* __restrict__ p, const float* __restrict__ u_in,
                                               const float* __restrict__ v_in, float* __restrict__ u_out,
                                               float* __restrict__ v_out, int i, int j0, int rows, int cols,
                                               size_t P, float h, float rh) {
    const size_t o = (size_t)i * P + j0;
    float un[4], vn[4];
    int n = 4;
    if (i >= 1 && i <= rows - 2 && j0 >= 1 && j0 + 3 <= cols - 2) {
        const float4 pc = __ldg(reinterpret_cast<const float4*>(p + o));
        const float4 pu = __ldg(reinterpret_cast<const float4*>(p + o - P));
        const float4 pd = __ldg(reinterpret_cast<const float4*>(p + o + P));
        const float4 u4 = __ldg(reinterpret_cast<const float4*>(u_in + o));
        const float4 v4 = __ldg(reinterpret_cast<const float4*>(v_in + o));
        const float pl0 = __ldg(p + o - 1), pr3 = __ldg(p + o + 4);
        const float pcv[6] = {pl0, pc.x, pc.y, pc.z, pc.w, pr3};
        const float puv[4] = {pu.x, pu.y, pu.z, pu.w}, pdv[4] = {pd.x, pd.y, pd.z, pd.w};
        const float uv[4] = {u4.x, u4.y, u4.z, u4.w}, vv[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float gu = div_by(__fmul_rn(0.5f, __fsub_rn(pcv[k + 2], pcv[k])), h, rh);
            const float gv = div_by(__fmul_rn(0.5f, __fsub_rn(pdv[k], puv[k])), h, rh);
            un[k] = __fsub_rn(uv[k], gu);
            vn[k] = __fsub_rn(vv[k], gv);
        }
        *reinterpret_cast<float4*>(u_out + o) = make_float4(un[0], un[1], un[2], un[3]);
        *reinterpret_cast<float4*>(v_out + o) = make_float4(vn[0], vn[1], vn[2], vn[3]);
    } else {
        n = min(4, cols - j0);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (k >= n) break;
            gradient_cell(p, u_in, v_in, i, j0 + k, rows, cols, P, h, rh, un[k], vn[k]);
            u_out[o + k] = un[k];
            v_out[o + k] = vn[k];
        }
    }
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k < n) bad |= !(isfinite(un[k]) && isfinite(vn[k]));
    return bad;
}

// One thread per four consecutive cells of a row (gradient_group).
__global__ void __launch_bounds__(256) gradient_kernel(const float* p0, const float* __restrict__ u_in,
                                                       const float* __restrict__ v_in, float* __restrict__ u_out,
                                                       float* __restrict__ v_out, int rows, int cols, int pitch,
                                                       float h, int* nonfinite, const float* p_alt, const int* sel) {
    const int j0 = 4 * (blockIdx.x * 32 + threadIdx.x), i = blockIdx.y * 8 + threadIdx.y;
    if (i >= rows || j0 >= cols) return;
    const float* __restrict__ p = (sel != nullptr && __ldcg(sel) != 0) ? p_alt : p0;
    const bool bad = gradient_group(p, u_in, v_in, u_out, v_out, i, j0, rows, cols, (size_t)pitch, h, __frcp_rn(h));
    if (bad && nonfinite) atomicOr(nonfinite, 1);
}

// Batched form: blocks of 32 x 8 threads over 128 columns x kGradBatchRows rows of one
// grid (gradient_batch_blocks per grid), numbered grid by grid (prefix[g] = first block of
// grid g, block_job[b] = grid of block b); each thread takes four cells of a row, as
// gradient_kernel, in kGradBatchRows / 8 rows.
constexpr int kGradBatchRows = 32;
__global__ void __launch_bounds__(256) gradient_batch_kernel(const AdvectJob* __restrict__ jobs,
                                                             const int* __restrict__ prefix,
                                                             const int* __restrict__ block_job, int* nonfinite) {
    const int b = blockIdx.x;
    const int g = __ldg(block_job + b);
    const AdvectJob& J = jobs[g];
    const int lb = b - __ldg(prefix + g);
    const int rows = J.A.rows, cols = J.A.cols;
    const int bx = ((cols + 3) / 4 + 31) / 32;
    const int j0 = 4 * ((lb % bx) * 32 + threadIdx.x);
    const float h = J.A.h, rh = __frcp_rn(h);
    bool bad = false;
#pragma unroll
    for (int r = 0; r < kGradBatchRows; r += 8) {
        const int i = (lb / bx) * kGradBatchRows + r + threadIdx.y;
        if (i >= rows || j0 >= cols) continue;
        bad |= gradient_group(J.in0, J.in1, J.in2, J.out0, J.out1, i, j0, rows, cols, (size_t)J.A.pitch, h, rh);
    }
    if (bad && nonfinite) atomicOr(nonfinite, 1);
}

// One launch = one pass over the tiles of up to kMaxStencilFields fields.
template <int TY, int SRB, bool DIFF>
__global__ void __launch_bounds__(kRegionW* TY, (TY <= 2 ? 2 : 1))
    stencil_kernel(const __grid_constant__ StencilLaunch L) {
        extern __shared__ float4 smem4[];
    int b = blockIdx.x, f = 0;
#pragma unroll 1
    while (f + 1 < L.nfields && b >= L.f[f + 1].tile_begin) ++f;
    const StencilField& F = L.f[f];
    float rn = 0.f, rd = 0.f;
    process_tile<TY, SRB, DIFF, kModeDirect | kModeGrad | kModeDiv>(F, b - F.tile_begin, F.x, F.y, false, rn, rd);
}

// One pass over the fields of a batch of grids of uneven size, up to kMaxWideFields
// of them, with their descriptors in the launch's parameters like the single-grid
// kernel's: one CTA per tile of the concatenated tile list, the tile's field found by a
// binary search of the fields' first tiles. No global load precedes the tile's own.
// (The previous form, a device-resident descriptor table that each CTA fetched into
// shared memory, with masked direct loads for edge tiles, made the batch's pressure
// passes 20-55 % slower than the same grid's single-grid passes.)
template <int TY, int SRB, bool DIFF>
__global__ void __launch_bounds__(kRegionW* TY, (TY <= 2 ? 2 : 1))
    stencil_wide_kernel(const __grid_constant__ WideLaunch L) {
    const int b = blockIdx.x;
    int lo = 0, hi = L.nfields - 1;
#pragma unroll 1
    while (lo < hi) {  // the last field whose first tile is <= b
        const int mid = (lo + hi + 1) >> 1;
        if (L.begin[mid] <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    const StencilField& F = L.f[lo];
    float rn = 0.f, rd = 0.f;
    process_tile<TY, SRB, DIFF, kModeDirect | kModeGrad | kModeDiv>(F, b - L.begin[lo], F.x, F.y, false, rn, rd);
}

// ---------------------------------------------------------------------------
// Residual-driven pressure solve in one persistent cooperative launch.

constexpr unsigned kBarrierSpinLimit = 1u << 24;  // default: ~2 s of polling, then give up

// Grid-wide barrier for a cooperative launch (all CTAs co-resident). The wait is
// bounded: after `limit` polls the CTA sets ctrl->error and continues, and every later
// barrier returns at once, so the kernel always terminates. Returns false once an error
// has been flagged.
__device__ __forceinline__ bool grid_barrier(SolveCtrl* ctrl, unsigned nblocks, unsigned limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
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

// Fixed-order block sum of two doubles (shuffle tree, then warps in order); every
// thread receives the result.
__device__ __forceinline__ void block_sum2(double& a, double& b) {
    __shared__ double sa[32], sb[32];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nw = (blockDim.x * blockDim.y + 31) / 32;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    __syncthreads();
    if ((tid & 31) == 0) {
        sa[tid >> 5] = a;
        sb[tid >> 5] = b;
    }
    __syncthreads();
    if (tid == 0) {
        double x = 0, y = 0;
        for (int w = 0; w < nw; ++w) {
            x += sa[w];
            y += sb[w];
        }
        sa[0] = x;
        sb[0] = y;
    }
    __syncthreads();
    a = sa[0];
    b = sb[0];
}

// Out-of-line tile call for the persistent kernel: keeps the pass loop's state out
// of the tile body's register budget.
template <int TY, int SRB>
__device__ __noinline__ void pressure_tile(const StencilField& F, int t, const float* x, float* y, bool resid,
                                           float& rn, float& rd) {
    // direct tiles with the residual sums in registers; the final gradient pass (zero
    // sweeps) stays staged
    process_tile<TY, SRB, false, kModeDirect | kModeResid>(F, t, x, y, resid, rn, rd);
}

template <int TY, int SRB>
__global__ void __launch_bounds__(kRegionW* TY, (TY <= 2 ? 2 : 1))
    pressure_solve_kernel(const __grid_constant__ PressureSolve P) {
    const unsigned G = gridDim.x;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    const int ntiles = P.mid.tiles_x * P.mid.tiles_y;
    int passes = 0;
    double ratio = 0.0;
    bool ok = true, done = false;
    int cur = -1;  // index in P.p of the latest pressure; -1 before the first pass
    // segment mode, converged in an earlier segment: the flag was written by an earlier
    // launch, so every CTA reads the same value and none waits at a barrier
    if (P.segment && __ldcg(&P.ctrl->converged)) return;
    const unsigned lim_set = P.poll_limit ? __ldcg(P.poll_limit) : 0u;
    const unsigned limit = lim_set ? lim_set : kBarrierSpinLimit;
    int pass = 0;
#pragma unroll 1
    for (; ok && !done && pass < P.max_passes; ++pass) {
        const StencilField& F = cur < 0 ? P.first : P.mid;
        const float* x = cur < 0 ? F.x : P.p[cur];
        const int dst = cur < 0 ? 0 : cur ^ 1;
        // the residual is formed and tested every second pass (and on the last one allowed):
        // a pass without it skips the residual sums and the reduction, and a solve runs at
        // most one pass beyond the one that met the target
        const bool check = (pass & 1) || pass + 1 >= P.max_passes;
        float rn = 0.f, rd = 0.f;
#pragma unroll 1
        for (int t = blockIdx.x; t < ntiles; t += G)
            pressure_tile<TY, SRB>(F, t, x, P.p[dst], check, rn, rd);
        double a = rn, b = rd;
        double* part = P.partials + (size_t)(pass & 1) * 2 * G;
        if (check) {
            block_sum2(a, b);
            if (tid == 0) {
                part[2 * blockIdx.x] = a;
                part[2 * blockIdx.x + 1] = b;
            }
        }
        ok = grid_barrier(P.ctrl, G, limit);
        passes++;
        cur = dst;
        if (!ok) break;
        if (!check) continue;
        // every CTA sums all partials in the same order, so all agree on the outcome
        a = 0.0;
        b = 0.0;
        for (unsigned i = tid; i < G; i += nt) {
            a += __ldcg(part + 2 * i);
            b += __ldcg(part + 2 * i + 1);
        }
        block_sum2(a, b);
        ratio = b > 0.0 ? sqrt(a / b) : sqrt(a);
        done = ratio <= (double)P.tol;
    }
    if (ok && cur >= 0) {
        if (P.segment) {
            // every CTA passed the last pass's barrier: the final pressure is complete
            const float4* src = reinterpret_cast<const float4*>(P.p[cur]);
            float4* dst = reinterpret_cast<float4*>(P.p_cur);
            const long n4 = (long)P.mid.rows * P.mid.pitch / 4;
            for (long e = (long)blockIdx.x * nt + tid; e < n4; e += (long)G * nt) dst[e] = __ldcg(src + e);
        } else {
            // the final pressure: which buffer holds it (the gradient pass that follows
            // reads it there), and a copy for the next step's warm start
            if (blockIdx.x == 0 && tid == 0) P.ctrl->cur = cur;
            if (P.p_out) {
                const float4* src = reinterpret_cast<const float4*>(P.p[cur]);
                float4* dst = reinterpret_cast<float4*>(P.p_out);
                const long n4 = (long)P.mid.rows * P.mid.pitch / 4;
                for (long e = (long)blockIdx.x * nt + tid; e < n4; e += (long)G * nt) dst[e] = __ldcg(src + e);
            }
        }
    }
    if (blockIdx.x == 0 && tid == 0) {
        P.ctrl->passes = (P.segment ? P.ctrl->passes : 0) + passes;
        P.ctrl->residual = ratio;
        P.ctrl->converged = ok && ratio <= (double)P.tol;
    }
}

template <int TY, int SRB>
constexpr size_t smem_bytes() {
    return 2ull * (4 * TY * SRB) * kRegionW * sizeof(float);  // field + constant term
}

template <int TY, int SRB>
cudaError_t prepare_variant() {
    const int smem = (int)smem_bytes<TY, SRB>();
    cudaError_t e = cudaFuncSetAttribute(stencil_kernel<TY, SRB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(stencil_kernel<TY, SRB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(pressure_solve_kernel<TY, SRB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(stencil_wide_kernel<TY, SRB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(stencil_wide_kernel<TY, SRB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem);
    return e;
}

template <int TY, int SRB>
cudaError_t launch_wide_variant(const WideLaunch& L, bool diffuse, cudaStream_t st) {
    if (L.nfields <= 0 || L.nfields > kMaxWideFields) return cudaErrorInvalidValue;
    const int total = L.begin[L.nfields];
    if (total <= 0) return cudaSuccess;
    if (diffuse)
        stencil_wide_kernel<TY, SRB, true><<<total, dim3(kRegionW, TY), smem_bytes<TY, SRB>(), st>>>(L);
    else
        stencil_wide_kernel<TY, SRB, false><<<total, dim3(kRegionW, TY), smem_bytes<TY, SRB>(), st>>>(L);
    return cudaGetLastError();
}

template <int TY, int SRB>
cudaError_t solve_blocks(int* blocks) {
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pressure_solve_kernel<TY, SRB>, kRegionW * TY,
                                                          smem_bytes<TY, SRB>());
    *blocks = per * sms;
    return e;
}

template <int TY, int SRB>
cudaError_t launch_solve_variant(const PressureSolve& P, int blocks, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kRegionW, TY);
    cfg.dynamicSmemBytes = smem_bytes<TY, SRB>();
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, pressure_solve_kernel<TY, SRB>, P);
}

template <int TY, int SRB>
cudaError_t launch_variant(const StencilLaunch& L, cudaStream_t st) {
    const size_t smem = smem_bytes<TY, SRB>();
    int blocks = 0;
    for (int i = 0; i < L.nfields; ++i) blocks += L.f[i].tiles_x * L.f[i].tiles_y;
    if (blocks == 0) return cudaSuccess;
    // all fields of one launch are of the same class (diffusion or pressure)
    const bool diff = L.f[0].kind == PASS_DIFFUSE_FIRST || L.f[0].kind == PASS_DIFFUSE;
    if (diff)
        stencil_kernel<TY, SRB, true><<<blocks, dim3(kRegionW, TY), smem, st>>>(L);
    else
        stencil_kernel<TY, SRB, false><<<blocks, dim3(kRegionW, TY), smem, st>>>(L);
    return cudaGetLastError();
}

}  // namespace

int stencil_max_halo(int tile_rows) { return tile_rows / 2 - 2; }

// Opt the kernels into more than 48 KB of dynamic shared memory on the current
// device. Called once per handle at creation, outside any stream capture.
cudaError_t stencil_prepare() {
    cudaError_t e = prepare_variant<2, 8>();
    if (e == cudaSuccess) e = prepare_variant<4, 8>();
    return e;
}

cudaError_t launch_gradient(const float* p, const float* u_in, const float* v_in, float* u_out, float* v_out, int rows,
                            int cols, int pitch, float h, int* nonfinite, cudaStream_t st, const float* p_alt,
                            const int* sel) {
    if (pitch % 4 != 0 || ((reinterpret_cast<uintptr_t>(p) | reinterpret_cast<uintptr_t>(p_alt) |
                            reinterpret_cast<uintptr_t>(u_in) | reinterpret_cast<uintptr_t>(v_in) |
                            reinterpret_cast<uintptr_t>(u_out) | reinterpret_cast<uintptr_t>(v_out)) & 15) != 0)
        return cudaErrorInvalidValue;  // the handles' fields are 128-byte aligned rows
    const dim3 grid(((cols + 3) / 4 + 31) / 32, (rows + 7) / 8);
    gradient_kernel<<<grid, dim3(32, 8), 0, st>>>(p, u_in, v_in, u_out, v_out, rows, cols, pitch, h, nonfinite, p_alt,
                                                  sel);
    return cudaGetLastError();
}

int gradient_batch_blocks(int rows, int cols) {
    return (((cols + 3) / 4 + 31) / 32) * ((rows + kGradBatchRows - 1) / kGradBatchRows);
}

cudaError_t launch_gradient_batch(const AdvectJob* jobs, const int* prefix, const int* block_job, int nblocks,
                                  int* nonfinite, cudaStream_t st) {
    if (nblocks <= 0) return cudaSuccess;
    gradient_batch_kernel<<<nblocks, dim3(32, 8), 0, st>>>(jobs, prefix, block_job, nonfinite);
    return cudaGetLastError();
}

cudaError_t launch_stencil(const StencilLaunch& L, int tile_rows, cudaStream_t st) {
    if (tile_rows == 128) return launch_variant<4, 8>(L, st);
    return launch_variant<2, 8>(L, st);
}

cudaError_t pressure_solve_max_blocks(int tile_rows, int* blocks) {
    if (tile_rows == 128) return solve_blocks<4, 8>(blocks);
    return solve_blocks<2, 8>(blocks);
}

cudaError_t launch_pressure_solve(const PressureSolve& P, int tile_rows, int blocks, cudaStream_t st) {
    if (blocks <= 0) return cudaErrorInvalidValue;
    if (tile_rows == 128) return launch_solve_variant<4, 8>(P, blocks, st);
    return launch_solve_variant<2, 8>(P, blocks, st);
}

cudaError_t launch_stencil_wide(const WideLaunch& L, bool diffuse, int tile_rows, cudaStream_t st) {
    if (tile_rows == 128) return launch_wide_variant<4, 8>(L, diffuse, st);
    return launch_wide_variant<2, 8>(L, diffuse, st);
}

}  // namespace fs
