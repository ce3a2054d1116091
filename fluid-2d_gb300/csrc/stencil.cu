// Temporally blocked 5-point Jacobi passes for diffusion and pressure.
//
// Reference behaviour (mworchel/fluid-2d src/fluid_solver_gpu.cu):
//   diffuse 290-312 + diffuse_iteration_kernel 69-85: per sweep, a D2D copy of the
//     field, one Jacobi kernel, a device sync, one boundary kernel, a device sync;
//   project 358-404 + kernels 164-206: clear div and p, divergence, Neumann fill,
//     Kp x (copy, Jacobi, fill), gradient subtract, two reflecting fills.
// That is ~20 B/cell of HBM traffic and two launches per sweep. Here one launch runs
// `sweeps` sweeps of one or more fields: each CTA loads a 128-column region (its
// output tile grown by a halo H >= sweeps), iterates in shared memory with the
// boundary fill's effect reproduced exactly after every sweep, and writes only its
// output tile back. The first pass of a solve fuses what precedes it
// (add_sources for diffusion, the divergence for pressure) and the last pressure
// pass fuses the gradient subtract and the two reflecting fills.
//
// Each thread owns one column of SR consecutive rows and keeps its constant terms
// (x0 or div) in registers; every sweep streams down the column from the shared copy
// of the previous sweep (double-buffered, one barrier per sweep) as two rolling
// windows in lockstep, so each pair of cell updates issues as packed f32x2
// instructions. The reference's per-sweep boundary fill is folded into the sweep (the
// cells next to a domain edge read what the fill would have stored there) and applied
// for real once, after the last sweep. All arithmetic uses
// explicit round-to-nearest intrinsics in the reference's operand order, so no FMA
// contraction changes its rounding (the one multiply feeding an add stays scalar). The reference divides by (1.0 + 4.0*a) in
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

__device__ __forceinline__ float diffuse_update(float x0, float L, float R, float U, float D, float a,
                                                float dh, float dl, float rf) {
    // (x0 + a*(L + R + U + D)) / (1 + 4a), fluid_solver_gpu.cu:81-82
    float s = __fadd_rn(L, R);
    s = __fadd_rn(s, U);
    s = __fadd_rn(s, D);
    const float num = __fadd_rn(x0, __fmul_rn(a, s));
    float q = __fmul_rn(num, rf);
    float e = __fmaf_rn(-q, dh, num);
    e = __fmaf_rn(-q, dl, e);
    return __fmaf_rn(e, rf, q);
}

__device__ __forceinline__ float pressure_update(float dv, float L, float R, float U, float D) {
    // (div + R + L + D + U) / 4, fluid_solver_gpu.cu:187-188
    float s = __fadd_rn(dv, R);
    s = __fadd_rn(s, L);
    s = __fadd_rn(s, D);
    s = __fadd_rn(s, U);
    return __fmul_rn(s, 0.25f);
}

// The same updates on two cells at once with the packed FP32 pipe (sm_100+): each lane
// of a float2 rounds exactly as the scalar form, so results are bit-identical; -q*dh is
// written q*(-dh), the same exact product.
__device__ __forceinline__ float2 diffuse_update2(float2 x0, float2 L, float2 R, float2 U, float2 D, float2 a,
                                                  float2 ndh, float2 ndl, float2 rf) {
    float2 s = __fadd2_rn(L, R);
    s = __fadd2_rn(s, U);
    s = __fadd2_rn(s, D);
    // x0 + a*s with two roundings, as the reference: formed lane by lane, because the
    // compiler may fuse a packed multiply feeding a packed add into one FFMA2
    const float2 num = make_float2(__fadd_rn(x0.x, __fmul_rn(a.x, s.x)), __fadd_rn(x0.y, __fmul_rn(a.y, s.y)));
    const float2 q = __fmul2_rn(num, rf);
    float2 e = __ffma2_rn(q, ndh, num);
    e = __ffma2_rn(q, ndl, e);
    return __ffma2_rn(e, rf, q);
}

__device__ __forceinline__ float2 pressure_update2(float2 dv, float2 L, float2 R, float2 U, float2 D) {
    float2 s = __fadd2_rn(dv, R);
    s = __fadd2_rn(s, L);
    s = __fadd2_rn(s, D);
    s = __fadd2_rn(s, U);
    return __fmul2_rn(s, make_float2(0.25f, 0.25f));
}

// All sweeps of one tile. Each thread owns one column of SR rows of the region and
// keeps only its constant term (x0 or div) in registers: every sweep streams down the
// column with a rolling up/centre/down window read from `cur` (the previous sweep) plus
// the left and right neighbours, and writes the new value to `nxt` — three shared loads
// and one store per cell update, and no per-row state carried across sweeps. One
// barrier per sweep.
//   EDGE = false: the region lies inside the domain interior; every cell updates, no
//                 checks (cells near the region border compute values that nothing
//                 stored depends on).
//   EDGE = true:  bit i of `live` marks interior cells (others keep their value). The
//                 reference fills the domain-edge cells after every sweep with their
//                 inner neighbour's new value times a sign (set_boundary_*,
//                 fluid_solver_gpu.cu:11-54), and the only cells that read an edge cell
//                 are those inner neighbours. So from the second sweep on, an interior
//                 cell next to an edge reads sign * (its own current value) in place of
//                 the edge cell — the same float the fill would have stored there — and
//                 the edge cells themselves are filled once, after the last sweep, by
//                 fill_edges. The first sweep reads the edge cells as loaded.
//                 up_bits / dn_bits: bit i set where row r0 + i is grid row 1 / rows - 2
//                 (its upper / lower neighbour is an edge cell); at_left / at_right: this
//                 column is grid column 1 / cols - 2.
template <bool DIFF, bool EDGE, int SR, int RH>
__device__ __forceinline__ void run_sweeps(const float2 (&k2)[SR / 2], int& co, int& no, int nsweeps, int r0,
                                           int tx, int txl, int txr, unsigned live, unsigned up_bits,
                                           unsigned dn_bits, bool at_left, bool at_right, float s_lr, float s_tb,
                                           float a, float dh, float dl, float rf) {
    constexpr int RW = kRegionW, H2 = SR / 2;
    extern __shared__ float4 smem4[];
    float* const S = reinterpret_cast<float*>(smem4);
    // offsets from this thread's first cell: the row above (clamped at the region top),
    // the row below the last (clamped at the bottom), the left and right neighbours
    // (clamped at the region sides); the clamped cells compute values nothing uses
    const int up_off = r0 > 0 ? -RW : 0;
    const int dn_off = (r0 + SR < RH) ? SR * RW : (SR - 1) * RW;
    const int l_off = txl - tx, r_off = txr - tx;
    const int base = r0 * RW + tx;
    const float2 a2 = make_float2(a, a), ndh2 = make_float2(-dh, -dh), ndl2 = make_float2(-dl, -dl);
    const float2 rf2 = make_float2(rf, rf);
#pragma unroll 1
    for (int s = 0; s < nsweeps; ++s) {
        const float* __restrict__ c = S + co + base;
        const float* __restrict__ cl = c + l_off;
        const float* __restrict__ cr = c + r_off;
        float* __restrict__ nx = S + no + base;
        // edge folding starts with the second sweep
        const unsigned ub = s > 0 ? up_bits : 0u, db = s > 0 ? dn_bits : 0u;
        const bool fl = s > 0 && at_left, fr = s > 0 && at_right;
        // two rolling windows down the segment in lockstep: rows j (x) and j + SR/2 (y)
        float2 up = make_float2(c[up_off], c[(H2 - 1) * RW]);
        float2 ce = make_float2(c[0], c[H2 * RW]);
#pragma unroll
        for (int j = 0; j < H2; ++j) {
            const float2 dn = make_float2(c[(j + 1) * RW], j + 1 + H2 < SR ? c[(j + 1 + H2) * RW] : c[dn_off]);
            float2 Lv = make_float2(cl[j * RW], cl[(j + H2) * RW]);
            float2 Rv = make_float2(cr[j * RW], cr[(j + H2) * RW]);
            float2 Dv = dn;
            if (EDGE) {
                if ((ub >> j) & 1u) up.x = __fmul_rn(s_tb, ce.x);
                if ((ub >> (j + H2)) & 1u) up.y = __fmul_rn(s_tb, ce.y);
                if ((db >> j) & 1u) Dv.x = __fmul_rn(s_tb, ce.x);
                if ((db >> (j + H2)) & 1u) Dv.y = __fmul_rn(s_tb, ce.y);
                if (fl) Lv = make_float2(__fmul_rn(s_lr, ce.x), __fmul_rn(s_lr, ce.y));
                if (fr) Rv = make_float2(__fmul_rn(s_lr, ce.x), __fmul_rn(s_lr, ce.y));
            }
            float2 nv = DIFF ? diffuse_update2(k2[j], Lv, Rv, up, Dv, a2, ndh2, ndl2, rf2)
                             : pressure_update2(k2[j], Lv, Rv, up, Dv);
            if (EDGE) {
                nv.x = ((live >> j) & 1u) ? nv.x : ce.x;
                nv.y = ((live >> (j + H2)) & 1u) ? nv.y : ce.y;
            }
            nx[j * RW] = nv.x;
            nx[(j + H2) * RW] = nv.y;
            up = ce;
            ce = dn;
        }
        __syncthreads();
        const int t = co;
        co = no;
        no = t;
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

// One tile of one pass: load the region (fusing add_sources or the divergence into
// the first pass), run F.sweeps sweeps (edge CTAs: with the boundary fill folded in and
// applied once at the end), store the
// output tile, then the optional gradient-subtract epilogue and the optional residual
// partial sums (for residual-driven pressure solves). xin/yout stand in for F.x/F.y so
// a persistent caller can ping-pong buffers across passes.
template <int TY, int SR, bool DIFF>
__device__ __forceinline__ void process_tile(const StencilField& F, int b, const float* __restrict__ xin,
                                             float* __restrict__ yout, bool resid,
                                             float& rnum, float& rden) {
    constexpr int RW = kRegionW, RH = TY * SR;
    extern __shared__ float4 smem4[];
    float* const S = reinterpret_cast<float*>(smem4);
    int co = 0, no = RH * RW;  // offsets of the current / next sweep buffers in S
    __syncthreads();  // the previous tile of this CTA may still be reading shared memory
    int tyi, txi;
    tile_coords(b, F.tiles_x, F.tiles_y, tyi, txi);
    const int H = F.halo;
    const int gy0 = tyi * F.tile_h - F.shift_y - H;
    const int gx0 = txi * F.tile_w - F.shift_x - H;
    const int rows = F.rows, cols = F.cols;
    const size_t pitch = (size_t)F.pitch;
    const int kind = F.kind;
    const int tx = threadIdx.x, r0 = threadIdx.y * SR;
    const int gc = gx0 + tx;
    const bool col_in = gc >= 0 && gc < cols;
    const bool col_int = gc >= 1 && gc <= cols - 2;
    const int txl = tx > 0 ? tx - 1 : 0;
    const int txr = tx < RW - 1 ? tx + 1 : RW - 1;

    float c[SR];
    float2 k2[SR / 2];  // constant terms: row i in k2[i].x (i < SR/2) or k2[i - SR/2].y
#define KREF(i) ((i) < SR / 2 ? k2[(i)].x : k2[(i) - SR / 2].y)

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
        const float* __restrict__ cst = F.cst;
#pragma unroll
        for (int i = 0; i < SR; ++i) {
            const int r = r0 + i;
            const int ru = r > 0 ? r - 1 : 0, rd = r < RH - 1 ? r + 1 : RH - 1;
            float s = __fsub_rn(S[co + r * RW + txr], S[co + r * RW + txl]);
            s = __fadd_rn(s, S[no + rd * RW + tx]);
            s = __fsub_rn(s, S[no + ru * RW + tx]);
            KREF(i) = ((m_int >> i) & 1u) ? __fmul_rn(cdiv, s) : 0.f;
            c[i] = (cst != nullptr && ((m_in >> i) & 1u)) ? __ldcg(cst + o0 + (size_t)i * pitch) : 0.f;
        }
        __syncthreads();
    } else if (kind == PASS_DIFFUSE_FIRST) {
        // add_sources_kernel (fluid_solver_gpu.cu:64) fused into the load
        const float dt = F.dt;
#pragma unroll
        for (int i = 0; i < SR; ++i) {
            const size_t o = o0 + (size_t)i * pitch;
            float x = ((m_in >> i) & 1u) ? __ldcg(xin + o) : 0.f;
            if ((m_int >> i) & 1u) x = __fadd_rn(x, __fmul_rn(dt, __ldcg(F.x2 + o)));
            c[i] = x;
            KREF(i) = x;
        }
    } else {
#pragma unroll
        for (int i = 0; i < SR; ++i) {
            const size_t o = o0 + (size_t)i * pitch;
            c[i] = ((m_in >> i) & 1u) ? __ldcg(xin + o) : 0.f;
            KREF(i) = ((m_int >> i) & 1u) ? __ldcg(F.cst + o) : 0.f;
        }
    }
#pragma unroll
    for (int i = 0; i < SR; ++i) S[co + (r0 + i) * RW + tx] = c[i];
    __syncthreads();

    // ------------------------------------------------------------------ sweeps
    const bool edge_cta = gy0 <= 0 || gy0 + RH - 1 >= rows - 1 || gx0 <= 0 || gx0 + RW - 1 >= cols - 1;
    if (edge_cta) {
        const int i1 = 1 - g0, i2 = rows - 2 - g0;  // segment rows of grid rows 1 and rows - 2
        const unsigned up_bits = (i1 >= 0 && i1 < SR) ? 1u << i1 : 0u;
        const unsigned dn_bits = (i2 >= 0 && i2 < SR) ? 1u << i2 : 0u;
        run_sweeps<DIFF, true, SR, RH>(k2, co, no, F.sweeps, r0, tx, txl, txr, m_int, up_bits, dn_bits, gc == 1,
                                       gc == cols - 2, F.s_lr, F.s_tb, F.a, F.dh, F.dl, F.rf);
        if (F.sweeps > 0) fill_edges<SR, RH>(co, r0, tx, txl, txr, g0, gc, rows, cols, F.s_lr, F.s_tb);
    } else {
        run_sweeps<DIFF, false, SR, RH>(k2, co, no, F.sweeps, r0, tx, txl, txr, 0u, 0u, 0u, false, false, F.s_lr,
                                        F.s_tb, F.a, F.dh, F.dl, F.rf);
    }
    // final values of this thread's column (S + co is complete after the last barrier)
#pragma unroll
    for (int i = 0; i < SR; ++i) c[i] = S[co + (r0 + i) * RW + tx];

    // ------------------------------------------------------------------ store
    const bool col_out = col_in && tx >= H && tx < H + F.tile_w;
    const unsigned m_out = col_out ? (range(H - r0, H + F.tile_h - r0) & m_in) : 0u;
    if (m_out) {
        float* __restrict__ y = yout;
        float* __restrict__ ko = F.cst_out;
        if (y) {
#pragma unroll
            for (int i = 0; i < SR; ++i)
                if ((m_out >> i) & 1u) y[o0 + (size_t)i * pitch] = c[i];
        }
        if (ko) {
#pragma unroll
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
        const float h = F.h;
        int bad = 0;
        // Rows go in batches of EB: first the cell each row reads u and v from (its own,
        // or its inner neighbour's on an edge) for the whole batch, so the global loads
        // are in flight together, then the arithmetic, in the reference's order.
        constexpr int EB = SR / 2;
    #pragma unroll
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
                        __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(S[co + rr * RW + rcr], S[co + rr * RW + rcl])), h);
                    const float gv =
                        __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(S[co + rrd * RW + rc], S[co + rru * RW + rc])), h);
                    un = su * __fsub_rn(uin[k], gu);
                    vn = sv * __fsub_rn(vin[k], gv);
                }
                F.u_out[o] = un;
                F.v_out[o] = vn;
                bad |= !(isfinite(un) && isfinite(vn));
            }
        }
        if (bad && F.nonfinite) atomicOr(F.nonfinite, 1);
    }

    // ------------------------------------------------ residual partial sums
    // ||div + sum(nbrs) - 4p||^2 and ||div||^2 over this tile's interior output
    // cells, from the final p (valid one ring beyond the tile: halo = sweeps + 1).
    if (resid && col_out) {
#pragma unroll
        for (int i = 0; i < SR; ++i) {
            const int r = r0 + i, gr = gy0 + r;
            if (r < H || r >= H + F.tile_h || !col_int || gr < 1 || gr > rows - 2) continue;
            const int ru = r > 0 ? r - 1 : 0, rd = r < RH - 1 ? r + 1 : RH - 1;
            float sres = KREF(i) + S[co + r * RW + txr];
            sres += S[co + r * RW + txl];
            sres += S[co + rd * RW + tx];
            sres += S[co + ru * RW + tx];
            const float res = sres - 4.f * c[i];
            rnum = fmaf(res, res, rnum);
            rden = fmaf(KREF(i), KREF(i), rden);
        }
    }
}

#undef KREF

// One launch = one pass over the tiles of up to kMaxStencilFields fields.
template <int TY, int SR, bool DIFF>
__global__ void __launch_bounds__(kRegionW* TY, (TY <= 4 ? 2 : 1))
    stencil_kernel(const __grid_constant__ StencilLaunch L) {
    constexpr int RH = TY * SR;
    extern __shared__ float4 smem4[];
    int b = blockIdx.x, f = 0;
#pragma unroll 1
    while (f + 1 < L.nfields && b >= L.f[f + 1].tile_begin) ++f;
    const StencilField& F = L.f[f];
    float rn = 0.f, rd = 0.f;
    process_tile<TY, SR, DIFF>(F, b - F.tile_begin, F.x, F.y, false, rn, rd);
}

// One pass over a device-resident table of fields (a batch of grids of uneven size):
// one CTA per tile of the concatenated tile list; tile_field[t] names the field of
// tile t and prefix[f] its first tile. The field's descriptor is staged in shared
// memory, where the tile body reads it many times.
template <int TY, int SR, bool DIFF>
__global__ void __launch_bounds__(kRegionW* TY, (TY <= 4 ? 2 : 1))
    stencil_table_kernel(const StencilField* __restrict__ tab, const int* __restrict__ prefix,
                         const int* __restrict__ tile_field) {
    __shared__ StencilField sF;
    static_assert(sizeof(StencilField) % 4 == 0, "descriptor copied as words");
    const int t = blockIdx.x;
    const int f = __ldg(tile_field + t);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if (tid < (int)(sizeof(StencilField) / 4))
        reinterpret_cast<int*>(&sF)[tid] = __ldg(reinterpret_cast<const int*>(tab + f) + tid);
    __syncthreads();
    float rn = 0.f, rd = 0.f;
    process_tile<TY, SR, DIFF>(sF, t - __ldg(prefix + f), sF.x, sF.y, false, rn, rd);
}

// ---------------------------------------------------------------------------
// Residual-driven pressure solve in one persistent cooperative launch.

constexpr unsigned kBarrierSpinLimit = 1u << 24;  // ~2 s of polling, then give up

// Grid-wide barrier for a cooperative launch (all CTAs co-resident). The wait is
// bounded: after kBarrierSpinLimit polls the CTA sets ctrl->error and continues, and
// every later barrier returns at once, so the kernel always terminates. Returns false
// once an error has been flagged.
__device__ __forceinline__ bool grid_barrier(SolveCtrl* ctrl, unsigned nblocks) {
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
                if (++spins > kBarrierSpinLimit) {
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
template <int TY, int SR>
__device__ __noinline__ void pressure_tile(const StencilField& F, int t, const float* x, float* y, bool resid,
                                           float& rn, float& rd) {
    process_tile<TY, SR, false>(F, t, x, y, resid, rn, rd);
}

template <int TY, int SR>
__global__ void __launch_bounds__(kRegionW* TY, (TY <= 4 ? 2 : 1))
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
    int pass = 0;
#pragma unroll 1
    for (; ok && !done && pass < P.max_passes; ++pass) {
        const StencilField& F = cur < 0 ? P.first : P.mid;
        const float* x = cur < 0 ? F.x : P.p[cur];
        const int dst = cur < 0 ? 0 : cur ^ 1;
        float rn = 0.f, rd = 0.f;
#pragma unroll 1
        for (int t = blockIdx.x; t < ntiles; t += G)
            pressure_tile<TY, SR>(F, t, x, P.p[dst], true, rn, rd);
        double a = rn, b = rd;
        block_sum2(a, b);
        double* part = P.partials + (size_t)(pass & 1) * 2 * G;
        if (tid == 0) {
            part[2 * blockIdx.x] = a;
            part[2 * blockIdx.x + 1] = b;
        }
        ok = grid_barrier(P.ctrl, G);
        passes++;
        cur = dst;
        if (!ok) break;
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
            // gradient subtract + reflecting fills from the final pressure
            const int nfin = P.fin.tiles_x * P.fin.tiles_y;
            float rn = 0.f, rd = 0.f;
#pragma unroll 1
            for (int t = blockIdx.x; t < nfin; t += G)
                pressure_tile<TY, SR>(P.fin, t, P.p[cur], P.p_out, false, rn, rd);
        }
    }
    if (blockIdx.x == 0 && tid == 0) {
        P.ctrl->passes = (P.segment ? P.ctrl->passes : 0) + passes;
        P.ctrl->residual = ratio;
        P.ctrl->converged = ok && ratio <= (double)P.tol;
    }
}

template <int TY, int SR>
constexpr size_t smem_bytes() {
    return 2ull * TY * SR * kRegionW * sizeof(float);
}

template <int TY, int SR>
cudaError_t prepare_variant() {
    const int smem = (int)smem_bytes<TY, SR>();
    cudaError_t e = cudaFuncSetAttribute(stencil_kernel<TY, SR, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(stencil_kernel<TY, SR, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(pressure_solve_kernel<TY, SR>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(stencil_table_kernel<TY, SR, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(stencil_table_kernel<TY, SR, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem);
    return e;
}

template <int TY, int SR>
cudaError_t launch_table_variant(const StencilField* tab, const int* prefix, const int* tile_field, int total,
                                 bool diffuse, cudaStream_t st) {
    if (total <= 0) return cudaSuccess;
    if (diffuse)
        stencil_table_kernel<TY, SR, true><<<total, dim3(kRegionW, TY), smem_bytes<TY, SR>(), st>>>(tab, prefix,
                                                                                                     tile_field);
    else
        stencil_table_kernel<TY, SR, false><<<total, dim3(kRegionW, TY), smem_bytes<TY, SR>(), st>>>(tab, prefix,
                                                                                                      tile_field);
    return cudaGetLastError();
}

template <int TY, int SR>
cudaError_t solve_blocks(int* blocks) {
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pressure_solve_kernel<TY, SR>, kRegionW * TY,
                                                          smem_bytes<TY, SR>());
    *blocks = per * sms;
    return e;
}

template <int TY, int SR>
cudaError_t launch_solve_variant(const PressureSolve& P, int blocks, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kRegionW, TY);
    cfg.dynamicSmemBytes = smem_bytes<TY, SR>();
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, pressure_solve_kernel<TY, SR>, P);
}

template <int TY, int SR>
cudaError_t launch_variant(const StencilLaunch& L, cudaStream_t st) {
    const size_t smem = smem_bytes<TY, SR>();
    int blocks = 0;
    for (int i = 0; i < L.nfields; ++i) blocks += L.f[i].tiles_x * L.f[i].tiles_y;
    if (blocks == 0) return cudaSuccess;
    // all fields of one launch are of the same class (diffusion or pressure)
    const bool diff = L.f[0].kind == PASS_DIFFUSE_FIRST || L.f[0].kind == PASS_DIFFUSE;
    if (diff)
        stencil_kernel<TY, SR, true><<<blocks, dim3(kRegionW, TY), smem, st>>>(L);
    else
        stencil_kernel<TY, SR, false><<<blocks, dim3(kRegionW, TY), smem, st>>>(L);
    return cudaGetLastError();
}

}  // namespace

int stencil_max_halo(int tile_rows) { return tile_rows / 2 - 2; }

// Opt the kernels into more than 48 KB of dynamic shared memory on the current
// device. Called once per handle at creation, outside any stream capture.
cudaError_t stencil_prepare() {
    cudaError_t e = prepare_variant<4, 16>();
    if (e == cudaSuccess) e = prepare_variant<8, 16>();
    return e;
}

cudaError_t launch_stencil(const StencilLaunch& L, int tile_rows, cudaStream_t st) {
    if (tile_rows == 128) return launch_variant<8, 16>(L, st);
    return launch_variant<4, 16>(L, st);
}

cudaError_t pressure_solve_max_blocks(int tile_rows, int* blocks) {
    if (tile_rows == 128) return solve_blocks<8, 16>(blocks);
    return solve_blocks<4, 16>(blocks);
}

cudaError_t launch_pressure_solve(const PressureSolve& P, int tile_rows, int blocks, cudaStream_t st) {
    if (blocks <= 0) return cudaErrorInvalidValue;
    if (tile_rows == 128) return launch_solve_variant<8, 16>(P, blocks, st);
    return launch_solve_variant<4, 16>(P, blocks, st);
}

cudaError_t launch_stencil_table(const StencilField* table, const int* prefix, const int* tile_field, int total_tiles,
                                 bool diffuse, int tile_rows, cudaStream_t st) {
    if (tile_rows == 128) return launch_table_variant<8, 16>(table, prefix, tile_field, total_tiles, diffuse, st);
    return launch_table_variant<4, 16>(table, prefix, tile_field, total_tiles, diffuse, st);
}

}  // namespace fs
