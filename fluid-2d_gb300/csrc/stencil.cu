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
// boundary fill applied after every sweep exactly as the reference does, and writes
// only its output tile back. The first pass of a solve fuses what precedes it
// (add_sources for diffusion, the divergence for pressure) and the last pressure
// pass fuses the gradient subtract and the two reflecting fills.
//
// Each thread owns one column of SR consecutive rows and keeps its current values
// and its constant term (x0 or div) in registers; neighbours come from the shared
// copy of the previous sweep (double-buffered, one barrier per sweep, a second one
// only in CTAs whose region touches a domain edge). All arithmetic uses explicit
// round-to-nearest intrinsics in the reference's operand order, so no FMA
// contraction changes its rounding. The reference divides by (1.0 + 4.0*a) in
// double; FP64 is slow on GB300, so the quotient is formed as
//   q = num*rf;  e = fma(-q, dh, num);  e = fma(-q, dl, e);  q = fma(e, rf, q)
// with dh + dl = 1 + 4a split into two floats and rf = (float)(1/(1 + 4a)). This
// Newton-corrected quotient agrees with (float)((double)num / (1.0 + 4.0*a)) except
// where the reference's double rounding lands exactly on a float tie (about one
// value in 10^8 in random testing).

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

template <int TY, int SR>
__global__ void __launch_bounds__(kRegionW* TY, (TY <= 4 ? 2 : 1))
    stencil_kernel(const __grid_constant__ StencilLaunch L) {
    constexpr int RW = kRegionW, RH = TY * SR;
    extern __shared__ float4 smem4[];
    float* cur = reinterpret_cast<float*>(smem4);
    float* nxt = cur + RH * RW;

    int b = blockIdx.x, f = 0;
#pragma unroll 1
    while (f + 1 < L.nfields && b >= L.f[f + 1].tile_begin) ++f;
    const StencilField& F = L.f[f];
    b -= F.tile_begin;
    const int tyi = b / F.tiles_x, txi = b - tyi * F.tiles_x;
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

    float c[SR], k[SR];

    // ------------------------------------------------------------------ load
    if (kind == PASS_PRESSURE_FIRST) {
        // divergence_kernel (fluid_solver_gpu.cu:173-174) on the region, from u, v
        // staged in the two shared buffers.
#pragma unroll
        for (int i = 0; i < SR; ++i) {
            const int gr = gy0 + r0 + i;
            const bool in = col_in && gr >= 0 && gr < rows;
            const size_t o = (size_t)gr * pitch + gc;
            cur[(r0 + i) * RW + tx] = in ? __ldg(F.x + o) : 0.f;
            nxt[(r0 + i) * RW + tx] = in ? __ldg(F.x2 + o) : 0.f;
        }
        __syncthreads();
        const float cdiv = F.cdiv;
#pragma unroll
        for (int i = 0; i < SR; ++i) {
            const int r = r0 + i, gr = gy0 + r;
            const int ru = r > 0 ? r - 1 : 0, rd = r < RH - 1 ? r + 1 : RH - 1;
            float s = __fsub_rn(cur[r * RW + txr], cur[r * RW + txl]);
            s = __fadd_rn(s, nxt[rd * RW + tx]);
            s = __fsub_rn(s, nxt[ru * RW + tx]);
            const bool interior = col_int && gr >= 1 && gr <= rows - 2;
            k[i] = interior ? __fmul_rn(cdiv, s) : 0.f;
            const bool in = col_in && gr >= 0 && gr < rows;
            c[i] = (F.cst != nullptr && in) ? __ldg(F.cst + (size_t)gr * pitch + gc) : 0.f;
        }
        __syncthreads();
    } else if (kind == PASS_DIFFUSE_FIRST) {
        // add_sources_kernel (fluid_solver_gpu.cu:64) fused into the load
        const float dt = F.dt;
#pragma unroll
        for (int i = 0; i < SR; ++i) {
            const int gr = gy0 + r0 + i;
            const bool in = col_in && gr >= 0 && gr < rows;
            const bool interior = col_int && gr >= 1 && gr <= rows - 2;
            const size_t o = (size_t)gr * pitch + gc;
            float x = in ? __ldg(F.x + o) : 0.f;
            if (interior) x = __fadd_rn(x, __fmul_rn(dt, __ldg(F.x2 + o)));
            c[i] = x;
            k[i] = x;
        }
    } else {
#pragma unroll
        for (int i = 0; i < SR; ++i) {
            const int gr = gy0 + r0 + i;
            const bool in = col_in && gr >= 0 && gr < rows;
            const bool interior = col_int && gr >= 1 && gr <= rows - 2;
            const size_t o = (size_t)gr * pitch + gc;
            c[i] = in ? __ldg(F.x + o) : 0.f;
            k[i] = interior ? __ldg(F.cst + o) : 0.f;
        }
    }
#pragma unroll
    for (int i = 0; i < SR; ++i) cur[(r0 + i) * RW + tx] = c[i];
    __syncthreads();

    // ------------------------------------------------------------------ sweeps
    const bool diffuse = (kind == PASS_DIFFUSE_FIRST || kind == PASS_DIFFUSE);
    const float a = F.a, dh = F.dh, dl = F.dl, rf = F.rf;
    const float s_lr = F.s_lr, s_tb = F.s_tb;
    const bool edge_cta = gy0 <= 0 || gy0 + RH - 1 >= rows - 1 || gx0 <= 0 || gx0 + RW - 1 >= cols - 1;
    const int nsweeps = F.sweeps;
#pragma unroll 1
    for (int s = 0; s < nsweeps; ++s) {
        float up = (r0 > 0) ? cur[(r0 - 1) * RW + tx] : c[0];
#pragma unroll
        for (int i = 0; i < SR; ++i) {
            const int r = r0 + i, gr = gy0 + r;
            float down;
            if (i + 1 < SR)
                down = c[i + 1];
            else
                down = (r + 1 < RH) ? cur[(r + 1) * RW + tx] : c[i];
            const float Lv = cur[r * RW + txl], Rv = cur[r * RW + txr];
            const float old = c[i];
            const bool interior = col_int && gr >= 1 && gr <= rows - 2;
            float nv = old;
            if (interior)
                nv = diffuse ? diffuse_update(k[i], Lv, Rv, up, down, a, dh, dl, rf)
                             : pressure_update(k[i], Lv, Rv, up, down);
            c[i] = nv;
            nxt[r * RW + tx] = nv;
            up = old;
        }
        __syncthreads();
        if (edge_cta) {
            // set_boundary_* (fluid_solver_gpu.cu:11-54): edges from the new inner
            // neighbour, corners untouched.
#pragma unroll
            for (int i = 0; i < SR; ++i) {
                const int r = r0 + i, gr = gy0 + r;
                float val;
                if (col_int) {
                    if (gr == 0)
                        val = s_tb * nxt[(r < RH - 1 ? r + 1 : r) * RW + tx];
                    else if (gr == rows - 1)
                        val = s_tb * nxt[(r > 0 ? r - 1 : r) * RW + tx];
                    else
                        continue;
                } else if (gr >= 1 && gr <= rows - 2) {
                    if (gc == 0)
                        val = s_lr * nxt[r * RW + txr];
                    else if (gc == cols - 1)
                        val = s_lr * nxt[r * RW + txl];
                    else
                        continue;
                } else {
                    continue;
                }
                c[i] = val;
                nxt[r * RW + tx] = val;
            }
            __syncthreads();
        }
        float* t = cur;
        cur = nxt;
        nxt = t;
    }

    // ------------------------------------------------------------------ store
    const bool col_out = col_in && tx >= H && tx < H + F.tile_w;
    if (col_out) {
#pragma unroll
        for (int i = 0; i < SR; ++i) {
            const int r = r0 + i, gr = gy0 + r;
            if (r < H || r >= H + F.tile_h || gr < 0 || gr >= rows) continue;
            const size_t o = (size_t)gr * pitch + gc;
            if (F.y) F.y[o] = c[i];
            if (F.cst_out) F.cst_out[o] = k[i];
        }
    }
    if (!F.epilogue || !col_out) return;

    // ---------------------------------------------- gradient subtract epilogue
    // remove_p_kernel (fluid_solver_gpu.cu:202-203) then the reflecting fills
    // set_boundary_opposite_horizontal(u) / _vertical(v) (fluid_solver_gpu.cu:402-403).
    // Edge cells take the updated value of their inner neighbour (negated for the
    // normal component), corners keep their input value.
    const float h = F.h;
    int bad = 0;
#pragma unroll
    for (int i = 0; i < SR; ++i) {
        const int r = r0 + i, gr = gy0 + r;
        if (r < H || r >= H + F.tile_h || gr < 0 || gr >= rows) continue;
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
            un = __ldg(F.u_in + o);
            vn = __ldg(F.v_in + o);
        } else {
            const int rr = min(max(ir - gy0, 0), RH - 1), rc = min(max(ic - gx0, 0), RW - 1);
            const int rcl = rc > 0 ? rc - 1 : 0, rcr = rc < RW - 1 ? rc + 1 : RW - 1;
            const int rru = rr > 0 ? rr - 1 : 0, rrd = rr < RH - 1 ? rr + 1 : RH - 1;
            const float gu = __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(cur[rr * RW + rcr], cur[rr * RW + rcl])), h);
            const float gv = __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(cur[rrd * RW + rc], cur[rru * RW + rc])), h);
            const size_t oi = (size_t)ir * pitch + ic;
            un = su * __fsub_rn(__ldg(F.u_in + oi), gu);
            vn = sv * __fsub_rn(__ldg(F.v_in + oi), gv);
        }
        F.u_out[o] = un;
        F.v_out[o] = vn;
        bad |= !(isfinite(un) && isfinite(vn));
    }
    if (bad && F.nonfinite) atomicOr(F.nonfinite, 1);
}

template <int TY, int SR>
constexpr size_t smem_bytes() {
    return 2ull * TY * SR * kRegionW * sizeof(float);
}

template <int TY, int SR>
cudaError_t prepare_variant() {
    return cudaFuncSetAttribute(stencil_kernel<TY, SR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_bytes<TY, SR>());
}

template <int TY, int SR>
cudaError_t launch_variant(const StencilLaunch& L, cudaStream_t st) {
    const size_t smem = smem_bytes<TY, SR>();
    int blocks = 0;
    for (int i = 0; i < L.nfields; ++i) blocks += L.f[i].tiles_x * L.f[i].tiles_y;
    if (blocks == 0) return cudaSuccess;
    stencil_kernel<TY, SR><<<blocks, dim3(kRegionW, TY), smem, st>>>(L);
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

}  // namespace fs
