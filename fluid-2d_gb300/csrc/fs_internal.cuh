// Internal definitions shared by the solver's CUDA translation units.
//
// Storage: every field is a rows x pitch float32 slab in HBM, pitch a multiple of 32
// floats (128 B) so that each row starts on a 128-byte line; element (i, j) is at
// i*pitch + j. The reference stores the same fields unpadded (linear_buffer,
// src/linear_buffer.hpp:34-40: pitch = cols*4 B), which leaves most rows misaligned.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fs {

// Boundary modes of the reference (fluid_solver_gpu.cu:11-54). The sign pair gives
// the factor applied to the inner neighbour on the left/right edges and on the
// top/bottom edges; corners are never written.
enum Bnd : int { BND_CONT = 0, BND_OPP_H = 1, BND_OPP_V = 2 };
inline __host__ __device__ float bnd_sign_lr(int m) { return m == BND_OPP_H ? -1.f : 1.f; }
inline __host__ __device__ float bnd_sign_tb(int m) { return m == BND_OPP_V ? -1.f : 1.f; }

// Stencil pass kinds. A diffusion or pressure solve is split into passes; each pass
// loads a tile with a halo, runs `sweeps` Jacobi sweeps on chip (registers, with
// shuffles and a shared-memory row exchange) and writes the tile back once (temporal
// blocking).
enum PassKind : int {
    PASS_DIFFUSE_FIRST = 0,  // x0 = x + dt*s fused in (add_sources); writes x0
    PASS_DIFFUSE = 1,        // reads x, x0
    PASS_PRESSURE_FIRST = 2, // div computed from u, v and written; p starts at 0 (or p_init)
    PASS_PRESSURE = 3,       // reads p, div
};

// Region width of the stencil kernels: 128 columns, one per thread of a CTA row in the
// load and store phases, four per lane of a warp in the sweeps.
constexpr int kRegionW = 128;

struct StencilField {
    // inputs
    const float* x;     // state in: x (diffuse), p (pressure; may be null = zero start), u (pressure first)
    const float* x2;    // sources s (diffuse first) or v (pressure first)
    const float* cst;   // x0 (diffuse) or div (pressure) for non-first passes
    // outputs
    float* y;           // state out (x or p); may be null for a last pressure pass
    float* cst_out;     // first pass: x0 or div out
    // gradient-subtract epilogue (last pressure pass): u,v in -> out
    const float* u_in;
    const float* v_in;
    float* u_out;
    float* v_out;
    // constants
    float a, dh, dl, rf;  // diffuse: a and the FP32 pair for 1/(1+4a) (see stencil.cu)
    float dt;             // add_sources
    float cdiv;           // divergence factor -0.5f*h
    float h;              // gradient divisor
    float s_lr, s_tb;     // boundary signs of this field
    int kind;             // PassKind
    int sweeps;           // Jacobi sweeps in this pass
    int epilogue;         // 1: gradient subtract + velocity fills after the sweeps
    int halo;             // H: region = tile grown by H on each side
    int rows, cols, pitch;
    int tile_w, tile_h, tiles_x, tiles_y, shift_x, shift_y;
    int realign;          // 1: start each region on a multiple of four columns (see realign_columns)
    int tile_begin;       // first block index of this field in the launch
    int* nonfinite;       // optional flag (epilogue outputs)
};

constexpr int kMaxStencilFields = 4;
struct StencilLaunch {
    StencilField f[kMaxStencilFields];
    int nfields;
};

// Control block of one residual-driven pressure solve (device memory, cleared before
// each solve): grid-barrier state, the barrier-timeout flag, and the outcome.
struct SolveCtrl {
    unsigned bar_count;
    unsigned bar_gen;
    int error;      // 1: a grid barrier gave up waiting (FS_ERR_TIMEOUT)
    int passes;     // passes executed (each runs `sweeps` Jacobi sweeps)
    int converged;  // 1: relative residual <= tol
    int cur;        // index in PressureSolve::p of the final pressure (whole solves)
    double residual;  // relative residual after the last executed pass
};

// A whole pressure solve run to a residual target by one persistent cooperative
// launch: `first` (divergence fused) then `mid` passes until the relative residual
// drops to tol or max_passes ran. Passes ping-pong between p[0] and p[1]; the launch
// records which holds the final pressure (ctrl->cur), copies it to p_out when given, and
// the gradient subtract follows as launch_gradient with that selector.
//
// Segment mode (learned corrections): the divergence already exists, `first` is a
// PASS_PRESSURE field whose x is p_cur and `fin` is unused. The launch does nothing if
// ctrl->converged is already set; otherwise it runs passes from p_cur until the target
// or max_passes and copies the final pressure back to p_cur. ctrl->passes accumulates.
struct PressureSolve {
    StencilField first, mid;
    float* p[2];
    float* p_out;      // receives the final pressure (warm start); may be null
    double* partials;  // 4 doubles per CTA (residual sums, double-buffered by pass)
    SolveCtrl* ctrl;
    float tol;
    int max_passes;
    int segment;                    // 1: segment mode
    float* p_cur;                   // segment: start and final pressure
    const unsigned* poll_limit;     // device word: polls before a grid barrier gives up
                                    // (0 or null = the default, about 2 s)
};

// Semi-Lagrangian advection parameters.
struct AdvectArgs {
    int rows, cols, pitch;
    float dt0;          // sqrt(rows*cols)*dt (fluid_solver_gpu.cu:334)
    float xmax, ymax;   // cols-1.5f, rows-1.5f
    float h;            // gradient jobs: 1/sqrt(rows*cols) (fluid_solver_gpu.cu:367)
};

// One grid's work in a batched advection launch. Splat: in0 = d0, in1 = u, in2 = v,
// out0 = accumulator. Finish: in0 = accumulator, out0 = density. Velocity: in0 = u0,
// in1 = v0, out0 = u, out1 = v.
struct AdvectJob {
    AdvectArgs A;
    const float* in0;
    const float* in1;
    const float* in2;
    float* out0;
    float* out1;
    int smooth;
};

// Tile geometry: tiles partition [0, n) starting at -shift, and never put a domain
// edge cell (index 0 or n-1) in a different tile from its inner neighbour, so the
// boundary fill of a tile only ever depends on cells of the same tile.
inline void tile_split(int n, int tile, int* count, int* shift) {
    int s = ((n - 1) % tile == 0) ? 1 : 0;
    *shift = s;
    *count = (n + s + tile - 1) / tile;
}

// Column tiling for passes whose interior tiles can take the stencil's direct path,
// which loads and stores a region's rows 16 bytes at a time and so needs each region to
// start on a multiple of four columns. With tile width 128 - 2H and halo H that holds
// for every tile when the width is a multiple of four and H + shift is too. Otherwise
// the width shrinks by three and the kernel moves each region's start down to the
// multiple of four below it (by a = 0..3 columns): the left margin becomes H + a and the
// right one H + 3 - a, both at least H.
inline void realign_columns(StencilField& f) {
    f.realign = 0;
    const int w = kRegionW - 2 * f.halo;
    if (w % 4 == 0 && (f.halo + f.shift_x) % 4 == 0) return;
    if (w - 3 < 1) return;
    f.tile_w = w - 3;
    tile_split(f.cols, f.tile_w, &f.tiles_x, &f.shift_x);
    f.realign = 1;
}

// Sets the calling thread's fs_last_error() message and returns code (solver.cu).
int record_error(int code, const char* msg);

// Launchers (stencil.cu, advect.cu).
cudaError_t stencil_prepare();
cudaError_t launch_stencil(const StencilLaunch& L, int tile_rows, cudaStream_t st);
// remove_p and the reflecting fills of u and v from a final pressure p whose edges are
// filled (the last pass of a multi-pass projection stores it): u_out, v_out on every cell.
cudaError_t launch_gradient(const float* p, const float* u_in, const float* v_in, float* u_out, float* v_out, int rows,
                            int cols, int pitch, float h, int* nonfinite, cudaStream_t st,
                            const float* p_alt = nullptr, const int* sel = nullptr);  // p_alt when *sel != 0
// The same over a batch's grids in one launch (gradient_batch_blocks(rows, cols) blocks per
// grid, numbered as launch_advect_batch's; a job's in0 = p, in1 = u_in, in2 = v_in,
// out0 = u_out, out1 = v_out, A.h the grid spacing; rows 16-byte aligned).
int gradient_batch_blocks(int rows, int cols);
cudaError_t launch_gradient_batch(const AdvectJob* jobs, const int* prefix, const int* block_job, int nblocks,
                                  int* nonfinite, cudaStream_t st);
int stencil_max_halo(int tile_rows);
// Co-resident CTAs of the persistent pressure solve on the current device.
cudaError_t pressure_solve_max_blocks(int tile_rows, int* blocks);
cudaError_t launch_pressure_solve(const PressureSolve& P, int tile_rows, int blocks, cudaStream_t st);
cudaError_t launch_splat(const float* d0, const float* u, const float* v, float* acc, const AdvectArgs& A,
                         cudaStream_t st);
cudaError_t launch_density_finish(const float* acc, float* d, int smooth, const AdvectArgs& A, int* nonfinite,
                                  cudaStream_t st);
// Tensor-core conv set-up (shared-memory opt-in) on the current device (conv.cu).
cudaError_t conv_prepare();
// fs_conv3x3 with a skip flag: when skip_if (nullable) points at a non-zero value the
// launch does nothing (a converged pressure solve skips its remaining corrections).
int conv3x3_launch(const void* x, const void* wpk, const float* w32, const float* bias, const void* skip, void* y,
                   float* yf, int H, int W, int img_h, int up, int relu, int use_tensor_cores, int* err,
                   const int* skip_if, void* stream);
// The whole network on `images` 32 x 32 grids, one launch (fs_net_infer32), with the
// same skip flag.
int net_infer32_launch(const void* x0, const void* wpk, const float* params, void* e1, float* y, int images,
                       int* err, const int* skip_if, void* stream);

// Learned corrections (net.cu). Coarse residual: block sums of the residual of p (null =
// zero) into bs[G*G], their squared norm into *norm2 and, when xin is given, the network
// input and its scale. Coarse smoothing: nu weighted-Jacobi sweeps of the coarse
// equation 4e_I - sum(e_J) = bs_I (Neumann) from channel 0 of y_in (null = zero) into
// channel 0 of y_out. Energy gain: adds to *out how much closer p_try is to the solution
// than p_cur in the A-norm (2 c.r - c.Ac, c = p_try - p_cur). Accept: unless *converged,
// p_cur becomes pa or pb when its gain (gain[0], gain[1]) is the larger positive one;
// counters[0] counts pa chosen, counters[1] otherwise. Every launcher takes a nullable
// skip flag with the meaning of conv3x3_launch's.
cudaError_t launch_coarse_residual(const float* div, const float* p, int rows, int cols, int pitch, int G, float* bs,
                                   double* norm2, float* scale, void* xin, const int* skip_if, cudaStream_t st);
cudaError_t launch_coarse_smooth(const float* y_in, float* y_out, const float* bs, const float* scale, float kappa,
                                 int G, int nu, const int* skip_if, cudaStream_t st);
// Both candidates' smoothing in one launch (one CTA each, run side by side).
cudaError_t launch_coarse_smooth_pair(const float* y_in_a, float* y_out_a, const float* y_in_b, float* y_out_b,
                                      const float* bs, const float* scale, float kappa, int G, int nu,
                                      const int* skip_if, cudaStream_t st);
// The network input (channel 0 = bs / RMS(bs), scale, norm) from given block sums.
cudaError_t launch_coarse_input(const float* bs, int G, float* scale, void* xin, double* norm2, const int* skip_if,
                                cudaStream_t st);
// Block sums on G x G from those on 2G x 2G; a G x G correction (channel 0 times
// scale*kappa) interpolated onto 2G x 2G in absolute units (channel-0 stride 32).
cudaError_t launch_coarse_sum2x2(const float* fine, float* coarse, int G, const int* skip_if, cudaStream_t st);
cudaError_t launch_coarse_interp(const float* y, float* e, int G, const float* scale, float kappa,
                                 const int* skip_if, cudaStream_t st);
cudaError_t launch_prolong(const float* y, const float* p_prev, float* p_out, int rows, int cols, int pitch, int G,
                           const float* scale, float kappa, const int* skip_if, cudaStream_t st);
// One damped (weight 1/2) Jacobi step of p into out, Neumann-filled edges (net.cu).
cudaError_t launch_damp(const float* div, const float* p, float* out, int rows, int cols, int pitch,
                        const int* skip_if, cudaStream_t st);
cudaError_t launch_energy_gain(const float* div, const float* p_cur, const float* p_try, int rows, int cols,
                               int pitch, double* out, const int* skip_if, cudaStream_t st);
// Mixed-precision defect correction (net.cu): r = residual of p_hi + p_lo in FP64
// (stored FP32; sums[0] += ||r||^2, sums[1] += ||div||^2, zeroed before), and
// (p_hi, p_lo) += e with the sum split back into two floats.
cudaError_t launch_residual_df(const float* div, const float* p_hi, const float* p_lo, float* r, int rows, int cols,
                               int pitch, double* sums, cudaStream_t st);
cudaError_t launch_accumulate_df(float* p_hi, float* p_lo, const float* e, long n_floats, cudaStream_t st);
cudaError_t launch_accept_best(float* p_cur, const float* pa, const float* pb, long n_floats, const double* gain,
                               const int* converged, unsigned long long* counters, cudaStream_t st);

int advect_batch_blocks(int rows, int cols);
// op 0: splat, 1: density finish, 2: velocity backtrace; each block (32x8 threads)
// covers 32x32 cells; prefix[g] = first block of job g, block_job[b] = job of block b.
cudaError_t launch_advect_batch(int op, const AdvectJob* jobs, const int* prefix, const int* block_job, int nblocks,
                                int* nonfinite, cudaStream_t st);
// Stencil pass over many fields of one class (diffusion or pressure) of a batch's grids,
// the descriptors carried in the launch's parameters (at most 32,764 bytes on this
// architecture): field f owns the tiles [begin[f], begin[f + 1]) of the launch.
constexpr int kMaxWideFields = 168;
struct WideLaunch {
    int nfields;
    int begin[kMaxWideFields + 1];
    StencilField f[kMaxWideFields];
};
static_assert(sizeof(WideLaunch) <= 32764, "a launch's parameter space holds 32,764 bytes");
cudaError_t launch_stencil_wide(const WideLaunch& L, bool diffuse, int tile_rows, cudaStream_t st);
cudaError_t launch_advect_velocity(const float* u0, const float* v0, float* u, float* v, const AdvectArgs& A,
                                   cudaStream_t st);

// Gauss-Seidel compatibility step (gs.cu): the host solver's method, bit for bit, on a
// square n x n grid of pitched fields; four scratch fields of the same shape.
struct GsFields {
    float *d, *u, *v;
    const float *ds, *us, *vs;
    float* scratch[5];
    float* aux;                 // two floats of device scratch
    SolveCtrl* ctrl;            // grid-barrier state of the tiled solves (larger grids)
    const unsigned* poll_limit; // device word: polls before a grid barrier gives up (0 = default)
};
int gs_max_size();                 // largest n of the one-CTA form on the current device (larger: tiled)
int gs_tiled_max_size();           // largest n the method accepts
cudaError_t gs_prepare();          // shared-memory opt-in on the current device, outside capture
cudaError_t gs_step(const GsFields& F, int n, int pitch, int kd, int kp, float diff, float visc, float dt,
                    cudaStream_t st, int* launches);

}  // namespace fs
