// Solver handle, step orchestration and the C ABI (include/fluid2d_gb300.h).
//
// One handle = one grid on one device with one stream. The step is the reference's
// fluid_solver_gpu::solve (mworchel/fluid-2d src/fluid_solver_gpu.cu:222-258) in the
// same stage order, planned as a short fixed sequence of fused kernels:
//
//   diffuse d,u,v  : ceil(Kd/K) stencil passes, all three fields in each launch
//                    (add_sources fused into the first pass)
//   advect d       : memset + forward splat + finish (Neumann fill + smoothing)
//   project        : ceil(Kp/K) stencil passes (divergence fused into the first,
//                    gradient subtract + reflecting fills into the last)
//   advect u,v     : one backtrace kernel for both components
//   project        : as above
//
// K is the temporal-blocking depth (sweeps per HBM pass). The sequence is captured
// once as a CUDA graph and replayed per step; it is re-captured only when dt or the
// rates change. The reference instead issues ~190 launches, 94 device copies and a
// device-wide synchronisation after every kernel per step.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/fluid2d_gb300.h"
#include "fs_internal.cuh"

#define FS_VERSION "0.1.0"

using namespace fs;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(e == cudaErrorMemoryAllocation ? FS_ERR_NOMEM : FS_ERR_CUDA, m);
}

#define CK(call)                                               \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);    \
    } while (0)

struct DeviceGuard {
    int prev = -1;
    bool changed = false;
    explicit DeviceGuard(int dev) {
        if (dev < 0) return;
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) {
            if (cudaSetDevice(dev) == cudaSuccess) changed = true;
        }
    }
    ~DeviceGuard() {
        if (changed) cudaSetDevice(prev);
    }
};

enum FieldId { F_D = 0, F_U = 1, F_V = 2 };

}  // namespace

// Lets other translation units of the library report through fs_last_error().
int fs::record_error(int code, const char* msg) { return fail(code, msg); }

// A launch of a profiled step: its kind, algorithmic bytes, and whether it ran on the
// density side branch (concurrently with the main stream).
struct ProfMark {
    int kind;
    double bytes;       // per-sweep model: every input read and output written once per sweep
    double pass_bytes;  // the arrays the launch itself must read and write once
    bool branch;
};

struct fs_solver {
    fs_config cfg{};
    int device = 0;
    int rows = 0, cols = 0, pitch = 0;
    size_t field_floats = 0;
    float* slab = nullptr;
    // state and sources
    float* st[3] = {};
    float* src[3] = {};
    // diffusion scratch per field: x0 and two ping-pong buffers
    float* x0[3] = {};
    float* pp[3][2] = {};
    // advection / projection scratch
    float* acc = nullptr;
    float* div = nullptr;
    float* p[2] = {};
    float* vel1[2] = {};
    float* pwarm[2] = {};
    int* flags = nullptr;  // [0]: non-finite; [1]: grid-barrier poll limit of the residual solves (0 = default)
    // residual-driven pressure solves: one control block per projection of a step,
    // and the per-CTA residual partial sums of the persistent kernel
    SolveCtrl* ctrl = nullptr;
    double* partials[2] = {};
    int solve_blocks = 0;
    // training-data capture: each projection's divergence and starting pressure
    float* cap_div[2] = {};
    float* cap_start[2] = {};
    // learned warm start (FS_WARM_LEARNED): network state on a G x G coarse grid
    struct Net {
        float* params = nullptr;          // FP32 [8][32*9*32 + 32]
        __nv_bfloat16* wpk = nullptr;     // packed BF16 weights, 8 x 9216
        __nv_bfloat16* act = nullptr;     // activations (see net_act)
        float* y = nullptr;               // FP32 output, G*G*32
        float* scale = nullptr;
        int* err = nullptr;
        unsigned long long* counters = nullptr;  // [guess used, fallback]
        double* res = nullptr;            // [coarse residual norm^2, energy gain: network, coarse only]
        float* bs = nullptr;              // coarse residual block sums of the current pressure, G*G
        float* yc = nullptr;              // coarse-only correction, G*G*32 (channel 0 used)
        int G = FS_NET_GRID;              // coarse grid side of the network (32 or 64)
        // second, finer coarse level (2G x 2G) on large grids: block sums and the two
        // candidates' corrections in absolute units, channel-0 stride 32; null when unused
        int G2 = 0;
        float* bs2 = nullptr;
        float* e2a = nullptr;
        float* e2b = nullptr;
        float* scale2 = nullptr;
        float* one = nullptr;             // device 1.0f (absolute units)
        void* mem = nullptr;
    } net;
    float* pguess = nullptr;  // fine starting pressure built from the network
    float* plo = nullptr;     // learned residual solves: low part of the pressure (p_hi + p_lo)
    float* rhs = nullptr;     // learned residual solves: FP64-formed residual, the correction's right side
    float* ecur = nullptr;    // learned residual solves: the correction being solved for
    SolveCtrl* host_ctrl = nullptr;  // pinned mirror of a control block (learned cycles)
    fs_source_event* d_events = nullptr;  // device copy of a source script
    int d_events_cap = 0;
    bool net_ready = false;
    long long steps_reported = -1;  // stats.steps when check_flags last reported the residual solves
    cudaStream_t stream = nullptr;
    // density advection runs on `side` beside the first projection (a parallel branch of
    // the step graph), forked and joined by side_ev
    cudaStream_t side = nullptr;
    cudaEvent_t side_ev[2] = {};
    // fs_solve_host on large grids: upload and download streams beside `stream`, and
    // the events that order them (created by the first such call)
    cudaStream_t xfer[2] = {};
    cudaEvent_t xev[6] = {};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    bool graph_valid = false;
    float g_diff = 0, g_visc = 0, g_dt = 0;
    int sweeps = 8;
    int tile_rows = 64;
    // diffuse the density on the side branch too (see density_branch_pays)
    bool density_branch = false;
    int launches_per_step = 0;
    int passes_per_step = 0;
    bool warm_valid = false;
    fs_stats stats{};
    // per-kernel event timing (fs_profile_step); null outside a profiled step
    fs_kernel_times* prof = nullptr;
    std::vector<cudaEvent_t> prof_events;
    std::vector<ProfMark> prof_marks;  // one per profiled launch
};

namespace {

// Default temporal-blocking depth (sweeps per pass). From 1024^2 up, 8 is within 3 %
// of the best depth measured on GB300 (4 to 16 sweeps, 64- and 128-row regions). A grid
// whose one-field pass at depth 8 fills less than half a wave of CTAs is launch-bound
// instead: there the fewest passes win (512^2: 0.222 -> 0.205 ms per 40/40 step; 130^2:
// 0.116 -> 0.087 ms per 20/20 step), as long as output tiles keep 16 rows. Solves to a
// residual target keep depth 8, since their pass count is not fixed.
int default_sweeps(const fs_config* cfg, int dev, int maxk) {
    const int k8 = std::min(8, maxk);
    if (cfg->pressure_tolerance > 0.f) return k8;
    const int tr = cfg->tile_rows ? cfg->tile_rows : 64;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) return k8;
    const int slots = sms * (tr <= 64 ? 2 : 1);
    auto tiles = [&](int halo) {
        const long tw = kRegionW - 2 * halo, th = tr - 2 * halo;
        return ((cfg->cols + tw - 1) / tw) * ((cfg->rows + th - 1) / th);
    };
    if (2 * tiles(k8 + 1) >= slots) return k8;
    const int kmax = std::min(maxk, (tr - 16) / 2 - 1);
    if (kmax <= k8) return k8;
    const int total = std::max(cfg->diffuse_iterations, cfg->pressure_iterations);
    const int passes = std::max(1, (total + kmax - 1) / kmax);
    return std::max(k8, (total + passes - 1) / passes);
}

// The step's stream at the device's highest priority and the side stream (density
// advection) at its lowest, so that the side branch of a step takes only the SMs the
// pressure passes leave free.
cudaError_t create_streams(fs_solver* s) {
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e != cudaSuccess) return e;
    if ((e = cudaStreamCreateWithPriority(&s->stream, cudaStreamNonBlocking, greatest)) != cudaSuccess) return e;
    return cudaStreamCreateWithPriority(&s->side, cudaStreamNonBlocking, least);
}

// Whether to diffuse the density on the step's side branch instead of in the same
// launches as u and v. Fields are independent, so the density passes can fill the SMs the
// u/v passes leave idle in their last wave; that pays where a fused three-field pass has
// a short last wave among few (1024^2: 0.359 -> 0.335 ms per 40/40 step, 2048^2: 1.034 ->
// 1.023 ms) and costs where the last wave is negligible (4096^2, 31 waves: +0.5 %) or the
// step is launch-bound (130^2: +5 %). So: when the fused pass fills 1 to 12 waves.
bool density_branch_pays(const fs_solver* s, int dev) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) return false;
    const int slots = sms * (s->tile_rows <= 64 ? 2 : 1);
    const long tw = kRegionW - 2 * s->sweeps, th = s->tile_rows - 2 * s->sweeps;
    if (tw <= 0 || th <= 0) return false;
    const long tiles3 = 3 * ((s->cols + tw - 1) / tw) * ((s->rows + th - 1) / th);
    return tiles3 >= slots && tiles3 <= 12L * slots;
}

// Split `total` sweeps into passes of at most `k` (at least one pass, possibly of
// zero sweeps, so that fused work such as add_sources always runs).
std::vector<int> split_sweeps(int total, int k) {
    int m = std::max(1, (total + k - 1) / k);
    std::vector<int> out(m, total / m);
    for (int i = 0; i < total % m; ++i) out[i] += 1;
    return out;
}

void set_geometry(StencilField& f, const fs_solver* s, int halo) {
    f.rows = s->rows;
    f.cols = s->cols;
    f.pitch = s->pitch;
    f.halo = halo;
    f.tile_w = kRegionW - 2 * halo;
    f.tile_h = s->tile_rows - 2 * halo;
    tile_split(s->cols, f.tile_w, &f.tiles_x, &f.shift_x);
    tile_split(s->rows, f.tile_h, &f.tiles_y, &f.shift_y);
}

void diffuse_constants(StencilField& f, int rows, int cols, float rate, float dt) {
    // a = dt * T(rows*cols) * rate in float (fluid_solver_gpu.cu:79)
    const float a = dt * (float)((size_t)rows * (size_t)cols) * rate;
    const double D = 1.0 + 4.0 * (double)a;
    f.a = a;
    f.dh = (float)D;
    f.dl = (float)(D - (double)f.dh);
    f.rf = (float)(1.0 / D);
}

AdvectArgs advect_args(const fs_solver* s, float dt) {
    AdvectArgs A;
    A.rows = s->rows;
    A.cols = s->cols;
    A.pitch = s->pitch;
    // float dt0 = sqrt(m_rows * m_cols) * dt, evaluated in double (fluid_solver_gpu.cu:334)
    A.dt0 = (float)(std::sqrt((double)((size_t)s->rows * (size_t)s->cols)) * (double)dt);
    A.xmax = (float)s->cols - 1.5f;
    A.ymax = (float)s->rows - 1.5f;
    return A;
}

float grid_h(int rows, int cols) {
    // h = 1.0f / sqrtf(m_rows * m_cols) (fluid_solver_gpu.cu:367)
    return 1.0f / sqrtf((float)((size_t)rows * (size_t)cols));
}

struct Counter {
    int launches = 0;
    int passes = 0;
};

double interior_cells(const fs_solver* s) { return (double)(s->rows - 2) * (double)(s->cols - 2); }

// Event before a launch on stream st (profiled steps only).
int prof_begin(fs_solver* s, cudaStream_t st) {
    if (!s->prof) return FS_OK;
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    s->prof_events.push_back(e);
    // an event-record node when the profiled step is being captured (fs_profile_step)
    CK(cudaEventRecordWithFlags(e, st, cudaEventRecordExternal));
    return FS_OK;
}

// Event after a launch on stream st, tagged with its kind, its algorithmic bytes and
// whether it ran on the density side branch (concurrently with the main stream).
int prof_end(fs_solver* s, cudaStream_t st, int kind, double bytes, double pass_bytes) {
    if (!s->prof) return FS_OK;
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    s->prof_events.push_back(e);
    CK(cudaEventRecordWithFlags(e, st, cudaEventRecordExternal));
    s->prof_marks.push_back({kind, bytes, pass_bytes, st != s->stream});
    return FS_OK;
}

#define PROF_BEGIN_ON(s, st)                          \
    do {                                              \
        int rc_ = prof_begin(s, st);                  \
        if (rc_ != FS_OK) return rc_;                 \
    } while (0)
#define PROF_END_PASS(s, st, kind, bytes, pass_bytes)        \
    do {                                                     \
        int rc_ = prof_end(s, st, kind, bytes, pass_bytes);  \
        if (rc_ != FS_OK) return rc_;                        \
    } while (0)
#define PROF_END_ON(s, st, kind, bytes) PROF_END_PASS(s, st, kind, bytes, bytes)
#define PROF_BEGIN(s) PROF_BEGIN_ON(s, (s)->stream)
#define PROF_END(s, kind, bytes) PROF_END_ON(s, (s)->stream, kind, bytes)

// Diffusion of a subset of {d, u, v}: add_sources fused into pass 0. Returns the
// buffer holding each field's result in out[].
int enqueue_diffuse(fs_solver* s, const int* fields, int nf, const float* rates, float dt, float** out,
                    Counter& cnt, cudaStream_t st = nullptr) {
    if (!st) st = s->stream;
    const std::vector<int> plan = split_sweeps(s->cfg.diffuse_iterations, s->sweeps);
    const float* cur[3] = {};
    for (int q = 0; q < nf; ++q) cur[q] = s->st[fields[q]];
    for (size_t pass = 0; pass < plan.size(); ++pass) {
        StencilLaunch L{};
        L.nfields = nf;
        int begin = 0;
        for (int q = 0; q < nf; ++q) {
            const int fid = fields[q];
            StencilField& f = L.f[q];
            set_geometry(f, s, plan[pass]);
            realign_columns(f);
            diffuse_constants(f, s->rows, s->cols, rates[q], dt);
            const int mode = fid == F_D ? BND_CONT : (fid == F_U ? BND_OPP_H : BND_OPP_V);
            f.s_lr = bnd_sign_lr(mode);
            f.s_tb = bnd_sign_tb(mode);
            f.sweeps = plan[pass];
            f.dt = dt;
            f.x = cur[q];
            float* dst = s->pp[fid][pass & 1];
            f.y = dst;
            if (pass == 0) {
                f.kind = PASS_DIFFUSE_FIRST;
                f.x2 = s->src[fid];
                f.cst_out = s->x0[fid];
            } else {
                f.kind = PASS_DIFFUSE;
                f.cst = s->x0[fid];
            }
            f.tile_begin = begin;
            begin += f.tiles_x * f.tiles_y;
            cur[q] = dst;
        }
        // per field: 12 B/cell per sweep (read x and x0, write x) + 12 B/cell add_sources;
        // the pass itself reads x and x0 (first: x and s) and writes x (first: and x0)
        const double bytes = nf * interior_cells(s) * (12.0 * plan[pass] + (pass == 0 ? 12.0 : 0.0));
        const double pass_bytes = nf * interior_cells(s) * (pass == 0 ? 16.0 : 12.0);
        PROF_BEGIN_ON(s, st);
        CK(launch_stencil(L, s->tile_rows, st));
        PROF_END_PASS(s, st, FS_KIND_STENCIL, bytes, pass_bytes);
        cnt.launches++;
        cnt.passes++;
    }
    for (int q = 0; q < nf; ++q) out[q] = const_cast<float*>(cur[q]);
    return FS_OK;
}

constexpr int kNetGMax = FS_NET_GRID_MAX;
constexpr int kNetC = 32;
constexpr int kNetLayer = 32 * 9 * 32 + 32;
// output units of the network on a G x G grid (restriction and prolongation use the same)
inline float net_kappa(int G) { return (float)G * (float)G / 16.0f; }
// activation buffers (BF16, 32 channels): xin, e1, pool1, e2, e3, pool2, b1, b2, d1, d2, out
constexpr int kNetActs = 11;
inline size_t net_act_pixels(int k, int G) {
    const int lv[kNetActs] = {0, 0, 1, 1, 1, 2, 2, 2, 1, 0, 0};
    const int g = G >> lv[k];
    return (size_t)g * g;
}
__nv_bfloat16* net_act(fs_solver* s, int k) {
    size_t off = 0;
    for (int i = 0; i < k; ++i) off += net_act_pixels(i, s->net.G) * kNetC;
    return s->net.act + off;
}

// Divergence of (u_in, v_in) into s->div: a pressure pass of zero sweeps.
int enqueue_div_pass(fs_solver* s, const float* u_in, const float* v_in, Counter& cnt) {
    const float h = grid_h(s->rows, s->cols);
    StencilLaunch L{};
    L.nfields = 1;
    StencilField& f = L.f[0];
    set_geometry(f, s, 1);
    f.s_lr = f.s_tb = 1.f;
    f.kind = PASS_PRESSURE_FIRST;
    f.sweeps = 0;
    f.cdiv = -0.5f * h;
    f.h = h;
    f.x = u_in;
    f.x2 = v_in;
    f.cst_out = s->div;
    CK(launch_stencil(L, s->tile_rows, s->stream));
    cnt.launches++;
    return FS_OK;
}

// Jacobi sweeps after each correction by default: at 1e-4, 300 steps, 2048^2 the learned
// corrections took 47.8 / 42.3 / 39.8 ms per step with 128 / 192 / 256 (20-step runs) while
// the network-free coarse corrections were fastest at 128 (48.1): a better correction
// needs fewer of them, so the learned mode's default is the longer cycle.
constexpr int kLearnedCycleSweeps = 256;
constexpr int kCoarseSweeps = 20;       // on the network's grid
constexpr int kCoarseSweepsFine = 200;  // on the finer coarse level

// One learned correction of p_cur (the current pressure, edges filled): two damped
// Jacobi steps (see launch_damp), then the block sums
// of its residual on the coarse grid, the 8-layer network on the tensor cores, coarse
// post-smoothing, bilinear interpolation into a candidate p_cur + correction; beside it
// the classical candidate (the coarse smoothing from zero, no network). The acceptance rule keeps
// the candidate that brings p_cur closest to the solution in the A-norm (the norm the
// Jacobi iteration contracts), or p_cur when neither gets closer, and counts whether the
// network's candidate won. Does nothing to p_cur once *converged (nullable) is set. rhs is
// the right side of the problem p_cur approximates: the divergence, or in a defect
// correction cycle the residual the correction solves for.
int enqueue_network_correction(fs_solver* s, const float* rhs, float* p_cur, const int* converged, Counter& cnt) {
    const int G = s->net.G;
    // one damped Jacobi step first: removes the checkerboard error plain Jacobi never damps
    CK(launch_damp(rhs, p_cur, s->p[0], s->rows, s->cols, s->pitch, converged, s->stream));
    CK(launch_damp(rhs, s->p[0], p_cur, s->rows, s->cols, s->pitch, converged, s->stream));
    cnt.launches += 2;
    const float kappa = net_kappa(G);
    const int G2 = s->net.G2;
    if (G2) {
        // block sums on the finer level, summed up for the network's level
        CK(launch_coarse_residual(rhs, p_cur, s->rows, s->cols, s->pitch, G2, s->net.bs2, nullptr, s->net.scale2,
                                  nullptr, converged, s->stream));
        CK(launch_coarse_sum2x2(s->net.bs2, s->net.bs, G, converged, s->stream));
        CK(launch_coarse_input(s->net.bs, G, s->net.scale, net_act(s, 0), s->net.res, converged, s->stream));
        cnt.launches += 4;
    } else {
        CK(launch_coarse_residual(rhs, p_cur, s->rows, s->cols, s->pitch, G, s->net.bs, s->net.res, s->net.scale,
                                  net_act(s, 0), converged, s->stream));
        cnt.launches += 2;
    }
    int rc;
    auto conv = [&](int li, int in, int out, int lvl, int up, int skip, int relu, float* yf) {
        const int g = G >> lvl;
        return conv3x3_launch(net_act(s, in), s->net.wpk + (size_t)li * 9216, nullptr,
                              s->net.params + (size_t)li * kNetLayer + 9216, skip >= 0 ? net_act(s, skip) : nullptr,
                              out >= 0 ? net_act(s, out) : nullptr, yf, g, g, g, up, relu, 1, s->net.err, converged,
                              s->stream);
    };
    // e1 (G) -> pool -> e2, e3 (G/2) -> pool -> b1, b2 (G/4) -> d1 (+e3) -> d2 (+e1) -> out:
    // one fused launch on the 32 x 32 grid, layer by layer on the 64 x 64 one
    if (G == 32) {
        if ((rc = net_infer32_launch(net_act(s, 0), s->net.wpk, s->net.params, net_act(s, 1), s->net.y, 1, s->net.err,
                                     converged, s->stream)) != FS_OK)
            return rc;
        cnt.launches += 1;
    } else {
        if ((rc = conv(0, 0, 1, 0, 0, -1, 1, nullptr)) != FS_OK) return rc;
        if ((rc = fs_net_avgpool2(net_act(s, 1), net_act(s, 2), G / 2, G / 2, s->stream)) != FS_OK) return rc;
        if ((rc = conv(1, 2, 3, 1, 0, -1, 1, nullptr)) != FS_OK) return rc;
        if ((rc = conv(2, 3, 4, 1, 0, -1, 1, nullptr)) != FS_OK) return rc;
        if ((rc = fs_net_avgpool2(net_act(s, 4), net_act(s, 5), G / 4, G / 4, s->stream)) != FS_OK) return rc;
        if ((rc = conv(3, 5, 6, 2, 0, -1, 1, nullptr)) != FS_OK) return rc;
        if ((rc = conv(4, 6, 7, 2, 0, -1, 1, nullptr)) != FS_OK) return rc;
        if ((rc = conv(5, 7, 8, 1, 1, 4, 1, nullptr)) != FS_OK) return rc;
        if ((rc = conv(6, 8, 9, 0, 1, 1, 1, nullptr)) != FS_OK) return rc;
        if ((rc = conv(7, 9, 10, 0, 0, -1, 0, s->net.y)) != FS_OK) return rc;
        cnt.launches += 10;
    }
    // candidate A: the network's correction, post-smoothed; B: the coarse smoothing alone
    float* pb = s->p[1];  // free between pressure passes
    CK(launch_coarse_smooth_pair(s->net.y, s->net.y, nullptr, s->net.yc, s->net.bs, s->net.scale, kappa, G,
                                 kCoarseSweeps, converged, s->stream));
    if (G2) {
        // both candidates continue on the finer coarse level, then go to the fine grid
        CK(launch_coarse_interp(s->net.y, s->net.e2a, G, s->net.scale, kappa, converged, s->stream));
        CK(launch_coarse_interp(s->net.yc, s->net.e2b, G, s->net.scale, kappa, converged, s->stream));
        CK(launch_coarse_smooth_pair(s->net.e2a, s->net.e2a, s->net.e2b, s->net.e2b, s->net.bs2, s->net.one, 1.f, G2,
                                     kCoarseSweepsFine, converged, s->stream));
        CK(launch_prolong(s->net.e2a, p_cur, s->pguess, s->rows, s->cols, s->pitch, G2, s->net.one, 1.f, converged,
                          s->stream));
        CK(launch_prolong(s->net.e2b, p_cur, pb, s->rows, s->cols, s->pitch, G2, s->net.one, 1.f, converged,
                          s->stream));
        cnt.launches += 5;
    } else {
        CK(launch_prolong(s->net.y, p_cur, s->pguess, s->rows, s->cols, s->pitch, G, s->net.scale, kappa, converged,
                          s->stream));
        CK(launch_prolong(s->net.yc, p_cur, pb, s->rows, s->cols, s->pitch, G, s->net.scale, kappa, converged,
                          s->stream));
        cnt.launches += 2;
    }
    CK(cudaMemsetAsync(s->net.res + 1, 0, 2 * sizeof(double), s->stream));
    CK(launch_energy_gain(rhs, p_cur, s->pguess, s->rows, s->cols, s->pitch, s->net.res + 1, converged, s->stream));
    CK(launch_energy_gain(rhs, p_cur, pb, s->rows, s->cols, s->pitch, s->net.res + 2, converged, s->stream));
    CK(launch_accept_best(p_cur, s->pguess, pb, (long)s->field_floats, s->net.res + 1, converged, s->net.counters,
                          s->stream));
    cnt.launches += 4;  // the smoothing pair, two energy gains, the choice
    return FS_OK;
}

// Starting pressure of a fixed-count projection with the learned warm start: the
// previous pressure (zero on the first step) in pwarm[slot], corrected once.
int enqueue_learned_guess(fs_solver* s, const float* u_in, const float* v_in, int slot, Counter& cnt) {
    int rc = enqueue_div_pass(s, u_in, v_in, cnt);
    if (rc != FS_OK) return rc;
    if (!s->warm_valid) CK(cudaMemsetAsync(s->pwarm[slot], 0, s->field_floats * sizeof(float), s->stream));
    return enqueue_network_correction(s, s->div, s->pwarm[slot], nullptr, cnt);
}

// Starting pressure of projection `slot`: the network's guess, the previous pressure,
// or null (zero, as the reference), and its copy for training-data capture.
int projection_start(fs_solver* s, const float* u_in, const float* v_in, int slot, Counter& cnt, const float** pin) {
    const bool warm = s->cfg.warm_start != FS_WARM_ZERO;
    *pin = (warm && s->warm_valid) ? s->pwarm[slot] : nullptr;
    if (s->cfg.warm_start == FS_WARM_LEARNED && s->net_ready) {
        int rc = enqueue_learned_guess(s, u_in, v_in, slot, cnt);
        if (rc != FS_OK) return rc;
        *pin = s->pwarm[slot];
    }
    if (s->cfg.capture) {
        if (*pin)
            CK(cudaMemcpyAsync(s->cap_start[slot], *pin, s->field_floats * sizeof(float), cudaMemcpyDeviceToDevice,
                               s->stream));
        else
            CK(cudaMemsetAsync(s->cap_start[slot], 0, s->field_floats * sizeof(float), s->stream));
    }
    return FS_OK;
}

int capture_div(fs_solver* s, int slot) {
    if (!s->cfg.capture) return FS_OK;
    CK(cudaMemcpyAsync(s->cap_div[slot], s->div, s->field_floats * sizeof(float), cudaMemcpyDeviceToDevice,
                       s->stream));
    return FS_OK;
}

// project (fluid_solver_gpu.cu:358-404): (u_in, v_in) -> (u_out, v_out). slot picks
// the warm-start pressure buffer (the two projections of a step keep separate ones).
// Residual-driven projection: one persistent cooperative launch runs depth-K passes
// until the relative residual ||div + sum(nbrs) - 4p|| / ||div|| is <= tol or the
// iteration cap is reached, then the gradient subtract (see pressure_solve_kernel).
int enqueue_fin_pass(fs_solver* s, const float* p, const float* u_in, const float* v_in, float* u_out, float* v_out,
                     Counter& cnt) {
    PROF_BEGIN(s);
    CK(launch_gradient(p, u_in, v_in, u_out, v_out, s->rows, s->cols, s->pitch, grid_h(s->rows, s->cols),
                       s->cfg.check_finite ? s->flags : nullptr, s->stream));
    PROF_END(s, FS_KIND_GRADIENT, interior_cells(s) * 20.0);  // read p, u, v; write u, v
    cnt.launches++;
    return FS_OK;
}

// Residual-driven projection with learned corrections: the current pressure starts
// as the previous one (zero on the first step); each cycle corrects it with the network
// (kept only if the coarse residual drops) and runs a segment of Jacobi passes until
// the residual target or the segment's budget. Outside a stream capture the host reads
// each segment's outcome and stops at convergence; inside one, all cycles are recorded
// and those after convergence do nothing. Cycles: learned_cycles, or as many as the
// iteration cap allows; the last gets the rest of the cap.
int enqueue_project_learned_cycles(fs_solver* s, const float* u_in, const float* v_in, float* u_out, float* v_out,
                                   int slot, Counter& cnt) {
    const int K = s->sweeps;
    const int per = s->cfg.learned_cycle_iterations > 0 ? s->cfg.learned_cycle_iterations : kLearnedCycleSweeps;
    const int cap = s->cfg.pressure_max_iterations;
    const int cycles = s->cfg.learned_cycles > 0 ? s->cfg.learned_cycles : std::max(1, (cap + per - 1) / per);
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(s->stream, &capture));
    const bool adaptive = capture == cudaStreamCaptureStatusNone && s->host_ctrl != nullptr;
    int rc = enqueue_div_pass(s, u_in, v_in, cnt);
    if (rc != FS_OK) return rc;
    float* pcur = s->pwarm[slot];
    if (!s->warm_valid) CK(cudaMemsetAsync(pcur, 0, s->field_floats * sizeof(float), s->stream));
    if (s->cfg.capture)
        CK(cudaMemcpyAsync(s->cap_start[slot], pcur, s->field_floats * sizeof(float), cudaMemcpyDeviceToDevice,
                           s->stream));
    CK(cudaMemsetAsync(s->ctrl + slot, 0, sizeof(SolveCtrl), s->stream));
    PressureSolve P{};
    set_geometry(P.mid, s, K + 1);
    realign_columns(P.mid);  // interior tiles take the direct path (P.first copies the tiling)
    P.mid.s_lr = P.mid.s_tb = 1.f;
    P.mid.sweeps = K;
    P.mid.h = grid_h(s->rows, s->cols);
    P.mid.kind = PASS_PRESSURE;
    P.mid.cst = s->div;
    P.first = P.mid;
    P.first.x = pcur;
    P.p[0] = s->p[0];
    P.p[1] = s->p[1];
    P.partials = s->partials[slot];
    P.ctrl = s->ctrl + slot;
    P.poll_limit = reinterpret_cast<const unsigned*>(s->flags + 1);
    P.tol = s->cfg.pressure_tolerance;
    P.segment = 1;
    P.p_cur = pcur;
    const int blocks = std::min(s->solve_blocks, P.mid.tiles_x * P.mid.tiles_y);
    for (int c = 0; c < cycles; ++c) {
        if ((rc = enqueue_network_correction(s, s->div, pcur, &P.ctrl->converged, cnt)) != FS_OK) return rc;
        const int budget = c + 1 < cycles ? per : std::max(per, cap - (cycles - 1) * per);
        P.max_passes = std::max(1, (budget + K - 1) / K);
        PROF_BEGIN(s);
        CK(launch_pressure_solve(P, s->tile_rows, blocks, s->stream));
        PROF_END(s, FS_KIND_STENCIL, 0.0);  // bytes depend on the iteration count reached
        cnt.launches++;
        cnt.passes++;
        if (adaptive && c + 1 < cycles) {
            CK(cudaMemcpyAsync(s->host_ctrl, P.ctrl, sizeof(SolveCtrl), cudaMemcpyDeviceToHost, s->stream));
            CK(cudaStreamSynchronize(s->stream));
            if (s->host_ctrl->converged || s->host_ctrl->error) break;
        }
    }
    if ((rc = enqueue_fin_pass(s, pcur, u_in, v_in, u_out, v_out, cnt)) != FS_OK) return rc;
    return capture_div(s, slot);
}

// Residual-driven projection with learned corrections as mixed-precision defect
// correction (outside a stream capture). The pressure is p_hi + p_lo (pwarm[slot] and
// plo): each cycle forms the residual r of that sum in FP64 (launch_residual_df), stops
// when ||r|| / ||div|| <= tol, and otherwise solves A e = r for a correction e in FP32 —
// from e = 0, one network correction (the same cycle as below, on r) and a segment of
// Jacobi passes until ||r - A e|| <= tol ||div|| or the segment's budget — and adds e to
// the pressure exactly (launch_accumulate_df). The FP32 iterate alone stalls near its
// rounding floor (about 4 eps |p| per cell); the correction's floor is relative to |e|,
// so the residual keeps falling cycle after cycle. The velocity is then corrected with
// p_hi, the pressure rounded to FP32 as the reference stores it.
int enqueue_project_learned_defect(fs_solver* s, const float* u_in, const float* v_in, float* u_out, float* v_out,
                                   int slot, Counter& cnt) {
    const int K = s->sweeps;
    const int per = s->cfg.learned_cycle_iterations > 0 ? s->cfg.learned_cycle_iterations : kLearnedCycleSweeps;
    const int cap = s->cfg.pressure_max_iterations;
    const int cycles = s->cfg.learned_cycles > 0 ? s->cfg.learned_cycles : std::max(1, (cap + per - 1) / per);
    const double tol = s->cfg.pressure_tolerance;
    int rc = enqueue_div_pass(s, u_in, v_in, cnt);
    if (rc != FS_OK) return rc;
    float* phi = s->pwarm[slot];
    const size_t fbytes = s->field_floats * sizeof(float);
    if (!s->warm_valid) CK(cudaMemsetAsync(phi, 0, fbytes, s->stream));
    CK(cudaMemsetAsync(s->plo, 0, fbytes, s->stream));
    if (s->cfg.capture) CK(cudaMemcpyAsync(s->cap_start[slot], phi, fbytes, cudaMemcpyDeviceToDevice, s->stream));
    double* dsums = reinterpret_cast<double*>(s->flags + 4);  // two doubles in the flag block
    double* hsums = reinterpret_cast<double*>(s->host_ctrl + 1);
    PressureSolve P{};
    set_geometry(P.mid, s, K + 1);
    realign_columns(P.mid);  // interior tiles take the direct path (P.first copies the tiling)
    P.mid.s_lr = P.mid.s_tb = 1.f;
    P.mid.sweeps = K;
    P.mid.h = grid_h(s->rows, s->cols);
    P.mid.kind = PASS_PRESSURE;
    P.mid.cst = s->rhs;
    P.first = P.mid;
    P.first.x = s->ecur;
    P.p[0] = s->p[0];
    P.p[1] = s->p[1];
    P.partials = s->partials[slot];
    P.ctrl = s->ctrl + slot;
    P.poll_limit = reinterpret_cast<const unsigned*>(s->flags + 1);
    P.segment = 1;
    P.p_cur = s->ecur;
    const int blocks = std::min(s->solve_blocks, P.mid.tiles_x * P.mid.tiles_y);
    int passes = 0, used = 0;
    double ratio = 1.0;
    bool converged = false, timed_out = false;
    for (int c = 0; c <= cycles; ++c) {
        CK(cudaMemsetAsync(dsums, 0, 2 * sizeof(double), s->stream));
        CK(launch_residual_df(s->div, phi, s->plo, s->rhs, s->rows, s->cols, s->pitch, dsums, s->stream));
        CK(cudaMemcpyAsync(hsums, dsums, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        cnt.launches++;
        ratio = hsums[1] > 0.0 ? std::sqrt(hsums[0] / hsums[1]) : std::sqrt(hsums[0]);
        converged = ratio <= tol;
        if (converged || c == cycles || used >= cap) break;
        // the correction: from zero, to the residual that would meet the target
        CK(cudaMemsetAsync(s->ecur, 0, fbytes, s->stream));
        CK(cudaMemsetAsync(P.ctrl, 0, sizeof(SolveCtrl), s->stream));
        if ((rc = enqueue_network_correction(s, s->rhs, s->ecur, nullptr, cnt)) != FS_OK) return rc;
        // the last cycle gets the rest of the cap, as in the FP32 form
        const int budget = c + 1 < cycles ? std::min(per, cap - used) : cap - used;
        P.max_passes = std::max(1, (budget + K - 1) / K);
        P.tol = (float)std::min(0.5, hsums[0] > 0.0 ? tol * std::sqrt(hsums[1] / hsums[0]) : 1.0);
        PROF_BEGIN(s);
        CK(launch_pressure_solve(P, s->tile_rows, blocks, s->stream));
        PROF_END(s, FS_KIND_STENCIL, 0.0);  // bytes depend on the iteration count reached
        cnt.launches++;
        cnt.passes++;
        CK(cudaMemcpyAsync(s->host_ctrl, P.ctrl, sizeof(SolveCtrl), cudaMemcpyDeviceToHost, s->stream));
        CK(launch_accumulate_df(phi, s->plo, s->ecur, (long)s->field_floats, s->stream));
        cnt.launches++;
        CK(cudaStreamSynchronize(s->stream));
        passes += s->host_ctrl->passes;
        used += s->host_ctrl->passes * K;
        if (s->host_ctrl->error) {
            timed_out = true;
            break;
        }
    }
    // the outcome, where check_flags and fs_get_stats read it
    SolveCtrl out{};
    out.passes = passes;
    out.converged = converged ? 1 : 0;
    out.error = timed_out ? 1 : 0;
    out.residual = ratio;
    *s->host_ctrl = out;
    CK(cudaMemcpyAsync(s->ctrl + slot, s->host_ctrl, sizeof(SolveCtrl), cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if ((rc = enqueue_fin_pass(s, phi, u_in, v_in, u_out, v_out, cnt)) != FS_OK) return rc;
    return capture_div(s, slot);
}

int enqueue_project_to_residual(fs_solver* s, const float* u_in, const float* v_in, float* u_out, float* v_out,
                                int slot, Counter& cnt) {
    if (s->cfg.warm_start == FS_WARM_LEARNED && s->net_ready) {
        cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(s->stream, &capture));
        if (capture == cudaStreamCaptureStatusNone && s->host_ctrl != nullptr && s->cfg.learned_defect)
            return enqueue_project_learned_defect(s, u_in, v_in, u_out, v_out, slot, cnt);
        return enqueue_project_learned_cycles(s, u_in, v_in, u_out, v_out, slot, cnt);
    }
    const bool warm = s->cfg.warm_start != FS_WARM_ZERO;
    const float h = grid_h(s->rows, s->cols);
    const int K = s->sweeps;
    PressureSolve P{};
    for (StencilField* f : {&P.first, &P.mid}) {
        set_geometry(*f, s, K + 1);
        realign_columns(*f);  // one tiling for both; the middle passes' interior tiles go direct
        f->s_lr = f->s_tb = 1.f;
        f->sweeps = K;
        f->cdiv = -0.5f * h;
        f->h = h;
    }
    const float* pin = nullptr;
    int rc = projection_start(s, u_in, v_in, slot, cnt, &pin);
    if (rc != FS_OK) return rc;
    P.first.kind = PASS_PRESSURE_FIRST;
    P.first.x = u_in;
    P.first.x2 = v_in;
    P.first.cst = pin;
    P.first.cst_out = s->div;
    P.mid.kind = PASS_PRESSURE;
    P.mid.cst = s->div;
    P.p[0] = s->p[0];
    P.p[1] = s->p[1];
    P.p_out = warm ? s->pwarm[slot] : nullptr;
    P.partials = s->partials[slot];
    P.ctrl = s->ctrl + slot;
    P.poll_limit = reinterpret_cast<const unsigned*>(s->flags + 1);
    P.tol = s->cfg.pressure_tolerance;
    P.max_passes = std::max(1, (s->cfg.pressure_max_iterations + K - 1) / K);
    CK(cudaMemsetAsync(P.ctrl, 0, sizeof(SolveCtrl), s->stream));
    const int blocks = std::min(s->solve_blocks, P.mid.tiles_x * P.mid.tiles_y);
    PROF_BEGIN(s);
    CK(launch_pressure_solve(P, s->tile_rows, blocks, s->stream));
    PROF_END(s, FS_KIND_STENCIL, 0.0);  // bytes depend on the iteration count reached
    // gradient subtract from the buffer the solve ended in (P.ctrl->cur)
    PROF_BEGIN(s);
    CK(launch_gradient(s->p[0], u_in, v_in, u_out, v_out, s->rows, s->cols, s->pitch, h,
                       s->cfg.check_finite ? s->flags : nullptr, s->stream, s->p[1], &P.ctrl->cur));
    PROF_END(s, FS_KIND_GRADIENT, interior_cells(s) * 20.0);  // read p, u, v; write u, v
    cnt.launches += 2;
    cnt.passes++;
    return capture_div(s, slot);
}

int enqueue_project(fs_solver* s, const float* u_in, const float* v_in, float* u_out, float* v_out, int slot,
                    Counter& cnt) {
    if (s->cfg.pressure_tolerance > 0.f) return enqueue_project_to_residual(s, u_in, v_in, u_out, v_out, slot, cnt);
    const std::vector<int> plan = split_sweeps(s->cfg.pressure_iterations, s->sweeps);
    const int m = (int)plan.size();
    const bool warm = s->cfg.warm_start != FS_WARM_ZERO;
    const float h = grid_h(s->rows, s->cols);
    const float* pin = nullptr;
    int rc = projection_start(s, u_in, v_in, slot, cnt, &pin);
    if (rc != FS_OK) return rc;
    // A single pass fuses the gradient subtract into its epilogue. With more passes the
    // last is an ordinary pass that stores the final pressure (edges filled) and a separate
    // bandwidth-bound launch subtracts the gradient (gradient_kernel): the epilogue's loads
    // and stores, issued behind the sweeps of each tile, had made that pass twice as long
    // as a middle one (60 against 29 us at 2048^2).
    const bool split = m >= 2;
    float* pfinal = nullptr;
    for (int pass = 0; pass < m; ++pass) {
        const bool last = pass == m - 1;
        const bool fused = last && !split;
        StencilLaunch L{};
        L.nfields = 1;
        StencilField& f = L.f[0];
        set_geometry(f, s, plan[pass] + (fused ? 1 : 0));
        if (pass > 0) realign_columns(f);  // the first pass's tiling is aligned at depth 8
        f.s_lr = f.s_tb = 1.f;
        f.sweeps = plan[pass];
        f.cdiv = -0.5f * h;
        f.h = h;
        float* pout = s->p[pass & 1];
        if (last && split && warm) pout = s->pwarm[slot];
        if (fused) pout = warm ? s->p[0] : nullptr;
        if (last) pfinal = pout;
        if (pass == 0) {
            f.kind = PASS_PRESSURE_FIRST;
            f.x = u_in;
            f.x2 = v_in;
            f.cst = pin;  // starting pressure (null: zero, as the reference)
            f.cst_out = s->div;
        } else {
            f.kind = PASS_PRESSURE;
            f.x = s->p[(pass - 1) & 1];
            f.cst = s->div;
        }
        f.y = pout;
        if (fused) {
            f.epilogue = 1;
            f.u_in = u_in;
            f.v_in = v_in;
            f.u_out = u_out;
            f.v_out = v_out;
            f.nonfinite = s->cfg.check_finite ? s->flags : nullptr;
        }
        // 12 B/cell per sweep (read p and div, write p), + 12 divergence, + 20 gradient;
        // the pass itself reads p and div (first: u and v, and p when warm) and writes p
        // (first: and div; a fused last pass: u and v instead of p)
        const double bytes =
            interior_cells(s) * (12.0 * plan[pass] + (pass == 0 ? 12.0 : 0.0) + (fused ? 20.0 : 0.0));
        const double pass_bytes =
            interior_cells(s) * ((pass == 0 ? 8.0 + (pin ? 4.0 : 0.0) + 4.0 : 8.0) + (fused ? 16.0 : 4.0));
        PROF_BEGIN(s);
        CK(launch_stencil(L, s->tile_rows, s->stream));
        PROF_END_PASS(s, s->stream, FS_KIND_STENCIL, bytes, pass_bytes);
        cnt.launches++;
        cnt.passes++;
        if (pass == 0 && (rc = capture_div(s, slot)) != FS_OK) return rc;
    }
    if (split) {
        // read p, u, v; write u, v
        PROF_BEGIN(s);
        CK(launch_gradient(pfinal, u_in, v_in, u_out, v_out, s->rows, s->cols, s->pitch, h,
                           s->cfg.check_finite ? s->flags : nullptr, s->stream));
        PROF_END_PASS(s, s->stream, FS_KIND_GRADIENT, interior_cells(s) * 20.0, interior_cells(s) * 20.0);
        cnt.launches++;
    }
    if (warm && m == 1) {
        CK(cudaMemcpyAsync(s->pwarm[slot], s->p[0], s->field_floats * sizeof(float), cudaMemcpyDeviceToDevice,
                           s->stream));
    }
    return FS_OK;
}

int enqueue_advect_density(fs_solver* s, const float* d0, float* d_out, const float* u, const float* v, float dt,
                           Counter& cnt, cudaStream_t st) {
    const AdvectArgs A = advect_args(s, dt);
    PROF_BEGIN_ON(s, st);
    CK(cudaMemsetAsync(s->acc, 0, s->field_floats * sizeof(float), st));
    PROF_END_ON(s, st, FS_KIND_MEMSET, 0.0);
    PROF_BEGIN_ON(s, st);
    CK(launch_splat(d0, u, v, s->acc, A, st));
    PROF_END_ON(s, st, FS_KIND_SPLAT, 16.0 * interior_cells(s));  // read d0, u, v; write d
    PROF_BEGIN_ON(s, st);
    CK(launch_density_finish(s->acc, d_out, s->cfg.smooth, A, s->cfg.check_finite ? s->flags : nullptr, st));
    PROF_END_ON(s, st, FS_KIND_FINISH, 8.0 * interior_cells(s));  // smooth: read d, write d
    cnt.launches += 2;
    return FS_OK;
}

// The density half of a step: forward advection of the diffused density by the step's
// initial velocity (still in the state), then smoothing — and, with diffuse = true, the
// density diffusion before it. It depends on nothing the velocity half writes before its
// second projection, so it runs on the side stream, beside the velocity diffusion and
// the first projection, and join_density() brings it back before the state velocity is
// rewritten. dif_d: the diffused density when diffuse = false.
int fork_density(fs_solver* s, const float* dif_d, float diff, float dt, bool diffuse, Counter& cnt) {
    CK(cudaEventRecord(s->side_ev[0], s->stream));
    CK(cudaStreamWaitEvent(s->side, s->side_ev[0], 0));
    cudaStream_t st = s->side;
    int rc;
    if (diffuse) {
        const int fd = F_D;
        float* out = nullptr;
        if ((rc = enqueue_diffuse(s, &fd, 1, &diff, dt, &out, cnt, st)) != FS_OK) return rc;
        dif_d = out;
    }
    if ((rc = enqueue_advect_density(s, dif_d, s->st[F_D], s->st[F_U], s->st[F_V], dt, cnt, st)) != FS_OK) return rc;
    CK(cudaEventRecord(s->side_ev[1], s->side));
    return FS_OK;
}

int join_density(fs_solver* s) {
    CK(cudaStreamWaitEvent(s->stream, s->side_ev[1], 0));
    return FS_OK;
}

// Velocity half of a step from the diffused velocity: project (into the u/v diffusion
// scratch, free by now, so that the state keeps the initial velocity the density
// advection reads), advect by itself, join the density half, project into the state.
int enqueue_velocity_tail(fs_solver* s, const float* dif_u, const float* dif_v, float dt, Counter& cnt) {
    int rc;
    float* pu = s->x0[F_U];
    float* pv = s->x0[F_V];
    if ((rc = enqueue_project(s, dif_u, dif_v, pu, pv, 0, cnt)) != FS_OK) return rc;
    PROF_BEGIN(s);
    CK(launch_advect_velocity(pu, pv, s->vel1[0], s->vel1[1], advect_args(s, dt), s->stream));
    PROF_END(s, FS_KIND_ADVECT, 16.0 * interior_cells(s));  // read u0, v0; write u, v
    cnt.launches++;
    if ((rc = join_density(s)) != FS_OK) return rc;
    return enqueue_project(s, s->vel1[0], s->vel1[1], s->st[F_U], s->st[F_V], 1, cnt);
}

int enqueue_step(fs_solver* s, float diff, float visc, float dt, Counter& cnt) {
    int rc;
    if (s->cfg.method == FS_METHOD_GAUSS_SEIDEL) {
        GsFields F;
        F.d = s->st[F_D];
        F.u = s->st[F_U];
        F.v = s->st[F_V];
        F.ds = s->src[F_D];
        F.us = s->src[F_U];
        F.vs = s->src[F_V];
        for (int k = 0; k < 3; ++k) F.scratch[k] = s->x0[k];
        F.scratch[3] = s->acc;
        F.scratch[4] = s->p[0];
        F.aux = s->div;  // unused by this method
        F.ctrl = s->ctrl;
        F.poll_limit = reinterpret_cast<const unsigned*>(s->flags + 1);
        int launches = 0;
        CK(gs_step(F, s->rows, s->pitch, s->cfg.diffuse_iterations, s->cfg.pressure_iterations, diff, visc, dt,
                   s->stream, &launches));
        cnt.launches += launches;
        return FS_OK;
    }
    if (!s->density_branch) {
        // one diffusion launch per pass serves all three fields
        const int fields[3] = {F_D, F_U, F_V};
        const float rates[3] = {diff, visc, visc};
        float* dif[3];
        if ((rc = enqueue_diffuse(s, fields, 3, rates, dt, dif, cnt)) != FS_OK) return rc;
        if ((rc = fork_density(s, dif[F_D], diff, dt, false, cnt)) != FS_OK) return rc;
        return enqueue_velocity_tail(s, dif[F_U], dif[F_V], dt, cnt);
    }
    // density (diffusion, then forward advection by the step's initial velocity and
    // smoothing) on the low-priority side branch; velocity: diffuse u and v in one launch
    // per pass, project, advect by itself, project
    if ((rc = fork_density(s, nullptr, diff, dt, true, cnt)) != FS_OK) return rc;
    const int fuv[2] = {F_U, F_V};
    const float ruv[2] = {visc, visc};
    float* dif_uv[2];
    if ((rc = enqueue_diffuse(s, fuv, 2, ruv, dt, dif_uv, cnt)) != FS_OK) return rc;
    return enqueue_velocity_tail(s, dif_uv[0], dif_uv[1], dt, cnt);
}

void destroy_graph(fs_solver* s) {
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    if (s->graph) cudaGraphDestroy(s->graph);
    s->gexec = nullptr;
    s->graph = nullptr;
    s->graph_valid = false;
}

int run_steps(fs_solver* s, float diff, float visc, float dt, int nsteps) {
    int rc;
    const bool warm = s->cfg.warm_start != FS_WARM_ZERO;
    for (int k = 0; k < nsteps; ++k) {
        // The first warm-start step starts from zero pressure; its graph differs.
        // learned corrections to a residual target stop at convergence, read on the host
        const bool adaptive = s->cfg.warm_start == FS_WARM_LEARNED && s->net_ready && s->cfg.pressure_tolerance > 0.f;
        bool graphable = s->cfg.use_graph && (!warm || s->warm_valid) && !adaptive;
        if (graphable && (!s->graph_valid || diff != s->g_diff || visc != s->g_visc || dt != s->g_dt)) {
            destroy_graph(s);
            Counter cnt;
            CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            rc = enqueue_step(s, diff, visc, dt, cnt);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(s->stream, &g);
            cudaGraphExec_t ge = nullptr;
            if (rc == FS_OK && e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, cudaGraphInstantiateFlagUseNodePriority);
            if (rc != FS_OK || e != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                if (s->cfg.pressure_tolerance > 0.f) {
                    // the runtime refused to capture the cooperative launch: step eagerly
                    cudaGetLastError();
                    s->cfg.use_graph = 0;
                    graphable = false;
                } else {
                    return rc != FS_OK ? rc : cuda_fail(e, "step graph capture");
                }
            } else {
                s->graph = g;
                s->gexec = ge;
                s->graph_valid = true;
                s->g_diff = diff;
                s->g_visc = visc;
                s->g_dt = dt;
                s->launches_per_step = cnt.launches;
                s->passes_per_step = cnt.passes;
            }
        }
        if (graphable) {
            CK(cudaGraphLaunch(s->gexec, s->stream));
            s->stats.kernel_launches += s->launches_per_step;
        } else {
            Counter cnt;
            if ((rc = enqueue_step(s, diff, visc, dt, cnt)) != FS_OK) return rc;
            s->launches_per_step = cnt.launches;
            s->passes_per_step = cnt.passes;
            s->stats.kernel_launches += cnt.launches;
        }
        s->warm_valid = true;
        s->stats.steps++;
    }
    return FS_OK;
}

// Reads the residual solves' control blocks into the stats (blocking).
int read_solve_ctrl(const fs_solver* s, SolveCtrl* out) {
    CK(cudaMemcpyAsync(out, s->ctrl, 2 * sizeof(SolveCtrl), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FS_OK;
}

int check_flags(fs_solver* s) {
    if (s->cfg.check_finite) {
        int h = 0;
        CK(cudaMemcpyAsync(&h, s->flags, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        if (h) {
            CK(cudaMemsetAsync(s->flags, 0, sizeof(int), s->stream));
            s->stats.nonfinite = 1;
            return fail(FS_ERR_NONFINITE, "the step produced a non-finite value");
        }
    }
    if (s->net_ready && s->net.err) {
        // a tensor-core wait of the network gave up (conv3x3_tc_kernel, net_infer32_kernel):
        // stop using the network until fs_set_network loads it again
        int h = 0;
        CK(cudaMemcpyAsync(&h, s->net.err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        if (h) {
            CK(cudaMemsetAsync(s->net.err, 0, sizeof(int), s->stream));
            s->net_ready = false;
            destroy_graph(s);
            return fail(FS_ERR_TIMEOUT, "learned correction: a tensor-core wait gave up; the network is disabled "
                                        "until fs_set_network");
        }
    }
    // the tiled Gauss-Seidel solves' grid barriers (control block 0), once per step
    if (s->cfg.method == FS_METHOD_GAUSS_SEIDEL && s->rows > gs_max_size() && s->stats.steps > 0 &&
        s->steps_reported != s->stats.steps) {
        s->steps_reported = s->stats.steps;
        SolveCtrl c[2];
        int rc = read_solve_ctrl(s, c);
        if (rc != FS_OK) return rc;
        if (c[0].error) return fail(FS_ERR_TIMEOUT, "Gauss-Seidel solve: a grid barrier timed out");
    }
    // the residual solves' outcome is reported once per step: later syncs without a new
    // step do not report it again
    if (s->cfg.pressure_tolerance > 0.f && s->stats.steps > 0 && s->steps_reported != s->stats.steps) {
        s->steps_reported = s->stats.steps;
        SolveCtrl c[2];
        int rc = read_solve_ctrl(s, c);
        if (rc != FS_OK) return rc;
        for (int k = 0; k < 2; ++k) {
            if (c[k].error) return fail(FS_ERR_TIMEOUT, "pressure solve: a grid barrier timed out");
            if (!c[k].converged)
                return fail(FS_ERR_NOT_CONVERGED, "pressure solve: iteration cap reached before the residual target");
        }
    }
    return FS_OK;
}

int copy_in(fs_solver* s, float* dst, const float* host) {
    CK(cudaMemcpy2DAsync(dst, s->pitch * sizeof(float), host, s->cols * sizeof(float), s->cols * sizeof(float),
                         s->rows, cudaMemcpyHostToDevice, s->stream));
    return FS_OK;
}

int copy_out(fs_solver* s, float* host, const float* src, cudaStream_t st) {
    CK(cudaMemcpy2DAsync(host, s->cols * sizeof(float), src, s->pitch * sizeof(float), s->cols * sizeof(float),
                         s->rows, cudaMemcpyDeviceToHost, st));
    return FS_OK;
}
int copy_out(fs_solver* s, float* host, const float* src) { return copy_out(s, host, src, s->stream); }

// Dense (rows x cols) staging buffers -> pitched fields, up to six at once (one per
// blockIdx.y): host uploads go to contiguous scratch first because contiguous
// host-to-device copies run ~35 % faster than row-by-row 2D copies into the pitched
// layout.
struct Repack6 {
    const float* src[6];
    float* dst[6];
};

__global__ void repack_kernel(const Repack6 R, int rows, int cols, int pitch) {
    const long n = (long)rows * cols;
    const float* __restrict__ src = R.src[blockIdx.y];
    float* __restrict__ dst = R.dst[blockIdx.y];
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const long i = e / cols, j = e - i * cols;
        dst[i * pitch + j] = src[e];
    }
}

int copy_dd(fs_solver* s, float* dst, const float* src) {
    if (dst == src) return FS_OK;
    CK(cudaMemcpyAsync(dst, src, s->field_floats * sizeof(float), cudaMemcpyDeviceToDevice, s->stream));
    return FS_OK;
}

}  // namespace

namespace {

// One source event, simulation.cpp:44-51: source(i, j) += value * width * height with
// width = cols and height = rows converted to float, multiplied left to right.
__device__ void apply_source_event(const fs_source_event& ev, float* sd, float* su, float* sv, int rows, int cols,
                                   int pitch) {
    if (ev.i < 0 || ev.i >= rows || ev.j < 0 || ev.j >= cols) return;
    const size_t o = (size_t)ev.i * pitch + ev.j;
    const float w = (float)cols, h = (float)rows;
    if (ev.kind == FS_SOURCE_DENSITY) {
        sd[o] = __fadd_rn(sd[o], __fmul_rn(__fmul_rn(ev.value, w), h));
    } else {
        su[o] = __fadd_rn(su[o], __fmul_rn(__fmul_rn(ev.value, w), h));
        sv[o] = __fadd_rn(sv[o], __fmul_rn(__fmul_rn(ev.value2, w), h));
    }
}

// Events are applied by one thread in array order: the additions to a cell happen in
// the order the reference's calls would make them.
__global__ void source_events_kernel(const fs_source_event* __restrict__ ev, int begin, int end, float* sd, float* su,
                                     float* sv, int rows, int cols, int pitch) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int k = begin; k < end; ++k) apply_source_event(ev[k], sd, su, sv, rows, cols, pitch);
}

__global__ void source_event_kernel(fs_source_event ev, float* sd, float* su, float* sv, int rows, int cols,
                                    int pitch) {
    if (blockIdx.x == 0 && threadIdx.x == 0) apply_source_event(ev, sd, su, sv, rows, cols, pitch);
}

int add_source(fs_solver* s, const fs_source_event& ev) {
    if (ev.i < 0 || ev.i >= s->rows || ev.j < 0 || ev.j >= s->cols)
        return fail(FS_ERR_ARG, "source cell outside the grid");
    DeviceGuard g(s->device);
    source_event_kernel<<<1, 32, 0, s->stream>>>(ev, s->src[F_D], s->src[F_U], s->src[F_V], s->rows, s->cols,
                                                 s->pitch);
    CK(cudaGetLastError());
    s->stats.kernel_launches++;
    return FS_OK;
}

int clear_sources(fs_solver* s) {
    for (int f = 0; f < 3; ++f) CK(cudaMemsetAsync(s->src[f], 0, s->field_floats * sizeof(float), s->stream));
    return FS_OK;
}

}  // namespace

extern "C" {

const char* fs_version(void) { return "fluid2d_gb300 " FS_VERSION " sm_103a"; }

const char* fs_last_error(void) { return g_err.c_str(); }

int fs_config_init(fs_config* cfg, int rows, int cols) {
    if (!cfg) return fail(FS_ERR_ARG, "fs_config_init: null config");
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->rows = rows;
    cfg->cols = cols;
    cfg->diffuse_iterations = 15;
    cfg->pressure_iterations = 20;
    cfg->smooth = 1;
    cfg->sweeps_per_pass = 0;
    cfg->tile_rows = 0;
    cfg->use_graph = 1;
    cfg->device = -1;
    cfg->warm_start = FS_WARM_ZERO;
    cfg->pressure_tolerance = 0.f;
    cfg->pressure_max_iterations = 0;
    cfg->check_finite = 1;
    cfg->learned_defect = 1;
    return FS_OK;
}

int fs_create(const fs_config* cfg, fs_solver** out) {
    if (!cfg || !out) return fail(FS_ERR_ARG, "fs_create: null argument");
    *out = nullptr;
    if (cfg->rows < 3 || cfg->cols < 3) return fail(FS_ERR_ARG, "fs_create: rows and cols must be >= 3");
    if ((long long)cfg->rows * cfg->cols > (1LL << 31)) return fail(FS_ERR_ARG, "fs_create: grid too large");
    if (cfg->diffuse_iterations < 0 || cfg->pressure_iterations < 0)
        return fail(FS_ERR_ARG, "fs_create: negative iteration count");
    if (cfg->warm_start != FS_WARM_ZERO && cfg->warm_start != FS_WARM_PREVIOUS && cfg->warm_start != FS_WARM_LEARNED)
        return fail(FS_ERR_ARG, "fs_create: unknown warm_start mode");
    if (cfg->warm_start == FS_WARM_LEARNED && (cfg->rows != cfg->cols || (cfg->rows - 2) % FS_NET_GRID != 0))
        return fail(FS_ERR_ARG, "fs_create: the learned warm start needs a square grid with interior % 32 == 0");
    if (cfg->learned_grid != 0 && cfg->learned_grid != FS_NET_GRID && cfg->learned_grid != FS_NET_GRID_MAX)
        return fail(FS_ERR_ARG, "fs_create: learned_grid must be 0, 32 or 64");
    if (cfg->warm_start == FS_WARM_LEARNED && cfg->learned_grid > 0 && (cfg->rows - 2) % cfg->learned_grid != 0)
        return fail(FS_ERR_ARG, "fs_create: the interior must be a multiple of learned_grid");
    if (cfg->tile_rows != 0 && cfg->tile_rows != 64 && cfg->tile_rows != 128)
        return fail(FS_ERR_ARG, "fs_create: tile_rows must be 0, 64 or 128");
    if (cfg->pressure_tolerance < 0.f || cfg->pressure_tolerance != cfg->pressure_tolerance)
        return fail(FS_ERR_ARG, "fs_create: pressure_tolerance must be >= 0");
    if (cfg->pressure_tolerance > 0.f && cfg->pressure_max_iterations < 1)
        return fail(FS_ERR_ARG, "fs_create: pressure_max_iterations must be >= 1 with a residual target");
    if (cfg->method != FS_METHOD_JACOBI && cfg->method != FS_METHOD_GAUSS_SEIDEL)
        return fail(FS_ERR_ARG, "fs_create: unknown method");
    if (cfg->method == FS_METHOD_GAUSS_SEIDEL) {
        // the host solver's grid is square (its cols() returns rows, src/grid.hpp:20-22),
        // its pressure starts from zero and its sweep counts are fixed
        if (cfg->rows != cfg->cols)
            return fail(FS_ERR_ARG, "fs_create: the Gauss-Seidel method needs a square grid");
        if (cfg->warm_start != FS_WARM_ZERO || cfg->pressure_tolerance > 0.f || cfg->capture)
            return fail(FS_ERR_ARG,
                        "fs_create: the Gauss-Seidel method takes no warm start, residual target or capture");
    }

    fs_solver* s = new fs_solver();
    s->cfg = *cfg;
    int dev = cfg->device;
    if (dev < 0) {
        if (cudaGetDevice(&dev) != cudaSuccess) {
            delete s;
            return fail(FS_ERR_CUDA, "fs_create: no CUDA device");
        }
    }
    s->device = dev;
    DeviceGuard g(dev);
    s->rows = cfg->rows;
    s->cols = cfg->cols;
    s->pitch = (cfg->cols + 31) / 32 * 32;
    s->field_floats = (size_t)s->rows * s->pitch;
    s->tile_rows = cfg->tile_rows ? cfg->tile_rows : 64;
    const int maxk = stencil_max_halo(s->tile_rows) - 1;
    s->sweeps = cfg->sweeps_per_pass > 0 ? std::min(cfg->sweeps_per_pass, maxk) : default_sweeps(cfg, dev, maxk);
    s->density_branch = density_branch_pays(s, dev);

    if (cfg->method == FS_METHOD_GAUSS_SEIDEL && cfg->rows > gs_tiled_max_size()) {
        delete s;
        return fail(FS_ERR_ARG, "fs_create: grid too large for the Gauss-Seidel method (fs_gauss_seidel_max_size)");
    }
    cudaError_t e = stencil_prepare();
    if (e == cudaSuccess) e = pressure_solve_max_blocks(s->tile_rows, &s->solve_blocks);
    if (e == cudaSuccess && cfg->method == FS_METHOD_GAUSS_SEIDEL) e = gs_prepare();
    if (e != cudaSuccess) {
        delete s;
        return cuda_fail(e, "fs_create: stencil kernel set-up");
    }
    const bool learned = cfg->warm_start == FS_WARM_LEARNED;
    const int nfields = 6 + 9 + 6 + 2 + (cfg->capture ? 4 : 0) + (learned ? 4 : 0);
    // tail: flags (256 B), two solve control blocks, two partial-sum arrays
    const size_t part_doubles = 4 * (size_t)std::max(1, s->solve_blocks);
    const size_t tail = 256 + 2 * 256 + 2 * part_doubles * sizeof(double);
    const size_t slab_bytes = (size_t)nfields * s->field_floats * sizeof(float) + tail;
    e = cudaMalloc(&s->slab, slab_bytes);
    if (e != cudaSuccess) {
        delete s;
        return cuda_fail(e, "fs_create: cudaMalloc");
    }
    float* p = s->slab;
    auto take = [&]() {
        float* r = p;
        p += s->field_floats;
        return r;
    };
    for (int f = 0; f < 3; ++f) s->st[f] = take();
    for (int f = 0; f < 3; ++f) s->src[f] = take();
    for (int f = 0; f < 3; ++f) {
        s->x0[f] = take();
        s->pp[f][0] = take();
        s->pp[f][1] = take();
    }
    s->acc = take();
    s->div = take();
    s->p[0] = take();
    s->p[1] = take();
    s->vel1[0] = take();
    s->vel1[1] = take();
    s->pwarm[0] = take();
    s->pwarm[1] = take();
    if (cfg->capture) {
        for (int k = 0; k < 2; ++k) {
            s->cap_div[k] = take();
            s->cap_start[k] = take();
        }
    }
    if (learned) {
        s->pguess = take();
        s->plo = take();
        s->rhs = take();
        s->ecur = take();
    }
    char* tailp = reinterpret_cast<char*>(p);
    s->flags = reinterpret_cast<int*>(tailp);
    s->ctrl = reinterpret_cast<SolveCtrl*>(tailp + 256);
    s->partials[0] = reinterpret_cast<double*>(tailp + 256 + 2 * 256);
    s->partials[1] = s->partials[0] + part_doubles;
    int rc = FS_OK;
    if ((e = cudaMemset(s->slab, 0, slab_bytes)) != cudaSuccess)
        rc = cuda_fail(e, "fs_create: cudaMemset");
    else if ((e = create_streams(s)) != cudaSuccess ||
             (e = cudaEventCreateWithFlags(&s->side_ev[0], cudaEventDisableTiming)) != cudaSuccess ||
             (e = cudaEventCreateWithFlags(&s->side_ev[1], cudaEventDisableTiming)) != cudaSuccess)
        rc = cuda_fail(e, "fs_create: cudaStreamCreate");
    if (rc == FS_OK && learned) {
        // coarse grid: learned_grid, else 32 (a finer 64 grid resolves more modes, but the
        // network and the coarse smoothing both capture the smooth ones less well there)
        s->net.G = cfg->learned_grid > 0 ? cfg->learned_grid : FS_NET_GRID;
        const int G = s->net.G;
        // the finer coarse level: 2G when the interior allows blocks of 16 cells or more
        const int N = cfg->rows - 2;
        s->net.G2 = (2 * G <= kNetGMax && N % (2 * G) == 0 && N / (2 * G) >= 16) ? 2 * G : 0;
        const int G2 = s->net.G2;
        size_t acts = 0;
        for (int k = 0; k < kNetActs; ++k) acts += net_act_pixels(k, G) * kNetC;
        const size_t bytes = (size_t)FS_NET_PARAMS * 4 + 8 * 9216 * 2 + acts * 2 + (size_t)G * G * kNetC * 4 +
                             256 * 4 + 2 * (size_t)G * G * 4 + (size_t)G * G * kNetC * 4 +
                             (size_t)G2 * G2 * 4 + 2 * (size_t)G2 * G2 * kNetC * 4;
        if ((e = cudaMalloc(&s->net.mem, bytes)) != cudaSuccess || (e = cudaMemset(s->net.mem, 0, bytes)) != cudaSuccess) {
            rc = cuda_fail(e, "fs_create: network buffers");
        } else {
            char* q = static_cast<char*>(s->net.mem);
            s->net.params = reinterpret_cast<float*>(q);
            q += (size_t)FS_NET_PARAMS * 4;
            s->net.wpk = reinterpret_cast<__nv_bfloat16*>(q);
            q += 8 * 9216 * 2;
            s->net.act = reinterpret_cast<__nv_bfloat16*>(q);
            q += acts * 2;
            s->net.y = reinterpret_cast<float*>(q);
            q += (size_t)G * G * kNetC * 4;
            s->net.res = reinterpret_cast<double*>(q);                          // 4 doubles
            s->net.counters = reinterpret_cast<unsigned long long*>(q + 32);    // 2
            s->net.scale = reinterpret_cast<float*>(q + 48);
            s->net.err = reinterpret_cast<int*>(q + 52);
            s->net.scale2 = reinterpret_cast<float*>(q + 56);
            s->net.one = reinterpret_cast<float*>(q + 60);
            s->net.bs = reinterpret_cast<float*>(q + 256 * 4);
            s->net.yc = s->net.bs + 2 * (size_t)G * G;
            float* tail = s->net.yc + (size_t)G * G * kNetC;
            if (G2) {
                s->net.bs2 = tail;
                s->net.e2a = s->net.bs2 + (size_t)G2 * G2;
                s->net.e2b = s->net.e2a + (size_t)G2 * G2 * kNetC;
            }
            const float one = 1.f;
            if ((e = cudaMemcpy(s->net.one, &one, sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
                rc = cuda_fail(e, "fs_create: network constants");
        }
    }
    // a control block and, behind it, the two FP64 residual sums of a defect-correction cycle
    if (rc == FS_OK && learned && (e = cudaMallocHost(&s->host_ctrl, 2 * sizeof(SolveCtrl))) != cudaSuccess)
        rc = cuda_fail(e, "fs_create: pinned control block");
    if (rc != FS_OK) {
        if (s->host_ctrl) cudaFreeHost(s->host_ctrl);
        if (s->net.mem) cudaFree(s->net.mem);
        if (s->stream) cudaStreamDestroy(s->stream);
        cudaFree(s->slab);
        delete s;
        return rc;
    }
    s->stats.sweeps_per_pass = s->sweeps;
    s->stats.tile_rows = s->tile_rows;
    *out = s;
    return FS_OK;
}

int fs_gauss_seidel_max_size(int* n) {
    if (!n) return fail(FS_ERR_ARG, "fs_gauss_seidel_max_size: null argument");
    *n = gs_max_size() > 0 ? gs_tiled_max_size() : 0;
    return *n > 0 ? FS_OK : fail(FS_ERR_CUDA, "fs_gauss_seidel_max_size: no CUDA device");
}

int fs_destroy(fs_solver* s) {
    if (!s) return FS_OK;
    DeviceGuard g(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (cudaStream_t x : s->xfer)
        if (x) {
            cudaStreamSynchronize(x);
            cudaStreamDestroy(x);
        }
    for (cudaEvent_t e : s->xev)
        if (e) cudaEventDestroy(e);
    if (s->side) {
        cudaStreamSynchronize(s->side);
        cudaStreamDestroy(s->side);
    }
    for (cudaEvent_t e : s->side_ev)
        if (e) cudaEventDestroy(e);
    destroy_graph(s);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->net.mem) cudaFree(s->net.mem);
    if (s->host_ctrl) cudaFreeHost(s->host_ctrl);
    if (s->d_events) cudaFree(s->d_events);
    cudaFree(s->slab);
    delete s;
    return FS_OK;
}

int fs_upload(fs_solver* s, const float* d, const float* u, const float* v) {
    if (!s || !d || !u || !v) return fail(FS_ERR_ARG, "fs_upload: null argument");
    DeviceGuard g(s->device);
    int rc;
    if ((rc = copy_in(s, s->st[F_D], d)) || (rc = copy_in(s, s->st[F_U], u)) || (rc = copy_in(s, s->st[F_V], v)))
        return rc;
    s->warm_valid = false;
    return FS_OK;
}

int fs_upload_sources(fs_solver* s, const float* ds, const float* us, const float* vs) {
    if (!s || !ds || !us || !vs) return fail(FS_ERR_ARG, "fs_upload_sources: null argument");
    DeviceGuard g(s->device);
    int rc;
    if ((rc = copy_in(s, s->src[F_D], ds)) || (rc = copy_in(s, s->src[F_U], us)) ||
        (rc = copy_in(s, s->src[F_V], vs)))
        return rc;
    return FS_OK;
}

int fs_download(fs_solver* s, float* d, float* u, float* v) {
    if (!s || !d || !u || !v) return fail(FS_ERR_ARG, "fs_download: null argument");
    DeviceGuard g(s->device);
    int rc;
    if ((rc = copy_out(s, d, s->st[F_D])) || (rc = copy_out(s, u, s->st[F_U])) || (rc = copy_out(s, v, s->st[F_V])))
        return rc;
    return FS_OK;
}

int fs_step(fs_solver* s, float diffusion_rate, float viscosity, float dt, int nsteps) {
    if (!s || nsteps < 0) return fail(FS_ERR_ARG, "fs_step: bad argument");
    DeviceGuard g(s->device);
    return run_steps(s, diffusion_rate, viscosity, dt, nsteps);
}

int fs_sync(fs_solver* s) {
    if (!s) return fail(FS_ERR_ARG, "fs_sync: null handle");
    DeviceGuard g(s->device);
    CK(cudaStreamSynchronize(s->stream));
    return check_flags(s);
}

int fs_set_barrier_poll_limit(fs_solver* s, unsigned polls) {
    if (!s) return fail(FS_ERR_ARG, "fs_set_barrier_poll_limit: null handle");
    DeviceGuard g(s->device);
    // a device word read by every residual solve at launch, so captured step graphs see it too
    CK(cudaMemcpyAsync(s->flags + 1, &polls, sizeof(unsigned), cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FS_OK;
}

// Grids of at least this many cells take the overlapped host step below. On smaller
// grids the copies are shorter than what the overlap costs (an eager step in place of one
// graph launch, and the diffusion split into two launches).
#ifndef FS_OVERLAP_MIN_CELLS
#define FS_OVERLAP_MIN_CELLS (1L << 20)
#endif

namespace {

int launch_repack(fs_solver* s, float* const* stage, float* const* dst, int count, cudaStream_t st = nullptr) {
    Repack6 R{};
    for (int k = 0; k < count; ++k) {
        R.src[k] = stage[k];
        R.dst[k] = dst[k];
    }
    repack_kernel<<<dim3(152 * 2, count), 256, 0, st ? st : s->stream>>>(R, s->rows, s->cols, s->pitch);
    CK(cudaGetLastError());
    return FS_OK;
}

// One Jacobi step on host grids with the copies overlapped: the six grids go up as three
// (field, source) pairs and each field diffuses while the next pair is on its way; the
// new density goes down while the velocity is projected and advected. Each field sees
// the same kernels as in enqueue_step, so the results are those of upload + step +
// download. host: density, u, v, density source, u source, v source; out: density, u, v.
int solve_host_overlapped(fs_solver* s, const float* const host[6], float* const out[3], float diff, float visc,
                          float dt) {
    if (!s->xfer[0]) {
        for (cudaStream_t& x : s->xfer) CK(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
        for (cudaEvent_t& e : s->xev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    cudaStream_t up = s->xfer[0], down = s->xfer[1];
    const size_t bytes = (size_t)s->rows * s->cols * sizeof(float);
    // staging: scratch that the step overwrites after reading it (diffusion x0 and the
    // first ping-pong buffer of each field)
    float* stage[6] = {s->x0[F_D], s->pp[F_D][0], s->x0[F_U], s->x0[F_V], s->pp[F_U][0], s->pp[F_V][0]};
    const float* from[6] = {host[0], host[3], host[1], host[2], host[4], host[5]};
    float* dst[6] = {s->st[F_D], s->src[F_D], s->st[F_U], s->st[F_V], s->src[F_U], s->src[F_V]};
    // uploads begin after the handle's earlier work, which may still read the scratch
    CK(cudaEventRecord(s->xev[0], s->stream));
    CK(cudaStreamWaitEvent(up, s->xev[0], 0));
    // Three pairs go up one after another — density and its source, then u and its source,
    // then v and its source — and each field diffuses as soon as its pair has landed, so
    // the GPU works while the rest is still on the link (a one-field diffusion takes about
    // as long as the next pair's upload). The density's advection, which needs the step's
    // initial u and v, runs on the side stream beside the first projection.
    const int pairs[3][2] = {{0, 1}, {2, 4}, {3, 5}};  // stage indices: field, source
    const int fields[3] = {F_D, F_U, F_V};
    const float rates[3] = {diff, visc, visc};
    float* dif[3] = {};
    Counter cnt;
    int rc;
    for (int q = 0; q < 3; ++q) {
        for (int k : pairs[q]) CK(cudaMemcpyAsync(stage[k], from[k], bytes, cudaMemcpyHostToDevice, up));
        CK(cudaEventRecord(s->xev[1 + q], up));
        CK(cudaStreamWaitEvent(s->stream, s->xev[1 + q], 0));
        float* const st2[2] = {stage[pairs[q][0]], stage[pairs[q][1]]};
        float* const ds2[2] = {dst[pairs[q][0]], dst[pairs[q][1]]};
        if ((rc = launch_repack(s, st2, ds2, 2)) != FS_OK) return rc;
        if ((rc = enqueue_diffuse(s, &fields[q], 1, &rates[q], dt, &dif[q], cnt)) != FS_OK) return rc;
    }
    if ((rc = fork_density(s, dif[0], diff, dt, false, cnt)) != FS_OK) return rc;
    CK(cudaEventRecord(s->xev[4], s->side));
    float* dif_uv[2] = {dif[1], dif[2]};
    if ((rc = enqueue_velocity_tail(s, dif_uv[0], dif_uv[1], dt, cnt)) != FS_OK) return rc;
    // the density download is issued after the velocity work so that a pageable
    // (host-blocking) copy still overlaps it
    CK(cudaStreamWaitEvent(down, s->xev[4], 0));
    if ((rc = copy_out(s, out[0], s->st[F_D], down)) != FS_OK) return rc;
    CK(cudaEventRecord(s->xev[5], down));
    if ((rc = copy_out(s, out[1], s->st[F_U])) || (rc = copy_out(s, out[2], s->st[F_V]))) return rc;
    CK(cudaStreamWaitEvent(s->stream, s->xev[5], 0));
    cnt.launches += 3;  // the repacks
    s->launches_per_step = cnt.launches;
    s->passes_per_step = cnt.passes;
    s->stats.kernel_launches += cnt.launches;
    s->warm_valid = true;
    s->stats.steps++;
    return FS_OK;
}

}  // namespace

namespace {

// One step on host grids without overlap (small grids): stage the six inputs densely in
// scratch fields the step overwrites anyway, spread them into the pitched state and
// source fields with one kernel, step (one graph launch), copy the state out.
int solve_host_serial(fs_solver* s, const float* const host[6], float* const out[3], float diff, float visc,
                      float dt) {
    float* stage[6] = {s->x0[0], s->x0[1], s->x0[2], s->pp[0][0], s->pp[1][0], s->pp[2][0]};
    Repack6 R;
    const size_t bytes = (size_t)s->rows * s->cols * sizeof(float);
    for (int k = 0; k < 6; ++k) {
        CK(cudaMemcpyAsync(stage[k], host[k], bytes, cudaMemcpyHostToDevice, s->stream));
        R.src[k] = stage[k];
    }
    R.dst[0] = s->st[F_D];
    R.dst[1] = s->st[F_U];
    R.dst[2] = s->st[F_V];
    R.dst[3] = s->src[F_D];
    R.dst[4] = s->src[F_U];
    R.dst[5] = s->src[F_V];
    repack_kernel<<<dim3(152 * 2, 6), 256, 0, s->stream>>>(R, s->rows, s->cols, s->pitch);
    CK(cudaGetLastError());
    s->stats.kernel_launches++;
    int rc;
    if ((rc = run_steps(s, diff, visc, dt, 1)) != FS_OK) return rc;
    if ((rc = copy_out(s, out[0], s->st[F_D])) || (rc = copy_out(s, out[1], s->st[F_U])) ||
        (rc = copy_out(s, out[2], s->st[F_V])))
        return rc;
    return FS_OK;
}

}  // namespace

int fs_solve_host(fs_solver* s, float* density, const float* density_source, float diffusion_rate, float* u,
                  float* v, const float* u_source, const float* v_source, float viscosity, float dt) {
    if (!s || !density || !density_source || !u || !v || !u_source || !v_source)
        return fail(FS_ERR_ARG, "fs_solve_host: null argument");
    DeviceGuard g(s->device);
    const float* host[6] = {density, u, v, density_source, u_source, v_source};
    float* const out[3] = {density, u, v};
    const bool overlap = s->cfg.method == FS_METHOD_JACOBI && (long)s->rows * s->cols >= FS_OVERLAP_MIN_CELLS;
    const int rc = overlap ? solve_host_overlapped(s, host, out, diffusion_rate, viscosity, dt)
                           : solve_host_serial(s, host, out, diffusion_rate, viscosity, dt);
    if (rc != FS_OK) {
        // copies from or into the caller's buffers may still be queued on any of the
        // handle's streams: let them finish before the caller gets control back
        for (cudaStream_t x : {s->xfer[0], s->xfer[1], s->side, s->stream})
            if (x) cudaStreamSynchronize(x);
        return rc;
    }
    CK(cudaStreamSynchronize(s->stream));
    return check_flags(s);
}

int fs_add_density_source(fs_solver* s, int i, int j, float value) {
    if (!s) return fail(FS_ERR_ARG, "fs_add_density_source: null handle");
    fs_source_event ev{0, FS_SOURCE_DENSITY, i, j, value, 0.f};
    return add_source(s, ev);
}

int fs_add_velocity_source(fs_solver* s, int i, int j, float horizontal, float vertical) {
    if (!s) return fail(FS_ERR_ARG, "fs_add_velocity_source: null handle");
    fs_source_event ev{0, FS_SOURCE_VELOCITY, i, j, horizontal, vertical};
    return add_source(s, ev);
}

int fs_update(fs_solver* s, float diffusion_rate, float viscosity, float dt) {
    if (!s) return fail(FS_ERR_ARG, "fs_update: null handle");
    DeviceGuard g(s->device);
    int rc = run_steps(s, diffusion_rate, viscosity, dt, 1);
    return rc != FS_OK ? rc : clear_sources(s);
}

int fs_run_script(fs_solver* s, const fs_source_event* events, int count, int nsteps, float diffusion_rate,
                  float viscosity, float dt) {
    if (!s || count < 0 || nsteps < 0 || (count > 0 && !events)) return fail(FS_ERR_ARG, "fs_run_script: bad argument");
    for (int k = 0; k < count; ++k) {
        const fs_source_event& e = events[k];
        if (e.step < 0 || e.step >= nsteps || (k > 0 && e.step < events[k - 1].step))
            return fail(FS_ERR_ARG, "fs_run_script: events must be sorted by step, within [0, nsteps)");
        if ((e.kind != FS_SOURCE_DENSITY && e.kind != FS_SOURCE_VELOCITY) || e.i < 0 || e.i >= s->rows || e.j < 0 ||
            e.j >= s->cols)
            return fail(FS_ERR_ARG, "fs_run_script: bad event kind or cell");
    }
    DeviceGuard g(s->device);
    if (count > s->d_events_cap) {
        CK(cudaStreamSynchronize(s->stream));
        if (s->d_events) cudaFree(s->d_events);
        s->d_events = nullptr;
        s->d_events_cap = 0;
        cudaError_t e = cudaMalloc(&s->d_events, (size_t)count * sizeof(fs_source_event));
        if (e != cudaSuccess) return cuda_fail(e, "fs_run_script: cudaMalloc");
        s->d_events_cap = count;
    }
    if (count > 0) {
        // the stream may still read an earlier script: wait before overwriting it
        CK(cudaStreamSynchronize(s->stream));
        CK(cudaMemcpy(s->d_events, events, (size_t)count * sizeof(fs_source_event), cudaMemcpyHostToDevice));
    }
    int begin = 0;
    for (int k = 0; k < nsteps; ++k) {
        int end = begin;
        while (end < count && events[end].step == k) ++end;
        if (end > begin) {
            source_events_kernel<<<1, 32, 0, s->stream>>>(s->d_events, begin, end, s->src[F_D], s->src[F_U],
                                                          s->src[F_V], s->rows, s->cols, s->pitch);
            CK(cudaGetLastError());
            s->stats.kernel_launches++;
        }
        begin = end;
        int rc = run_steps(s, diffusion_rate, viscosity, dt, 1);
        if (rc != FS_OK) return rc;
        if ((rc = clear_sources(s)) != FS_OK) return rc;
    }
    return FS_OK;
}

int fs_stage(fs_solver* s, int stage, float rate, float dt) {
    if (!s) return fail(FS_ERR_ARG, "fs_stage: null handle");
    if (s->cfg.method != FS_METHOD_JACOBI) return fail(FS_ERR_STATE, "fs_stage: Jacobi method only");
    DeviceGuard g(s->device);
    Counter cnt;
    int rc = FS_OK;
    switch (stage) {
        case FS_STAGE_DIFFUSE_DENSITY: {
            const int f[1] = {F_D};
            const float r[1] = {rate};
            float* out[1];
            if ((rc = enqueue_diffuse(s, f, 1, r, dt, out, cnt)) == FS_OK) rc = copy_dd(s, s->st[F_D], out[0]);
            break;
        }
        case FS_STAGE_DIFFUSE_VELOCITY: {
            const int f[2] = {F_U, F_V};
            const float r[2] = {rate, rate};
            float* out[2];
            if ((rc = enqueue_diffuse(s, f, 2, r, dt, out, cnt)) == FS_OK &&
                (rc = copy_dd(s, s->st[F_U], out[0])) == FS_OK)
                rc = copy_dd(s, s->st[F_V], out[1]);
            break;
        }
        case FS_STAGE_ADVECT_DENSITY:
            rc = enqueue_advect_density(s, s->st[F_D], s->st[F_D], s->st[F_U], s->st[F_V], dt, cnt, s->stream);
            break;
        case FS_STAGE_PROJECT:
            if ((rc = enqueue_project(s, s->st[F_U], s->st[F_V], s->vel1[0], s->vel1[1], 0, cnt)) == FS_OK &&
                (rc = copy_dd(s, s->st[F_U], s->vel1[0])) == FS_OK)
                rc = copy_dd(s, s->st[F_V], s->vel1[1]);
            break;
        case FS_STAGE_ADVECT_VELOCITY: {
            cudaError_t e = launch_advect_velocity(s->st[F_U], s->st[F_V], s->vel1[0], s->vel1[1], advect_args(s, dt),
                                                   s->stream);
            if (e != cudaSuccess) return cuda_fail(e, "advect_velocity");
            cnt.launches++;
            if ((rc = copy_dd(s, s->st[F_U], s->vel1[0])) == FS_OK) rc = copy_dd(s, s->st[F_V], s->vel1[1]);
            break;
        }
        default:
            return fail(FS_ERR_ARG, "fs_stage: unknown stage");
    }
    s->stats.kernel_launches += cnt.launches;
    return rc;
}

int fs_profile_step(fs_solver* s, float diffusion_rate, float viscosity, float dt, fs_kernel_times* out) {
    if (!s || !out) return fail(FS_ERR_ARG, "fs_profile_step: null argument");
    if (s->cfg.method != FS_METHOD_JACOBI) return fail(FS_ERR_STATE, "fs_profile_step: Jacobi method only");
    DeviceGuard g(s->device);
    std::memset(out, 0, sizeof(*out));
    s->prof = out;
    s->prof_events.clear();
    s->prof_marks.clear();
    Counter cnt;
    // The step is captured with an event-record node around every launch and replayed
    // as one graph, so its launches follow one another as in the timed graph (no host
    // launch latency between them); steps that read results on the host run eagerly.
    const bool adaptive = s->cfg.warm_start == FS_WARM_LEARNED && s->net_ready && s->cfg.pressure_tolerance > 0.f;
    int rc = FS_OK;
    cudaError_t e = cudaSuccess;
    if (!adaptive) {
        cudaGraph_t gr = nullptr;
        cudaGraphExec_t ge = nullptr;
        e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            rc = enqueue_step(s, diffusion_rate, viscosity, dt, cnt);
            e = cudaStreamEndCapture(s->stream, &gr);
        }
        if (rc == FS_OK && e == cudaSuccess) e = cudaGraphInstantiate(&ge, gr, 0);
        if (rc == FS_OK && e == cudaSuccess) e = cudaGraphLaunch(ge, s->stream);
        if (rc == FS_OK && e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (ge) cudaGraphExecDestroy(ge);
        if (gr) cudaGraphDestroy(gr);
        if (rc == FS_OK && e != cudaSuccess) rc = cuda_fail(e, "fs_profile_step: graph");
    } else {
        rc = enqueue_step(s, diffusion_rate, viscosity, dt, cnt);
    }
    s->prof = nullptr;
    e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->side);
    if (rc == FS_OK && e != cudaSuccess) rc = cuda_fail(e, "fs_profile_step: sync");
    if (rc == FS_OK) {
        for (size_t k = 0; k < s->prof_marks.size() && 2 * k + 1 < s->prof_events.size(); ++k) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, s->prof_events[2 * k], s->prof_events[2 * k + 1]);
            const ProfMark& m = s->prof_marks[k];
            out->launches[m.kind] += 1;
            out->ms[m.kind] += ms;
            out->algorithmic_bytes[m.kind] += m.bytes;
            out->pass_bytes[m.kind] += m.pass_bytes;
            if (m.branch) {
                out->branch_launches[m.kind] += 1;
                out->branch_ms[m.kind] += ms;
            }
        }
        s->stats.kernel_launches += cnt.launches;
        s->stats.steps++;
        s->warm_valid = true;
    }
    for (cudaEvent_t ev : s->prof_events) cudaEventDestroy(ev);
    s->prof_events.clear();
    s->prof_marks.clear();
    return rc;
}

int fs_set_network(fs_solver* s, const float* params, long long count) {
    if (!s || !params) return fail(FS_ERR_ARG, "fs_set_network: null argument");
    if (count != FS_NET_PARAMS) return fail(FS_ERR_ARG, "fs_set_network: expected FS_NET_PARAMS parameters");
    if (s->cfg.warm_start != FS_WARM_LEARNED || !s->net.mem)
        return fail(FS_ERR_STATE, "fs_set_network: the handle was not created with FS_WARM_LEARNED");
    DeviceGuard g(s->device);
    CK(conv_prepare());
    CK(cudaMemcpyAsync(s->net.params, params, (size_t)count * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    for (int li = 0; li < 8; ++li) {
        int rc = fs_conv_pack_weights(s->net.params + (size_t)li * kNetLayer, s->net.wpk + (size_t)li * 9216, s->stream);
        if (rc != FS_OK) return rc;
    }
    CK(cudaStreamSynchronize(s->stream));
    s->net_ready = true;
    destroy_graph(s);  // the step plan changes
    return FS_OK;
}

int fs_capture_view(fs_solver* s, int slot, float** div, float** p_start, float** p_final) {
    if (!s || slot < 0 || slot > 1) return fail(FS_ERR_ARG, "fs_capture_view: bad argument");
    if (div) *div = s->cap_div[slot];
    if (p_start) *p_start = s->cap_start[slot];
    if (p_final) *p_final = s->cfg.warm_start != FS_WARM_ZERO ? s->pwarm[slot] : nullptr;
    if (!s->cfg.capture) return fail(FS_ERR_STATE, "fs_capture_view: the handle was created without capture");
    return FS_OK;
}

namespace {
struct CheckpointHeader {
    char magic[8];
    int32_t rows, cols, warm_valid, reserved;
    int64_t steps;
};
static_assert(sizeof(CheckpointHeader) == 32, "checkpoint header layout");
constexpr char kCkpMagic[8] = {'F', 'S', '2', 'D', 'C', 'K', 'P', '1'};
}  // namespace

int fs_checkpoint_save(fs_solver* s, const char* path) {
    if (!s || !path) return fail(FS_ERR_ARG, "fs_checkpoint_save: null argument");
    DeviceGuard g(s->device);
    const size_t n = (size_t)s->rows * s->cols;
    std::vector<float> buf(n * 8);
    float* fields[8] = {s->st[F_D], s->st[F_U], s->st[F_V], s->src[F_D], s->src[F_U], s->src[F_V], s->pwarm[0],
                        s->pwarm[1]};
    for (int k = 0; k < 8; ++k) {
        int rc = copy_out(s, buf.data() + k * n, fields[k]);
        if (rc != FS_OK) return rc;
    }
    CK(cudaStreamSynchronize(s->stream));
    CheckpointHeader h{};
    std::memcpy(h.magic, kCkpMagic, 8);
    h.rows = s->rows;
    h.cols = s->cols;
    h.warm_valid = s->warm_valid ? 1 : 0;
    h.steps = s->stats.steps;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(FS_ERR_ARG, "fs_checkpoint_save: cannot open the file");
    const bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size();
    std::fclose(f);
    return ok ? FS_OK : fail(FS_ERR_ARG, "fs_checkpoint_save: write failed");
}

int fs_checkpoint_load(fs_solver* s, const char* path) {
    if (!s || !path) return fail(FS_ERR_ARG, "fs_checkpoint_load: null argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(FS_ERR_ARG, "fs_checkpoint_load: cannot open the file");
    CheckpointHeader h{};
    const size_t n = (size_t)s->rows * s->cols;
    std::vector<float> buf(n * 8);
    bool ok = std::fread(&h, sizeof(h), 1, f) == 1 && std::memcmp(h.magic, kCkpMagic, 8) == 0 && h.rows == s->rows &&
              h.cols == s->cols && std::fread(buf.data(), sizeof(float), buf.size(), f) == buf.size();
    std::fclose(f);
    if (!ok) return fail(FS_ERR_ARG, "fs_checkpoint_load: not a checkpoint of this grid size");
    DeviceGuard g(s->device);
    float* fields[8] = {s->st[F_D], s->st[F_U], s->st[F_V], s->src[F_D], s->src[F_U], s->src[F_V], s->pwarm[0],
                        s->pwarm[1]};
    for (int k = 0; k < 8; ++k) {
        int rc = copy_in(s, fields[k], buf.data() + k * n);
        if (rc != FS_OK) return rc;
    }
    CK(cudaStreamSynchronize(s->stream));
    s->warm_valid = h.warm_valid != 0;
    s->stats.steps = h.steps;
    return FS_OK;
}

int fs_memcpy_device(void* dst, const void* src, unsigned long long bytes, void* stream) {
    if (!dst || !src) return fail(FS_ERR_ARG, "fs_memcpy_device: null pointer");
    CK(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return FS_OK;
}

int fs_get_stats(const fs_solver* s, fs_stats* out) {
    if (!s || !out) return fail(FS_ERR_ARG, "fs_get_stats: null argument");
    *out = s->stats;
    out->launches_per_step = s->launches_per_step;
    out->passes_per_step = s->passes_per_step;
    out->sweeps_per_pass = s->sweeps;
    out->tile_rows = s->tile_rows;
    out->pressure_iterations_last[0] = out->pressure_iterations_last[1] = s->cfg.pressure_iterations;
    if (s->net_ready) {
        DeviceGuard g(s->device);
        unsigned long long c[2] = {0, 0};
        CK(cudaMemcpyAsync(c, s->net.counters, sizeof(c), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        out->learned_used = (long long)c[0];
        out->learned_fallback = (long long)c[1];
    }
    if (s->cfg.pressure_tolerance > 0.f && s->stats.steps > 0) {
        DeviceGuard g(s->device);
        SolveCtrl c[2];
        int rc = read_solve_ctrl(s, c);
        if (rc != FS_OK) return rc;
        for (int k = 0; k < 2; ++k) {
            out->pressure_iterations_last[k] = c[k].passes * s->sweeps;
            out->pressure_residual_last[k] = c[k].residual;
        }
    }
    return FS_OK;
}

int fs_device_view_get(fs_solver* s, fs_device_view* out) {
    if (!s || !out) return fail(FS_ERR_ARG, "fs_device_view_get: null argument");
    out->density = s->st[F_D];
    out->u = s->st[F_U];
    out->v = s->st[F_V];
    out->density_source = s->src[F_D];
    out->u_source = s->src[F_U];
    out->v_source = s->src[F_V];
    out->rows = s->rows;
    out->cols = s->cols;
    out->pitch = s->pitch;
    out->stream = (void*)s->stream;
    return FS_OK;
}

int fs_host_alloc(void** ptr, unsigned long long bytes) {
    if (!ptr) return fail(FS_ERR_ARG, "fs_host_alloc: null argument");
    *ptr = nullptr;
    cudaError_t e = cudaMallocHost(ptr, (size_t)bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocHost");
    return FS_OK;
}

int fs_host_free(void* ptr) {
    if (!ptr) return FS_OK;
    CK(cudaFreeHost(ptr));
    return FS_OK;
}

}  // extern "C"
