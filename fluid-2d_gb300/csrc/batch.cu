// Batched stepping of many independent grids of uneven size (fs_batch_* in
// include/fluid2d_gb300.h).
//
// The reference advances one grid per fluid_solver_gpu object, one kernel per sweep
// (fluid_solver_gpu.cu:222-404). A batch here advances every grid of the batch with
// the same stage sequence as a single handle, but each sub-step is ONE launch over
// all grids: a stencil pass carries the grids' field descriptors in its launch
// parameters (tiles of all grids concatenated, one CTA per tile; a pass of more fields
// than the parameter space holds is split into launches of equal field counts), and the
// advection stages walk a device table of per-grid jobs (a block -> job map).
// The grids are dealt to a few lanes (longest-processing-time first, by cells) and each
// lane runs its own sequence of launches on its own stream, so one lane's small final
// wave overlaps another lane's work instead of idling the GPU between sub-steps. The
// whole step, lanes forked from and joined back to the batch's stream, is captured once
// as a CUDA graph. Grids share dt, the rates and the sweep counts; each grid has its own
// size, state and sources.
//
// Memory: one slab, field-major — for each of the 21 per-grid field kinds, the
// buffers of all grids follow each other — so e.g. all splat accumulators form one
// contiguous range cleared by a single memset.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "host_common.h"

using namespace fs;

namespace {

enum Kind {
    K_ST_D, K_ST_U, K_ST_V,     // state
    K_SRC_D, K_SRC_U, K_SRC_V,  // sources
    K_X0_D, K_X0_U, K_X0_V,     // diffusion x0
    K_PP_D0, K_PP_D1, K_PP_U0, K_PP_U1, K_PP_V0, K_PP_V1,  // diffusion ping-pong
    K_ACC, K_DIV, K_P0, K_P1, K_VEL_U, K_VEL_V,
    K_COUNT
};

}  // namespace

struct fs_batch {
    fs_config cfg{};
    int device = 0;
    int count = 0;
    std::vector<int> rows, cols, pitch;
    std::vector<size_t> off;  // per-grid offset (floats) inside each field-kind range
    size_t range_floats = 0;  // floats per field kind (all grids)
    float* slab = nullptr;
    int* flags = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    bool graph_valid = false;
    float g_diff = 0, g_visc = 0, g_dt = 0;
    int sweeps = 8, tile_rows = 64;
    // host-built plan: the stencil launches (their descriptors travel as parameters) and
    // the advection job tables, which are mirrored in one device buffer
    std::vector<WideLaunch> h_wide;
    std::vector<AdvectJob> h_jobs;
    std::vector<int> h_jprefix;
    std::vector<int> h_map;   // block -> job for every advection op
    struct Pass {
        size_t first;  // launches h_wide[first, first + count)
        int count;
        bool diffuse;
    };
    // one lane: its grids, its passes (diffusion, project 1, project 2) and advection
    // jobs, and the stream it runs on (lane 0: the batch's stream)
    struct Lane {
        std::vector<int> grids;
        std::vector<Pass> passes;
        // ops 0-2: splat, finish, velocity backtrace; 3, 4: the gradient pass of projection 1, 2
        size_t job_off[5] = {}, jprefix_off[5] = {}, jmap_off[5] = {};
        int job_blocks[5] = {};
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
    };
    std::vector<Lane> lanes;
    cudaEvent_t fork = nullptr;
    int n_diffuse = 0, n_project = 0;
    bool split = false;  // projections end with a separate gradient launch
    void* d_plan = nullptr;
    size_t d_plan_bytes = 0;
    AdvectJob* d_jobs = nullptr;
    int* d_jprefix = nullptr;
    int* d_map = nullptr;
    int launches_per_step = 0;
    fs_stats stats{};

    float* fld(int kind, int g) const { return slab + (size_t)kind * range_floats + off[g]; }
};

namespace {

int fail(int code, const char* msg) { return record_error(code, msg); }

constexpr int kBatchLanes = 4;

// One stencil pass over the fields fl: ceil(n / kMaxWideFields) launches with as even a
// share of the fields as possible, each field's tiles numbered from its launch's start.
fs_batch::Pass add_pass(fs_batch* b, const std::vector<StencilField>& fl, bool diffuse) {
    const int n = (int)fl.size();
    const int nl = (n + kMaxWideFields - 1) / kMaxWideFields;
    fs_batch::Pass P{b->h_wide.size(), nl, diffuse};
    int f0 = 0;
    for (int l = 0; l < nl; ++l) {
        const int cnt = n / nl + (l < n % nl ? 1 : 0);
        b->h_wide.emplace_back();
        WideLaunch& W = b->h_wide.back();
        std::memset(&W, 0, sizeof(W));
        W.nfields = cnt;
        int tiles = 0;
        for (int i = 0; i < cnt; ++i) {
            W.f[i] = fl[f0 + i];
            W.f[i].tile_begin = tiles;
            W.begin[i] = tiles;
            tiles += W.f[i].tiles_x * W.f[i].tiles_y;
        }
        W.begin[cnt] = tiles;
        f0 += cnt;
    }
    return P;
}

// Builds the launches and job tables of one step for (diff, visc, dt) and uploads the
// tables.
int build_plan(fs_batch* b, float diff, float visc, float dt) {
    b->h_wide.clear();
    b->h_jobs.clear();
    b->h_jprefix.clear();
    b->h_map.clear();
    const int K = b->sweeps;
    const std::vector<int> dplan = plan_passes(b->cfg.diffuse_iterations, K);
    const std::vector<int> pplan = plan_passes(b->cfg.pressure_iterations, K);
    b->n_diffuse = (int)dplan.size();
    b->n_project = (int)pplan.size();
    // multi-pass projections end with an ordinary pass and a separate gradient launch (the
    // fused gradient epilogue's loads and stores made the last pass ~1.6x a middle one)
    const bool split = b->n_project >= 2;
    b->split = split;
    const int dkinds[3][5] = {{K_ST_D, K_SRC_D, K_X0_D, K_PP_D0, K_PP_D1},
                              {K_ST_U, K_SRC_U, K_X0_U, K_PP_U0, K_PP_U1},
                              {K_ST_V, K_SRC_V, K_X0_V, K_PP_V0, K_PP_V1}};
    const float rates[3] = {diff, visc, visc};
    const int modes[3] = {BND_CONT, BND_OPP_H, BND_OPP_V};
    const int dlast = (b->n_diffuse - 1) & 1;  // ping-pong buffer holding the diffusion result
    for (fs_batch::Lane& L : b->lanes) {
        L.passes.clear();
        // ---- diffusion passes over the lane's grids x {d, u, v}; add_sources fused in pass 0
        for (size_t pass = 0; pass < dplan.size(); ++pass) {
            std::vector<StencilField> fl;
            for (int g : L.grids)
                for (int q = 0; q < 3; ++q) {
                    StencilField f{};
                    field_geometry(f, b->rows[g], b->cols[g], b->pitch[g], b->tile_rows, dplan[pass]);
                    realign_columns(f);
                    field_diffusion(f, b->rows[g], b->cols[g], rates[q], dt);
                    f.s_lr = bnd_sign_lr(modes[q]);
                    f.s_tb = bnd_sign_tb(modes[q]);
                    f.sweeps = dplan[pass];
                    f.dt = dt;
                    const int* k = dkinds[q];
                    f.x = pass == 0 ? b->fld(k[0], g) : b->fld(k[3 + ((pass - 1) & 1)], g);
                    f.y = b->fld(k[3 + (pass & 1)], g);
                    if (pass == 0) {
                        f.kind = PASS_DIFFUSE_FIRST;
                        f.x2 = b->fld(k[1], g);
                        f.cst_out = b->fld(k[2], g);
                    } else {
                        f.kind = PASS_DIFFUSE;
                        f.cst = b->fld(k[2], g);
                    }
                    fl.push_back(f);
                }
            L.passes.push_back(add_pass(b, fl, true));
        }
        // ---- two projections over the lane's grids (one pressure field each)
        for (int proj = 0; proj < 2; ++proj) {
            for (int pass = 0; pass < b->n_project; ++pass) {
                const bool last = pass == b->n_project - 1;
                std::vector<StencilField> fl;
                for (int g : L.grids) {
                    StencilField f{};
                    field_geometry(f, b->rows[g], b->cols[g], b->pitch[g], b->tile_rows,
                                   pplan[pass] + (last && !split ? 1 : 0));
                    realign_columns(f);
                    const float h = grid_spacing(b->rows[g], b->cols[g]);
                    f.s_lr = f.s_tb = 1.f;
                    f.sweeps = pplan[pass];
                    f.cdiv = -0.5f * h;
                    f.h = h;
                    const float* uin = proj == 0 ? b->fld(K_PP_U0 + dlast, g) : b->fld(K_VEL_U, g);
                    const float* vin = proj == 0 ? b->fld(K_PP_V0 + dlast, g) : b->fld(K_VEL_V, g);
                    if (pass == 0) {
                        f.kind = PASS_PRESSURE_FIRST;
                        f.x = uin;
                        f.x2 = vin;
                        f.cst_out = b->fld(K_DIV, g);
                    } else {
                        f.kind = PASS_PRESSURE;
                        f.x = b->fld(K_P0 + ((pass - 1) & 1), g);
                        f.cst = b->fld(K_DIV, g);
                    }
                    f.y = last && !split ? nullptr : b->fld(K_P0 + (pass & 1), g);
                    if (last && !split) {
                        f.epilogue = 1;
                        f.u_in = uin;
                        f.v_in = vin;
                        f.u_out = b->fld(K_ST_U, g);
                        f.v_out = b->fld(K_ST_V, g);
                        f.nonfinite = b->cfg.check_finite ? b->flags : nullptr;
                    }
                    fl.push_back(f);
                }
                L.passes.push_back(add_pass(b, fl, false));
            }
        }
        // ---- advection jobs: splat, finish, velocity backtrace; with multi-pass
        // projections, the gradient subtract of each projection (gradient_batch_kernel)
        for (int op = 0; op < (split ? 5 : 3); ++op) {
            L.job_off[op] = b->h_jobs.size();
            L.jprefix_off[op] = b->h_jprefix.size();
            L.jmap_off[op] = b->h_map.size();
            int blocks = 0;
            int jobs = 0;
            for (int g : L.grids) {
                AdvectJob J{};
                J.A = make_advect_args(b->rows[g], b->cols[g], b->pitch[g], dt);
                J.smooth = b->cfg.smooth;
                if (op == 0) {
                    J.in0 = b->fld(K_PP_D0 + dlast, g);
                    J.in1 = b->fld(K_ST_U, g);
                    J.in2 = b->fld(K_ST_V, g);
                    J.out0 = b->fld(K_ACC, g);
                } else if (op == 1) {
                    J.in0 = b->fld(K_ACC, g);
                    J.out0 = b->fld(K_ST_D, g);
                } else if (op == 2) {
                    J.in0 = b->fld(K_ST_U, g);
                    J.in1 = b->fld(K_ST_V, g);
                    J.out0 = b->fld(K_VEL_U, g);
                    J.out1 = b->fld(K_VEL_V, g);
                } else {
                    // the last pass's pressure; the velocity the projection started from
                    J.A.h = grid_spacing(b->rows[g], b->cols[g]);
                    J.in0 = b->fld(K_P0 + ((b->n_project - 1) & 1), g);
                    J.in1 = op == 3 ? b->fld(K_PP_U0 + dlast, g) : b->fld(K_VEL_U, g);
                    J.in2 = op == 3 ? b->fld(K_PP_V0 + dlast, g) : b->fld(K_VEL_V, g);
                    J.out0 = b->fld(K_ST_U, g);
                    J.out1 = b->fld(K_ST_V, g);
                }
                b->h_jprefix.push_back(blocks);
                const int nb = op >= 3 ? gradient_batch_blocks(b->rows[g], b->cols[g])
                                       : advect_batch_blocks(b->rows[g], b->cols[g]);
                blocks += nb;
                b->h_map.insert(b->h_map.end(), nb, jobs++);
                b->h_jobs.push_back(J);
            }
            b->h_jprefix.push_back(blocks);
            L.job_blocks[op] = blocks;
        }
    }
    // ---- upload the job tables (one buffer)
    const size_t job_bytes = b->h_jobs.size() * sizeof(AdvectJob);
    const size_t jpre_bytes = b->h_jprefix.size() * sizeof(int);
    const size_t map_bytes = b->h_map.size() * sizeof(int);
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t need = up(job_bytes) + up(jpre_bytes) + up(map_bytes);
    if (need > b->d_plan_bytes) {
        if (b->d_plan) cudaFree(b->d_plan);
        b->d_plan = nullptr;
        b->d_plan_bytes = 0;
        FS_CK(cudaMalloc(&b->d_plan, need));
        b->d_plan_bytes = need;
    }
    char* base = static_cast<char*>(b->d_plan);
    b->d_jobs = reinterpret_cast<AdvectJob*>(base);
    b->d_jprefix = reinterpret_cast<int*>(base + up(job_bytes));
    b->d_map = reinterpret_cast<int*>(base + up(job_bytes) + up(jpre_bytes));
    FS_CK(cudaMemcpyAsync(b->d_jobs, b->h_jobs.data(), job_bytes, cudaMemcpyHostToDevice, b->stream));
    FS_CK(cudaMemcpyAsync(b->d_jprefix, b->h_jprefix.data(), jpre_bytes, cudaMemcpyHostToDevice, b->stream));
    FS_CK(cudaMemcpyAsync(b->d_map, b->h_map.data(), map_bytes, cudaMemcpyHostToDevice, b->stream));
    FS_CK(cudaStreamSynchronize(b->stream));  // host vectors may change before the next upload
    return FS_OK;
}

int enqueue_pass(fs_batch* b, const fs_batch::Pass& P, cudaStream_t st, int& launches) {
    for (int i = 0; i < P.count; ++i) {
        FS_CK(launch_stencil_wide(b->h_wide[P.first + i], P.diffuse, b->tile_rows, st));
        launches++;
    }
    return FS_OK;
}

int enqueue_lane(fs_batch* b, const fs_batch::Lane& L, int& launches) {
    int rc;
    const cudaStream_t st = L.stream;
    size_t pi = 0;
    for (int k = 0; k < b->n_diffuse; ++k)
        if ((rc = enqueue_pass(b, L.passes[pi++], st, launches)) != FS_OK) return rc;
    int* nf = b->cfg.check_finite ? b->flags : nullptr;
    FS_CK(launch_advect_batch(0, b->d_jobs + L.job_off[0], b->d_jprefix + L.jprefix_off[0],
                              b->d_map + L.jmap_off[0], L.job_blocks[0], nullptr, st));
    FS_CK(launch_advect_batch(1, b->d_jobs + L.job_off[1], b->d_jprefix + L.jprefix_off[1],
                              b->d_map + L.jmap_off[1], L.job_blocks[1], nf, st));
    launches += 2;
    auto gradient = [&](int op) {
        if (!b->split) return cudaSuccess;
        launches++;
        return launch_gradient_batch(b->d_jobs + L.job_off[op], b->d_jprefix + L.jprefix_off[op],
                                     b->d_map + L.jmap_off[op], L.job_blocks[op], nf, st);
    };
    for (int k = 0; k < b->n_project; ++k)
        if ((rc = enqueue_pass(b, L.passes[pi++], st, launches)) != FS_OK) return rc;
    FS_CK(gradient(3));
    FS_CK(launch_advect_batch(2, b->d_jobs + L.job_off[2], b->d_jprefix + L.jprefix_off[2],
                              b->d_map + L.jmap_off[2], L.job_blocks[2], nullptr, st));
    launches++;
    for (int k = 0; k < b->n_project; ++k)
        if ((rc = enqueue_pass(b, L.passes[pi++], st, launches)) != FS_OK) return rc;
    FS_CK(gradient(4));
    return FS_OK;
}

// One step: clear every splat accumulator, fork the lanes from the batch's stream, run
// each lane's sequence on its stream, join them back.
int enqueue_step(fs_batch* b, int& launches) {
    int rc;
    FS_CK(cudaMemsetAsync(b->slab + (size_t)K_ACC * b->range_floats, 0, b->range_floats * sizeof(float), b->stream));
    const size_t nl = b->lanes.size();
    if (nl > 1) FS_CK(cudaEventRecord(b->fork, b->stream));
    for (size_t l = 1; l < nl; ++l) FS_CK(cudaStreamWaitEvent(b->lanes[l].stream, b->fork, 0));
    for (size_t l = 0; l < nl; ++l)
        if ((rc = enqueue_lane(b, b->lanes[l], launches)) != FS_OK) return rc;
    for (size_t l = 1; l < nl; ++l) {
        FS_CK(cudaEventRecord(b->lanes[l].done, b->lanes[l].stream));
        FS_CK(cudaStreamWaitEvent(b->stream, b->lanes[l].done, 0));
    }
    return FS_OK;
}

void drop_graph(fs_batch* b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->gexec = nullptr;
    b->graph = nullptr;
    b->graph_valid = false;
}

int check_index(const fs_batch* b, int index) {
    if (!b || index < 0 || index >= b->count) return fail(FS_ERR_ARG, "fs_batch: grid index out of range");
    return FS_OK;
}

int copy_in(fs_batch* b, int g, int kind, const float* host) {
    FS_CK(cudaMemcpy2DAsync(b->fld(kind, g), b->pitch[g] * sizeof(float), host, b->cols[g] * sizeof(float),
                            b->cols[g] * sizeof(float), b->rows[g], cudaMemcpyHostToDevice, b->stream));
    return FS_OK;
}

int copy_out(fs_batch* b, int g, int kind, float* host) {
    FS_CK(cudaMemcpy2DAsync(host, b->cols[g] * sizeof(float), b->fld(kind, g), b->pitch[g] * sizeof(float),
                            b->cols[g] * sizeof(float), b->rows[g], cudaMemcpyDeviceToHost, b->stream));
    return FS_OK;
}

}  // namespace

extern "C" {

int fs_batch_create(const fs_config* cfg, int count, const int* rows, const int* cols, fs_batch** out) {
    if (!cfg || !rows || !cols || !out || count < 1) return fail(FS_ERR_ARG, "fs_batch_create: bad argument");
    *out = nullptr;
    for (int g = 0; g < count; ++g)
        if (rows[g] < 3 || cols[g] < 3) return fail(FS_ERR_ARG, "fs_batch_create: rows and cols must be >= 3");
    if (cfg->diffuse_iterations < 0 || cfg->pressure_iterations < 0)
        return fail(FS_ERR_ARG, "fs_batch_create: negative iteration count");
    if (cfg->pressure_tolerance != 0.f || cfg->warm_start != FS_WARM_ZERO)
        return fail(FS_ERR_ARG, "fs_batch_create: batches use fixed sweep counts and zero-start pressure");
    if (cfg->tile_rows != 0 && cfg->tile_rows != 64 && cfg->tile_rows != 128)
        return fail(FS_ERR_ARG, "fs_batch_create: tile_rows must be 0, 64 or 128");
    fs_batch* b = new fs_batch();
    b->cfg = *cfg;
    int dev = cfg->device;
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) {
        delete b;
        return fail(FS_ERR_CUDA, "fs_batch_create: no CUDA device");
    }
    b->device = dev;
    DeviceScope scope(dev);
    b->count = count;
    b->tile_rows = cfg->tile_rows ? cfg->tile_rows : 64;
    const int maxk = stencil_max_halo(b->tile_rows) - 1;
    b->sweeps = cfg->sweeps_per_pass > 0 ? std::min(cfg->sweeps_per_pass, maxk) : std::min(8, maxk);
    size_t total = 0;
    for (int g = 0; g < count; ++g) {
        b->rows.push_back(rows[g]);
        b->cols.push_back(cols[g]);
        b->pitch.push_back(pitch_for(cols[g]));
        b->off.push_back(total);
        total += ((size_t)rows[g] * b->pitch[g] + 63) / 64 * 64;  // 256-byte aligned grids
    }
    b->range_floats = total;
    const size_t bytes = (size_t)K_COUNT * total * sizeof(float) + 256;
    cudaError_t e = stencil_prepare();
    if (e == cudaSuccess) e = cudaMalloc(&b->slab, bytes);
    if (e == cudaSuccess) e = cudaMemset(b->slab, 0, bytes);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        int rc = cuda_error(e, "fs_batch_create");
        if (b->stream) cudaStreamDestroy(b->stream);
        if (b->slab) cudaFree(b->slab);
        delete b;
        return rc;
    }
    b->flags = reinterpret_cast<int*>(b->slab + (size_t)K_COUNT * total);
    // lanes: grids dealt longest-first to the lane with the fewest cells so far
    const int nlanes = std::min(kBatchLanes, count);
    b->lanes.resize(nlanes);
    std::vector<int> order(count);
    for (int g = 0; g < count; ++g) order[g] = g;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return (long long)rows[x] * cols[x] > (long long)rows[y] * cols[y];
    });
    std::vector<long long> load(nlanes, 0);
    for (int g : order) {
        const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        b->lanes[l].grids.push_back(g);
        load[l] += (long long)rows[g] * cols[g];
    }
    for (auto& L : b->lanes) std::sort(L.grids.begin(), L.grids.end());
    b->lanes[0].stream = b->stream;
    int rc = FS_OK;
    for (int l = 1; l < nlanes && rc == FS_OK; ++l) {
        if ((e = cudaStreamCreateWithFlags(&b->lanes[l].stream, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&b->lanes[l].done, cudaEventDisableTiming)) != cudaSuccess)
            rc = cuda_error(e, "fs_batch_create: lane streams");
    }
    if (rc == FS_OK && nlanes > 1 && (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess)
        rc = cuda_error(e, "fs_batch_create: lane events");
    if (rc != FS_OK) {
        fs_batch_destroy(b);
        return rc;
    }
    *out = b;
    return FS_OK;
}

int fs_batch_destroy(fs_batch* b) {
    if (!b) return FS_OK;
    DeviceScope scope(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    if (b->d_plan) cudaFree(b->d_plan);
    for (size_t l = 1; l < b->lanes.size(); ++l) {
        if (b->lanes[l].stream) cudaStreamDestroy(b->lanes[l].stream);
        if (b->lanes[l].done) cudaEventDestroy(b->lanes[l].done);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->stream) cudaStreamDestroy(b->stream);
    cudaFree(b->slab);
    delete b;
    return FS_OK;
}

int fs_batch_upload(fs_batch* b, int index, const float* d, const float* u, const float* v) {
    int rc = check_index(b, index);
    if (rc != FS_OK) return rc;
    if (!d || !u || !v) return fail(FS_ERR_ARG, "fs_batch_upload: null pointer");
    DeviceScope scope(b->device);
    if ((rc = copy_in(b, index, K_ST_D, d)) || (rc = copy_in(b, index, K_ST_U, u)) ||
        (rc = copy_in(b, index, K_ST_V, v)))
        return rc;
    return FS_OK;
}

int fs_batch_upload_sources(fs_batch* b, int index, const float* ds, const float* us, const float* vs) {
    int rc = check_index(b, index);
    if (rc != FS_OK) return rc;
    if (!ds || !us || !vs) return fail(FS_ERR_ARG, "fs_batch_upload_sources: null pointer");
    DeviceScope scope(b->device);
    if ((rc = copy_in(b, index, K_SRC_D, ds)) || (rc = copy_in(b, index, K_SRC_U, us)) ||
        (rc = copy_in(b, index, K_SRC_V, vs)))
        return rc;
    return FS_OK;
}

int fs_batch_download(fs_batch* b, int index, float* d, float* u, float* v) {
    int rc = check_index(b, index);
    if (rc != FS_OK) return rc;
    if (!d || !u || !v) return fail(FS_ERR_ARG, "fs_batch_download: null pointer");
    DeviceScope scope(b->device);
    if ((rc = copy_out(b, index, K_ST_D, d)) || (rc = copy_out(b, index, K_ST_U, u)) ||
        (rc = copy_out(b, index, K_ST_V, v)))
        return rc;
    return FS_OK;
}

int fs_batch_step(fs_batch* b, float diffusion_rate, float viscosity, float dt, int nsteps) {
    if (!b || nsteps < 0) return fail(FS_ERR_ARG, "fs_batch_step: bad argument");
    DeviceScope scope(b->device);
    int rc;
    if (!b->graph_valid || diffusion_rate != b->g_diff || viscosity != b->g_visc || dt != b->g_dt) {
        drop_graph(b);
        if ((rc = build_plan(b, diffusion_rate, viscosity, dt)) != FS_OK) return rc;
        int launches = 0;
        if (b->cfg.use_graph) {
            FS_CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            rc = enqueue_step(b, launches);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(b->stream, &g);
            if (rc != FS_OK) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e != cudaSuccess) return cuda_error(e, "fs_batch_step: capture");
            b->graph = g;
            FS_CK(cudaGraphInstantiate(&b->gexec, g, 0));
        } else {
            // stencil launches + three advection launches (+ two gradient launches), per lane
            for (const fs_batch::Lane& L : b->lanes) {
                for (const fs_batch::Pass& P : L.passes) launches += P.count;
                launches += 3 + (b->split ? 2 : 0);
            }
        }
        b->launches_per_step = launches;
        b->graph_valid = true;
        b->g_diff = diffusion_rate;
        b->g_visc = viscosity;
        b->g_dt = dt;
    }
    for (int k = 0; k < nsteps; ++k) {
        if (b->cfg.use_graph) {
            FS_CK(cudaGraphLaunch(b->gexec, b->stream));
        } else {
            int launches = 0;
            if ((rc = enqueue_step(b, launches)) != FS_OK) return rc;
        }
        b->stats.kernel_launches += b->launches_per_step;
        b->stats.steps++;
    }
    return FS_OK;
}

int fs_batch_sync(fs_batch* b) {
    if (!b) return fail(FS_ERR_ARG, "fs_batch_sync: null handle");
    DeviceScope scope(b->device);
    FS_CK(cudaStreamSynchronize(b->stream));
    if (b->cfg.check_finite) {
        int h = 0;
        FS_CK(cudaMemcpy(&h, b->flags, sizeof(int), cudaMemcpyDeviceToHost));
        if (h) {
            FS_CK(cudaMemset(b->flags, 0, sizeof(int)));
            b->stats.nonfinite = 1;
            return fail(FS_ERR_NONFINITE, "a batched step produced a non-finite value");
        }
    }
    return FS_OK;
}

int fs_batch_get_stats(const fs_batch* b, fs_stats* out) {
    if (!b || !out) return fail(FS_ERR_ARG, "fs_batch_get_stats: null argument");
    *out = b->stats;
    out->launches_per_step = b->launches_per_step;
    out->passes_per_step = b->n_diffuse + 2 * b->n_project;
    out->sweeps_per_pass = b->sweeps;
    out->tile_rows = b->tile_rows;
    out->pressure_iterations_last[0] = out->pressure_iterations_last[1] = b->cfg.pressure_iterations;
    return FS_OK;
}

int fs_batch_stream(fs_batch* b, void** stream) {
    if (!b || !stream) return fail(FS_ERR_ARG, "fs_batch_stream: null argument");
    *stream = (void*)b->stream;
    return FS_OK;
}

}  // extern "C"
