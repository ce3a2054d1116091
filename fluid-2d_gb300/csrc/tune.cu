// Autotuner for the stencil tiling: picks the region height (tile_rows) and the
// temporal-blocking depth (sweeps_per_pass) for one grid shape and sweep plan, or for a
// batch of grids, by timing whole steps on the device, and caches the choice in a text
// file.
//
// No counterpart in the reference, whose launch shape is fixed (32x32 blocks,
// kernel_launcher.hpp:14-16, 28-30) and whose sweep counts are hard-coded.
//
// Cache file: one line per key,
//   <device name>|<SMs>|<rows>|<cols>|<kd>|<kp>|<tol>|<warm> <tile_rows> <sweeps> <ms>
// Later lines win, so a re-tune appends.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "host_common.h"

using namespace fs;

namespace {

std::string tune_key(const fs_config* c) {
    int dev = c->device;
    if (dev < 0) cudaGetDevice(&dev);
    cudaDeviceProp prop;
    std::memset(&prop, 0, sizeof(prop));
    cudaGetDeviceProperties(&prop, dev);
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s|%d|%d|%d|%d|%d|%g|%d", prop.name, prop.multiProcessorCount, c->rows, c->cols,
                  c->diffuse_iterations, c->pressure_iterations, (double)c->pressure_tolerance, c->warm_start);
    for (char* p = buf; *p; ++p)
        if (*p == ' ') *p = '_';
    return buf;
}

bool cache_lookup(const char* path, const std::string& key, int* tile_rows, int* sweeps, double* ms) {
    if (!path) return false;
    FILE* f = std::fopen(path, "r");
    if (!f) return false;
    char k[512];
    int tr, sw;
    double t;
    bool found = false;
    while (std::fscanf(f, "%511s %d %d %lf", k, &tr, &sw, &t) == 4) {
        if (key == k) {
            *tile_rows = tr;
            *sweeps = sw;
            *ms = t;
            found = true;
        }
    }
    std::fclose(f);
    return found;
}

void cache_store(const char* path, const std::string& key, int tile_rows, int sweeps, double ms) {
    if (!path) return;
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%s %d %d %.6f\n", key.c_str(), tile_rows, sweeps, ms);
    std::fclose(f);
}

// The state the candidates are timed on: zero density and a smooth velocity field with
// divergence everywhere, u = 0.5 sin(6 pi x) cos(4 pi y), v = 0.5 cos(4 pi x) sin(6 pi y)
// on the unit square (boundary included), so that a pressure solve to a residual target
// does the sweeps it would do on a real flow instead of converging on a zero field.
void tuning_state(int rows, int cols, std::vector<float>& d, std::vector<float>& u, std::vector<float>& v) {
    const size_t n = (size_t)rows * (size_t)cols;
    d.assign(n, 0.f);
    u.resize(n);
    v.resize(n);
    const double pi = 3.14159265358979323846;
    std::vector<double> sx6(cols), cx4(cols), cy4(rows), sy6(rows);
    for (int j = 0; j < cols; ++j) {
        const double x = (double)j / (double)(cols - 1);
        sx6[j] = std::sin(6.0 * pi * x);
        cx4[j] = std::cos(4.0 * pi * x);
    }
    for (int i = 0; i < rows; ++i) {
        const double y = (double)i / (double)(rows - 1);
        cy4[i] = std::cos(4.0 * pi * y);
        sy6[i] = std::sin(6.0 * pi * y);
    }
    for (int i = 0; i < rows; ++i)
        for (int j = 0; j < cols; ++j) {
            u[(size_t)i * cols + j] = (float)(0.5 * sx6[j] * cy4[i]);
            v[(size_t)i * cols + j] = (float)(0.5 * cx4[j] * sy6[i]);
        }
}

// Mean milliseconds per step of `cfg` on the tuning state with the given physics.
int time_config(const fs_config* cfg, float diff, float visc, float dt, int steps, const std::vector<float>& d0,
                const std::vector<float>& u0, const std::vector<float>& v0, double* ms) {
    fs_solver* s = nullptr;
    int rc = fs_create(cfg, &s);
    if (rc != FS_OK) return rc;
    rc = fs_upload(s, d0.data(), u0.data(), v0.data());
    if (rc != FS_OK) {
        fs_destroy(s);
        return rc;
    }
    fs_device_view v;
    fs_device_view_get(s, &v);
    cudaStream_t st = (cudaStream_t)v.stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    rc = fs_step(s, diff, visc, dt, 2);  // warm-up (captures the graph)
    if (rc == FS_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
        rc = record_error(FS_ERR_CUDA, "fs_autotune: cudaEventCreate");
    if (rc == FS_OK) {
        cudaEventRecord(e0, st);
        rc = fs_step(s, diff, visc, dt, steps);
        cudaEventRecord(e1, st);
    }
    if (rc == FS_OK) rc = fs_sync(s);
    if (rc == FS_OK || rc == FS_ERR_NOT_CONVERGED) {
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        *ms = t / steps;
        rc = FS_OK;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    fs_destroy(s);
    return rc;
}

}  // namespace

extern "C" int fs_autotune(fs_config* cfg, float diffusion_rate, float viscosity, float dt, int steps,
                           const char* cache_path, double* best_ms) {
    if (!cfg || steps < 1) return record_error(FS_ERR_ARG, "fs_autotune: bad argument");
    DeviceScope scope(cfg->device);
    const std::string key = tune_key(cfg);
    int tr = 0, sw = 0;
    double ms = 0.0;
    if (cache_lookup(cache_path, key, &tr, &sw, &ms)) {
        cfg->tile_rows = tr;
        cfg->sweeps_per_pass = sw;
        if (best_ms) *best_ms = ms;
        return FS_OK;
    }
    std::vector<float> d0, u0, v0;
    tuning_state(cfg->rows, cfg->cols, d0, u0, v0);
    const int heights[2] = {64, 128};
    const int depths[8] = {2, 4, 6, 8, 10, 12, 14, 16};
    double best = 1e30;
    int best_tr = 0, best_sw = 0;
    for (int h : heights) {
        for (int d : depths) {
            if (d > stencil_max_halo(h) - 1) continue;
            fs_config c = *cfg;
            c.tile_rows = h;
            c.sweeps_per_pass = d;
            double t = 0.0;
            int rc = time_config(&c, diffusion_rate, viscosity, dt, steps, d0, u0, v0, &t);
            if (rc != FS_OK) return rc;
            if (t < best) {
                best = t;
                best_tr = h;
                best_sw = d;
            }
        }
    }
    cfg->tile_rows = best_tr;
    cfg->sweeps_per_pass = best_sw;
    if (best_ms) *best_ms = best;
    cache_store(cache_path, key, best_tr, best_sw, best);
    return FS_OK;
}

// ---------------------------------------------------------------------------
// Autotuner for batches: the same search over whole batch steps. Every candidate
// builds its own batch (the tiling is fixed at creation), uploads each grid's tuning
// state and times `steps` graph replays after one warm-up step.

namespace {

std::string batch_tune_key(const fs_config* c, int count, const int* rows, const int* cols) {
    int dev = c->device;
    if (dev < 0) cudaGetDevice(&dev);
    cudaDeviceProp prop;
    std::memset(&prop, 0, sizeof(prop));
    cudaGetDeviceProperties(&prop, dev);
    unsigned long long h = 1469598103934665603ull;  // FNV-1a over the shapes
    for (int k = 0; k < count; ++k)
        for (int x : {rows[k], cols[k]}) {
            h ^= (unsigned)x;
            h *= 1099511628211ull;
        }
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s|%d|batch%d:%016llx|%d|%d", prop.name, prop.multiProcessorCount, count, h,
                  c->diffuse_iterations, c->pressure_iterations);
    for (char* p = buf; *p; ++p)
        if (*p == ' ') *p = '_';
    return buf;
}

struct TuningGrid {
    std::vector<float> d, u, v;
};

int time_batch(const fs_config* cfg, int count, const int* rows, const int* cols,
               const std::vector<const TuningGrid*>& state, float diff, float visc, float dt, int steps, double* ms) {
    fs_batch* b = nullptr;
    int rc = fs_batch_create(cfg, count, rows, cols, &b);
    if (rc != FS_OK) return rc;
    for (int k = 0; k < count && rc == FS_OK; ++k)
        rc = fs_batch_upload(b, k, state[k]->d.data(), state[k]->u.data(), state[k]->v.data());
    void* stream = nullptr;
    if (rc == FS_OK) rc = fs_batch_stream(b, &stream);
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (rc == FS_OK) rc = fs_batch_step(b, diff, visc, dt, 1);  // warm-up (captures the graph)
    if (rc == FS_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
        rc = record_error(FS_ERR_CUDA, "fs_batch_autotune: cudaEventCreate");
    if (rc == FS_OK) {
        cudaEventRecord(e0, st);
        rc = fs_batch_step(b, diff, visc, dt, steps);
        cudaEventRecord(e1, st);
    }
    if (rc == FS_OK) rc = fs_batch_sync(b);
    if (rc == FS_OK) {
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        *ms = t / steps;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    fs_batch_destroy(b);
    return rc;
}

}  // namespace

extern "C" int fs_batch_autotune(fs_config* cfg, int count, const int* rows, const int* cols, float diffusion_rate,
                                 float viscosity, float dt, int steps, const char* cache_path, double* best_ms) {
    if (!cfg || !rows || !cols || count < 1 || steps < 1) return record_error(FS_ERR_ARG, "fs_batch_autotune: bad argument");
    for (int k = 0; k < count; ++k)
        if (rows[k] < 3 || cols[k] < 3) return record_error(FS_ERR_ARG, "fs_batch_autotune: rows and cols must be >= 3");
    DeviceScope scope(cfg->device);
    const std::string key = batch_tune_key(cfg, count, rows, cols);
    int tr = 0, sw = 0;
    double ms = 0.0;
    if (cache_lookup(cache_path, key, &tr, &sw, &ms)) {
        cfg->tile_rows = tr;
        cfg->sweeps_per_pass = sw;
        if (best_ms) *best_ms = ms;
        return FS_OK;
    }
    // one tuning state per distinct shape
    std::vector<std::pair<std::pair<int, int>, TuningGrid>> shapes;
    std::vector<const TuningGrid*> state(count);
    for (int k = 0; k < count; ++k) {
        size_t i = 0;
        while (i < shapes.size() && shapes[i].first != std::make_pair(rows[k], cols[k])) ++i;
        if (i == shapes.size()) {
            shapes.emplace_back(std::make_pair(rows[k], cols[k]), TuningGrid{});
            TuningGrid& g = shapes.back().second;
            tuning_state(rows[k], cols[k], g.d, g.u, g.v);
        }
    }
    for (int k = 0; k < count; ++k)
        for (const auto& s : shapes)
            if (s.first == std::make_pair(rows[k], cols[k])) state[k] = &s.second;
    // depths: every even depth up to 16, and the depths that split the pressure sweeps
    // into two, three or four equal passes
    std::vector<int> depths = {2, 4, 6, 8, 10, 12, 14, 16};
    for (int n = 2; n <= 4; ++n) {
        const int d = (cfg->pressure_iterations + n - 1) / n;
        bool have = false;
        for (int x : depths) have |= x == d;
        if (d >= 2 && !have) depths.push_back(d);
    }
    const int heights[2] = {64, 128};
    double best = 1e30;
    int best_tr = 0, best_sw = 0;
    for (int h : heights) {
        for (int d : depths) {
            if (d > stencil_max_halo(h) - 1) continue;
            fs_config c = *cfg;
            c.tile_rows = h;
            c.sweeps_per_pass = d;
            c.use_graph = 1;
            double t = 0.0;
            int rc = time_batch(&c, count, rows, cols, state, diffusion_rate, viscosity, dt, steps, &t);
            if (rc != FS_OK) return rc;
            if (t < best) {
                best = t;
                best_tr = h;
                best_sw = d;
            }
        }
    }
    cfg->tile_rows = best_tr;
    cfg->sweeps_per_pass = best_sw;
    if (best_ms) *best_ms = best;
    cache_store(cache_path, key, best_tr, best_sw, best);
    return FS_OK;
}
