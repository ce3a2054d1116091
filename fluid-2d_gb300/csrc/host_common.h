// Host-side helpers shared by the single-grid and batched drivers: pass planning,
// tile geometry, the reference's step constants, and CUDA error reporting.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/fluid2d_gb300.h"
#include "fs_internal.cuh"

namespace fs {

inline int cuda_error(cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return record_error(e == cudaErrorMemoryAllocation ? FS_ERR_NOMEM : FS_ERR_CUDA, m.c_str());
}

#define FS_CK(call)                                              \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return ::fs::cuda_error(e_, #call); \
    } while (0)

struct DeviceScope {
    int prev = -1;
    bool changed = false;
    explicit DeviceScope(int dev) {
        if (dev < 0) return;
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) {
            if (cudaSetDevice(dev) == cudaSuccess) changed = true;
        }
    }
    ~DeviceScope() {
        if (changed) cudaSetDevice(prev);
    }
};

// Split `total` sweeps into passes of at most `k` (at least one pass, possibly of
// zero sweeps, so that fused work such as add_sources always runs).
inline std::vector<int> plan_passes(int total, int k) {
    int m = std::max(1, (total + k - 1) / k);
    std::vector<int> out(m, total / m);
    for (int i = 0; i < total % m; ++i) out[i] += 1;
    return out;
}

inline void field_geometry(StencilField& f, int rows, int cols, int pitch, int tile_rows, int halo) {
    f.rows = rows;
    f.cols = cols;
    f.pitch = pitch;
    f.halo = halo;
    f.tile_w = kRegionW - 2 * halo;
    f.tile_h = tile_rows - 2 * halo;
    tile_split(cols, f.tile_w, &f.tiles_x, &f.shift_x);
    tile_split(rows, f.tile_h, &f.tiles_y, &f.shift_y);
}

// a = dt * float(rows*cols) * rate (fluid_solver_gpu.cu:79) and the FP32 pair for
// dividing by the reference's double divisor 1 + 4a.
inline void field_diffusion(StencilField& f, int rows, int cols, float rate, float dt) {
    const float a = dt * (float)((size_t)rows * (size_t)cols) * rate;
    const double D = 1.0 + 4.0 * (double)a;
    f.a = a;
    f.dh = (float)D;
    f.dl = (float)(D - (double)f.dh);
    f.rf = (float)(1.0 / D);
}

// dt0 = sqrt(rows*cols)*dt evaluated in double (fluid_solver_gpu.cu:334).
inline AdvectArgs make_advect_args(int rows, int cols, int pitch, float dt) {
    AdvectArgs A;
    A.rows = rows;
    A.cols = cols;
    A.pitch = pitch;
    A.dt0 = (float)(std::sqrt((double)((size_t)rows * (size_t)cols)) * (double)dt);
    A.xmax = (float)cols - 1.5f;
    A.ymax = (float)rows - 1.5f;
    return A;
}

// h = 1.0f / sqrtf(rows*cols) (fluid_solver_gpu.cu:367).
inline float grid_spacing(int rows, int cols) { return 1.0f / sqrtf((float)((size_t)rows * (size_t)cols)); }

inline int pitch_for(int cols) { return (cols + 31) / 32 * 32; }

}  // namespace fs
