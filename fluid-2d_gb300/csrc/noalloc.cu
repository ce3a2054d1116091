// fs_project_noalloc: the pressure projection for callers that cannot allocate device
// memory.
//
// Who needs it: code that calls the solver from inside a host framework that owns all
// device memory (a fixed pool or budget, no raw cudaMalloc allowed), plug-ins whose host
// application hands them device buffers but no allocator, and frame loops that must not
// allocate after start-up so they can neither stall on the allocator nor fail with
// out-of-memory mid-run. fs_create() allocates the solver's scratch with cudaMalloc, so
// these callers cannot use a handle.
//
// This entry point takes the caller's device buffers for its inputs and outputs and
// keeps its own scratch (the divergence and two pressure buffers) in one file-scope
// __device__ array of fixed size, FS_NOALLOC_MAX_CELLS floats per buffer (3 x 4 MiB).
// That array exists on every GPU that loads this library and stays allocated there
// until the process exits. Nothing here calls cudaMalloc, cudaFree or any allocating
// routine.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress (and sets the kernels' shared-memory limit) and caches it for
// that device; make that first call before any stream capture begins on the device,
// since the set-up calls are not stream work. A cudaDeviceReset() on a
// device releases the array and leaves the cached address stale: calls on that device
// after a reset are not supported. Every call shares the
// one array: calls that can overlap on the GPU (different streams, or different host
// threads on the same device) race on it and must be serialised by the caller. The
// array keeps the previous call's contents; nothing in it needs to start at zero (the
// pressure solve starts from zero in registers, and each buffer is written before it
// is read).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/fluid2d_gb300.h"
#include "fs_internal.cuh"

namespace {

using namespace fs;

constexpr size_t kCells = (size_t)FS_NOALLOC_MAX_CELLS;

// div | p ping | p pong, each kCells floats.
static __device__ __align__(256) float g_project_scratch[3 * kCells];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
float* g_scratch_on_device[kMaxDevices] = {};

int scratch_for_current_device(float** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return record_error(FS_ERR_CUDA, "fs_project_noalloc: cudaGetDevice failed");
    if (dev < 0 || dev >= kMaxDevices) return record_error(FS_ERR_ARG, "fs_project_noalloc: device ordinal >= 64");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_on_device[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_project_scratch);
        if (e != cudaSuccess || p == nullptr)
            return record_error(FS_ERR_CUDA, "fs_project_noalloc: cudaGetSymbolAddress of the scratch array failed");
        e = stencil_prepare();
        if (e != cudaSuccess)
            return record_error(FS_ERR_CUDA, "fs_project_noalloc: setting the stencil kernels' shared memory failed");
        g_scratch_on_device[dev] = static_cast<float*>(p);
    }
    *out = g_scratch_on_device[dev];
    return FS_OK;
}

}  // namespace

extern "C" int fs_project_noalloc(const float* u, const float* v, float* u_out, float* v_out, int rows, int cols,
                                  int pitch, int iterations, void* stream) {
    if (!u || !v || !u_out || !v_out) return record_error(FS_ERR_ARG, "fs_project_noalloc: null pointer");
    if (rows < 3 || cols < 3) return record_error(FS_ERR_ARG, "fs_project_noalloc: rows and cols must be >= 3");
    if (pitch < cols) return record_error(FS_ERR_ARG, "fs_project_noalloc: pitch must be >= cols");
    if (iterations < 0) return record_error(FS_ERR_ARG, "fs_project_noalloc: negative iteration count");
    if ((size_t)rows * (size_t)pitch > kCells)
        return record_error(FS_ERR_ARG,
                            "fs_project_noalloc: rows * pitch exceeds FS_NOALLOC_MAX_CELLS (1048576 floats); "
                            "use a solver handle for larger grids");
    // The last pass reads u and v around each output cell while other CTAs write the
    // outputs, so no output may overlap an input or the other output anywhere in its
    // rows x pitch extent (the inputs may overlap each other: they are only read).
    {
        const size_t extent = (size_t)rows * (size_t)pitch * sizeof(float);
        auto overlap = [extent](const void* a, const void* b) {
            const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
            return x < y + extent && y < x + extent;
        };
        if (overlap(u_out, u) || overlap(u_out, v) || overlap(v_out, u) || overlap(v_out, v) || overlap(u_out, v_out))
            return record_error(FS_ERR_ARG,
                                "fs_project_noalloc: an output overlaps an input or the other output (rows * pitch "
                                "floats each)");
    }

    float* base = nullptr;
    int rc = scratch_for_current_device(&base);
    if (rc != FS_OK) return rc;
    float* div = base;
    float* pbuf[2] = {base + kCells, base + 2 * kCells};
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // Same plan as a handle's projection: depth-8 temporally blocked passes over
    // 64-row regions, divergence fused into the first pass, gradient subtract and
    // reflecting fills into the last.
    const int depth = 8, tile_rows = 64;
    const int m = std::max(1, (iterations + depth - 1) / depth);
    std::vector<int> plan(m, iterations / m);
    for (int i = 0; i < iterations % m; ++i) plan[i] += 1;
    const float h = 1.0f / sqrtf((float)((size_t)rows * (size_t)cols));
    for (int pass = 0; pass < m; ++pass) {
        const bool last = pass == m - 1;
        StencilLaunch L{};
        L.nfields = 1;
        StencilField& f = L.f[0];
        const int halo = plan[pass] + (last ? 1 : 0);
        f.rows = rows;
        f.cols = cols;
        f.pitch = pitch;
        f.halo = halo;
        f.tile_w = kRegionW - 2 * halo;
        f.tile_h = tile_rows - 2 * halo;
        tile_split(cols, f.tile_w, &f.tiles_x, &f.shift_x);
        tile_split(rows, f.tile_h, &f.tiles_y, &f.shift_y);
        if (pass > 0 && !last) realign_columns(f);  // as for a handle's fixed-count projection
        f.s_lr = f.s_tb = 1.f;
        f.sweeps = plan[pass];
        f.cdiv = -0.5f * h;
        f.h = h;
        if (pass == 0) {
            f.kind = PASS_PRESSURE_FIRST;
            f.x = u;
            f.x2 = v;
            f.cst = nullptr;  // pressure starts at zero
            f.cst_out = div;
        } else {
            f.kind = PASS_PRESSURE;
            f.x = pbuf[(pass - 1) & 1];
            f.cst = div;
        }
        f.y = last ? nullptr : pbuf[pass & 1];
        if (last) {
            f.epilogue = 1;
            f.u_in = u;
            f.v_in = v;
            f.u_out = u_out;
            f.v_out = v_out;
        }
        cudaError_t e = launch_stencil(L, tile_rows, st);
        if (e != cudaSuccess) return record_error(FS_ERR_CUDA, "fs_project_noalloc: stencil launch failed");
    }
    return FS_OK;
}
