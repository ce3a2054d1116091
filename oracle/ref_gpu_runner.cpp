// Runner for the reference's own GPU kernels — TEST INFRASTRUCTURE ONLY.
//
// oracle/build_oracle.py compiles mworchel/fluid-2d src/fluid_solver_gpu.cu, unmodified,
// into a device-only fatbinary for sm_103a (oracle/_ref/ref_gpu.fatbin). Device code does
// not depend on the host architecture, so that file runs on any GB300 host. This runner
// loads it with the CUDA driver API and drives the reference's kernels in the order and
// with the launch shapes of the reference's host code:
//   fluid_solver_gpu::solve      src/fluid_solver_gpu.cu:222-258
//   set_boundary_* wrappers      src/fluid_solver_gpu.cu:260-276 (1-D, 64 threads, max(rows, cols))
//   add_sources                  src/fluid_solver_gpu.cu:278-288 (2-D, 32x32 blocks)
//   diffuse                      src/fluid_solver_gpu.cu:290-312
//   smooth                       src/fluid_solver_gpu.cu:314-323
//   advect                       src/fluid_solver_gpu.cu:325-356 (dt0 in double, then float)
//   project                      src/fluid_solver_gpu.cu:358-404 (h = 1 / sqrtf(rows*cols))
// with unpadded device buffers (pitch = cols * 4 B, src/linear_buffer.hpp:34-40) and the
// launch grid of src/kernel_launcher.hpp:9-31. Every floating-point operation of a step
// except dt0 and h runs in the reference's compiled kernels, so outputs of this runner are
// outputs of the reference's solver. The sweep counts are parameters; the reference
// hard-codes kd = 15 and kp = 20 (src/fluid_solver_gpu.cu:238, 245-247, 252).
//
// Used only to generate and check the golden fixtures under tests/golden and by the GPU
// tests that compare against the reference live; never part of the product.

#include <cuda.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

// Kernel-argument image of element_accessor<float> (src/gpu_buffer.hpp:8-26): pointer, pitch.
struct Accessor {
    CUdeviceptr data;
    size_t pitch;
};

// Mangled names of the float instantiations in the fatbinary (nm of the same compile).
const char* const kNames[] = {
    "_Z30set_boundary_continuous_kernelIfEv16element_accessorIT_Emm",
    "_Z39set_boundary_opposite_horizontal_kernelIfEv16element_accessorIT_Emm",
    "_Z37set_boundary_opposite_vertical_kernelIfEv16element_accessorIT_Emm",
    "_Z18add_sources_kernelIfEv16element_accessorIT_ES2_mmf",
    "_Z24diffuse_iteration_kernelIfEv16element_accessorIT_ES2_S2_mmS1_f",
    "_Z13smooth_kernelIfEv16element_accessorIT_ES2_mm",
    "_Z13advect_kernelIfEv16element_accessorIT_ES2_S2_S2_mmf",
    "_Z19advect_trace_kernelIfEv16element_accessorIT_ES2_S2_S2_mmf",
    "_Z27calculate_divergence_kernelIfEv16element_accessorIT_ES2_S2_mmf",
    "_Z18p_iteration_kernelIfEv16element_accessorIT_ES2_S2_mm",
    "_Z15remove_p_kernelIfEv16element_accessorIT_ES2_S2_mmf",
};
enum { K_BND_CONT, K_BND_H, K_BND_V, K_ADD, K_DIFF, K_SMOOTH, K_ADV, K_TRACE, K_DIV, K_P, K_REMOVE, K_COUNT };

std::string g_err;
CUcontext g_ctx = nullptr;
CUmodule g_mod = nullptr;
CUfunction g_fn[K_COUNT];

bool ok(CUresult r, const char* what) {
    if (r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "unknown CUDA error");
    return false;
}

struct Runner {
    size_t rows, cols;
    bool good = true;
    // Buffers of fluid_solver_gpu (src/fluid_solver_gpu.cuh:62-70).
    CUdeviceptr d = 0, u = 0, v = 0, src = 0, t1 = 0, t2 = 0, t3 = 0;

    Runner(size_t r, size_t c) : rows(r), cols(c) {
        for (CUdeviceptr* p : {&d, &u, &v, &src, &t1, &t2, &t3})
            if (good) good = ok(cuMemAlloc(p, bytes()), "cuMemAlloc");
    }
    ~Runner() {
        for (CUdeviceptr p : {d, u, v, src, t1, t2, t3})
            if (p) cuMemFree(p);
    }
    size_t bytes() const { return sizeof(float) * rows * cols; }
    Accessor acc(CUdeviceptr p) const { return Accessor{p, sizeof(float) * cols}; }

    void launch(int k, unsigned gx, unsigned gy, unsigned bx, unsigned by, void** args) {
        if (good) good = ok(cuLaunchKernel(g_fn[k], gx, gy, 1, bx, by, 1, 0, nullptr, args, nullptr), kNames[k]);
        if (good) good = ok(cuCtxSynchronize(), kNames[k]);
    }
    // kernel_launcher::launch_2d(kernel, width = cols, height = rows, ...)
    void launch2d(int k, void** args) {
        const unsigned w = (unsigned)cols, h = (unsigned)rows;
        launch(k, (w + 31) / 32, (h + 31) / 32, 32, 32, args);
    }
    // kernel_launcher::launch_1d(kernel, max(cols, rows), ...)
    void bnd(int k, CUdeviceptr x) {
        Accessor a = acc(x);
        size_t r = rows, c = cols;
        void* args[] = {&a, &r, &c};
        const unsigned w = (unsigned)(rows > cols ? rows : cols);
        launch(k, (w + 63) / 64, 1, 64, 1, args);
    }
    void copy(CUdeviceptr dst, CUdeviceptr s) {
        if (good) good = ok(cuMemcpyDtoD(dst, s, bytes()), "cuMemcpyDtoD");
    }
    void clear(CUdeviceptr x) {
        if (good) good = ok(cuMemsetD8(x, 0, bytes()), "cuMemsetD8");
    }

    void add_sources(CUdeviceptr x, const float* host_src, float dt) {
        if (good) good = ok(cuMemcpyHtoD(src, host_src, bytes()), "cuMemcpyHtoD");
        Accessor a = acc(x), s = acc(src);
        size_t r = rows, c = cols;
        void* args[] = {&a, &s, &r, &c, &dt};
        launch2d(K_ADD, args);
    }
    void diffuse(CUdeviceptr x, int bnd_kernel, float rate, float dt, int iters) {
        copy(t1, x);
        for (int k = 0; k < iters; ++k) {
            copy(t2, x);
            Accessor a = acc(x), p = acc(t2), i = acc(t1);
            size_t r = rows, c = cols;
            void* args[] = {&a, &p, &i, &r, &c, &rate, &dt};
            launch2d(K_DIFF, args);
            bnd(bnd_kernel, x);
        }
    }
    void smooth(CUdeviceptr x) {
        copy(t1, x);
        Accessor a = acc(x), i = acc(t1);
        size_t r = rows, c = cols;
        void* args[] = {&a, &i, &r, &c};
        launch2d(K_SMOOTH, args);
    }
    void advect(CUdeviceptr x, CUdeviceptr hu, CUdeviceptr hv, int bnd_kernel, float dt, bool trace) {
        copy(t1, x);
        // float dt0 = sqrt(m_rows * m_cols) * dt: the integer overload of sqrt returns double.
        const float dt0 = (float)(std::sqrt((double)(rows * cols)) * (double)dt);
        Accessor a = acc(x), i = acc(t1), au = acc(hu), av = acc(hv);
        size_t r = rows, c = cols;
        float t = dt0;
        void* args[] = {&a, &i, &au, &av, &r, &c, &t};
        if (trace) {
            clear(x);
            launch2d(K_TRACE, args);
        } else {
            launch2d(K_ADV, args);
        }
        bnd(bnd_kernel, x);
    }
    void project(CUdeviceptr hu, CUdeviceptr hv, int iters) {
        clear(t1);
        clear(t2);
        float h = 1.0f / sqrtf((float)(rows * cols));
        {
            Accessor dv = acc(t1), au = acc(hu), av = acc(hv);
            size_t r = rows, c = cols;
            void* args[] = {&dv, &au, &av, &r, &c, &h};
            launch2d(K_DIV, args);
        }
        bnd(K_BND_CONT, t1);
        for (int k = 0; k < iters; ++k) {
            copy(t3, t2);
            Accessor p = acc(t2), pp = acc(t3), dv = acc(t1);
            size_t r = rows, c = cols;
            void* args[] = {&p, &pp, &dv, &r, &c};
            launch2d(K_P, args);
            bnd(K_BND_CONT, t2);
        }
        {
            Accessor au = acc(hu), av = acc(hv), p = acc(t2);
            size_t r = rows, c = cols;
            void* args[] = {&au, &av, &p, &r, &c, &h};
            launch2d(K_REMOVE, args);
        }
        bnd(K_BND_H, hu);
        bnd(K_BND_V, hv);
    }
    // fluid_solver_gpu::solve (src/fluid_solver_gpu.cu:222-258), device state kept between steps
    // (the reference's download and re-upload of the state between two calls is an exact copy).
    void step(const float* ds, float diff, const float* us, const float* vs, float visc, float dt, int kd, int kp) {
        add_sources(d, ds, dt);
        diffuse(d, K_BND_CONT, diff, dt, kd);
        advect(d, u, v, K_BND_CONT, dt, true);
        smooth(d);
        add_sources(u, us, dt);
        add_sources(v, vs, dt);
        diffuse(u, K_BND_H, visc, dt, kd);
        diffuse(v, K_BND_V, visc, dt, kd);
        project(u, v, kp);
        copy(t2, u);
        copy(t3, v);
        advect(u, t2, t3, K_BND_H, dt, false);
        advect(v, t2, t3, K_BND_V, dt, false);
        project(u, v, kp);
    }
};

}  // namespace

extern "C" {

const char* ref_gpu_last_error() { return g_err.c_str(); }

// Load the fatbinary on device 0. Returns 0 on success.
int ref_gpu_load(const char* fatbin_path) {
    if (g_mod) return 0;
    FILE* f = std::fopen(fatbin_path, "rb");
    if (!f) {
        g_err = std::string("cannot open ") + fatbin_path;
        return 1;
    }
    std::vector<char> image;
    char buf[65536];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) image.insert(image.end(), buf, buf + got);
    std::fclose(f);
    CUdevice dev;
    if (!ok(cuInit(0), "cuInit") || !ok(cuDeviceGet(&dev, 0), "cuDeviceGet") ||
        !ok(cuDevicePrimaryCtxRetain(&g_ctx, dev), "cuDevicePrimaryCtxRetain") ||
        !ok(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent") ||
        !ok(cuModuleLoadData(&g_mod, image.data()), "cuModuleLoadData"))
        return 2;
    for (int k = 0; k < K_COUNT; ++k)
        if (!ok(cuModuleGetFunction(&g_fn[k], g_mod, kNames[k]), kNames[k])) return 3;
    return 0;
}

// nsteps reference steps on host arrays (row-major rows x cols, boundary included); state
// d, u, v in/out, sources constant over the steps. Returns 0 on success.
int ref_gpu_solve(long rows, long cols, float* d, const float* ds, float diff, float* u, float* v,
                  const float* us, const float* vs, float visc, float dt, int kd, int kp, int nsteps) {
    if (!g_mod) {
        g_err = "ref_gpu_load has not succeeded";
        return 1;
    }
    if (rows < 3 || cols < 3 || kd < 0 || kp < 0 || nsteps < 0) {
        g_err = "bad arguments";
        return 1;
    }
    if (!ok(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent")) return 2;
    Runner r((size_t)rows, (size_t)cols);
    if (r.good) r.good = ok(cuMemcpyHtoD(r.d, d, r.bytes()), "upload d");
    if (r.good) r.good = ok(cuMemcpyHtoD(r.u, u, r.bytes()), "upload u");
    if (r.good) r.good = ok(cuMemcpyHtoD(r.v, v, r.bytes()), "upload v");
    for (int s = 0; s < nsteps && r.good; ++s) r.step(ds, diff, us, vs, visc, dt, kd, kp);
    if (r.good) r.good = ok(cuMemcpyDtoH(d, r.d, r.bytes()), "download d");
    if (r.good) r.good = ok(cuMemcpyDtoH(u, r.u, r.bytes()), "download u");
    if (r.good) r.good = ok(cuMemcpyDtoH(v, r.v, r.bytes()), "download v");
    return r.good ? 0 : 2;
}

// One stage of the reference's step on host arrays (rows x cols): the kernels of one
// helper of src/fluid_solver_gpu.cu with its copies and fills.
//   0 add_sources (x += dt * src, interior)           278-288
//   1 diffuse(x, mode, rate, dt, iters)                290-312
//   2 advect(x, u, v, continuous, dt, trace = true)    325-356
//   3 smooth(x)                                        314-323
//   4 advect(x, u, v, mode, dt, trace = false)         325-356
//   5 project(u, v, iters)                             358-404
// mode: 0 continuous, 1 opposite horizontal, 2 opposite vertical.
int ref_gpu_stage(int stage, long rows, long cols, float* x, const float* src, float* u, float* v, int mode,
                  float rate, float dt, int iters) {
    if (!g_mod) {
        g_err = "ref_gpu_load has not succeeded";
        return 1;
    }
    if (rows < 3 || cols < 3 || iters < 0 || mode < 0 || mode > 2 || stage < 0 || stage > 5) {
        g_err = "bad arguments";
        return 1;
    }
    if (!ok(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent")) return 2;
    Runner r((size_t)rows, (size_t)cols);
    const int bk = mode == 0 ? K_BND_CONT : mode == 1 ? K_BND_H : K_BND_V;
    const bool has_x = stage != 5, has_uv = stage == 2 || stage == 4 || stage == 5;
    if (has_x && r.good) r.good = ok(cuMemcpyHtoD(r.d, x, r.bytes()), "upload x");
    if (has_uv && r.good) r.good = ok(cuMemcpyHtoD(r.u, u, r.bytes()), "upload u");
    if (has_uv && r.good) r.good = ok(cuMemcpyHtoD(r.v, v, r.bytes()), "upload v");
    if (r.good) {
        switch (stage) {
            case 0: r.add_sources(r.d, src, dt); break;
            case 1: r.diffuse(r.d, bk, rate, dt, iters); break;
            case 2: r.advect(r.d, r.u, r.v, K_BND_CONT, dt, true); break;
            case 3: r.smooth(r.d); break;
            case 4: r.advect(r.d, r.u, r.v, bk, dt, false); break;
            case 5: r.project(r.u, r.v, iters); break;
        }
    }
    if (has_x && stage != 5 && r.good) r.good = ok(cuMemcpyDtoH(x, r.d, r.bytes()), "download x");
    if (stage == 5 && r.good) r.good = ok(cuMemcpyDtoH(u, r.u, r.bytes()), "download u");
    if (stage == 5 && r.good) r.good = ok(cuMemcpyDtoH(v, r.v, r.bytes()), "download v");
    return r.good ? 0 : 2;
}

}  // extern "C"
