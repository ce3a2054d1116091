// Headless versions of the reference's two render kernels, on the solver's resident
// state (the SFML texture/window halves are out of scope: no graphics stack).
//
//   density  -> RGBA8, grid_to_image_kernel (src/density_grid_renderer.cu:10-29): each
//               channel is uint8(max(0, min(255, m_c * d))) (truncating), alpha 255.
//   velocity -> line vertices, velocity_to_lines_kernel (src/velocity_grid_renderer.cu:
//               8-44): one line per cell from (j*hs, i*vs); every 8th row and column the
//               end point moves by 250000 * (u, v) / sqrtf(rows*cols); all white. Vertex
//               layout is SFML's sf::Vertex: position (2 floats), colour (4 bytes),
//               texture coordinates (2 floats, zero) = 20 bytes; two per cell.

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fluid2d_gb300.h"
#include "fs_internal.cuh"

namespace fs {
namespace {

__global__ void density_rgba_kernel(const float* __restrict__ d, int rows, int cols, int pitch, float mr, float mg,
                                    float mb, uint8_t* __restrict__ out) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)rows * cols) return;
    const int i = (int)(e / cols), j = (int)(e % cols);
    const float v = d[(size_t)i * pitch + j];
    uchar4 px;
    px.x = (uint8_t)fmaxf(0.f, fminf(255.f, mr * v));
    px.y = (uint8_t)fmaxf(0.f, fminf(255.f, mg * v));
    px.z = (uint8_t)fmaxf(0.f, fminf(255.f, mb * v));
    px.w = 255;
    reinterpret_cast<uchar4*>(out)[e] = px;
}

struct Vertex {
    float x, y;
    uint8_t r, g, b, a;
    float tu, tv;
};
static_assert(sizeof(Vertex) == 20, "sf::Vertex layout");

__global__ void velocity_lines_kernel(const float* __restrict__ u, const float* __restrict__ v, int rows, int cols,
                                      int pitch, float hs, float vs, Vertex* __restrict__ out) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)rows * cols) return;
    const int i = (int)(e / cols), j = (int)(e % cols);
    Vertex s, t;
    s.x = __fmul_rn((float)j, hs);
    s.y = __fmul_rn((float)i, vs);
    t.x = s.x;
    t.y = s.y;
    if (i % 8 == 0 && j % 8 == 0) {
        const float norm = sqrtf((float)((size_t)rows * (size_t)cols));
        t.x = __fadd_rn(t.x, __fdiv_rn(__fmul_rn(250000.f, u[(size_t)i * pitch + j]), norm));
        t.y = __fadd_rn(t.y, __fdiv_rn(__fmul_rn(250000.f, v[(size_t)i * pitch + j]), norm));
    }
    s.r = s.g = s.b = s.a = 255;
    t.r = t.g = t.b = t.a = 255;
    s.tu = s.tv = t.tu = t.tv = 0.f;
    out[2 * e] = s;
    out[2 * e + 1] = t;
}

}  // namespace
}  // namespace fs

using namespace fs;

extern "C" int fs_render_density(const float* density, int rows, int cols, int pitch, float mr, float mg, float mb,
                                 void* rgba, void* stream) {
    if (!density || !rgba || rows < 1 || cols < 1 || pitch < cols)
        return record_error(FS_ERR_ARG, "fs_render_density: bad argument");
    const long n = (long)rows * cols;
    density_rgba_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(density, rows, cols, pitch, mr,
                                                                                        mg, mb, (uint8_t*)rgba);
    return cudaGetLastError() == cudaSuccess ? FS_OK : record_error(FS_ERR_CUDA, "fs_render_density: launch");
}

extern "C" int fs_render_velocity_lines(const float* u, const float* v, int rows, int cols, int pitch,
                                        float hscale, float vscale, void* vertices, void* stream) {
    if (!u || !v || !vertices || rows < 1 || cols < 1 || pitch < cols)
        return record_error(FS_ERR_ARG, "fs_render_velocity_lines: bad argument");
    const long n = (long)rows * cols;
    velocity_lines_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(u, v, rows, cols, pitch,
                                                                                          hscale, vscale,
                                                                                          (Vertex*)vertices);
    return cudaGetLastError() == cudaSuccess ? FS_OK : record_error(FS_ERR_CUDA, "fs_render_velocity_lines: launch");
}
