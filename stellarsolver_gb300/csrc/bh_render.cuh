// bh_render.cuh -- headless point rendering of the bodies, in place of the
// reference's OpenGL viewer (StellarSolverVisualizer.cpp:4-20, 208-253):
// every body is a one-pixel point, orthographic projection of [x0,x1]x[y0,y1]
// onto width x height pixels, colour (1,1,1) with alpha 0.1, blended with
// (SRC_ALPHA, ONE) over a (0,0,0,0.5) clear.  The blend is done in exact
// integer arithmetic (points per pixel, then one conversion), so the CPU
// restatement in the oracle matches it byte for byte.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ssg {

// Pixel of a point: column floor((x - x0) * sx), row from the top, or -1 when
// the point falls outside the image.  sx = width / (x1 - x0), sy likewise.
__host__ __device__ __forceinline__ int render_pixel(float x, float y, int width, int height,
                                                     float x0, float sx, float y0, float sy) {
#ifdef __CUDA_ARCH__
    const float fx = __fmul_rn(__fsub_rn(x, x0), sx);
    const float fy = __fmul_rn(__fsub_rn(y, y0), sy);
#else
    const float fx = (x - x0) * sx;
    const float fy = (y - y0) * sy;
#endif
    if (!(fx >= 0.0f) || !(fy >= 0.0f) || !(fx < (float)width) || !(fy < (float)height)) return -1;
    const int ix = (int)fx, iy = (int)fy;  // non-negative: truncation is floor
    if (ix >= width || iy >= height) return -1;
    return (height - 1 - iy) * width + ix;
}

// RGBA8 of a pixel hit by c points: colour min(1, 0.1 c), alpha
// min(1, 0.5 + 0.01 c), each rounded to nearest in units of 1/255.
__host__ __device__ __forceinline__ uint32_t render_rgba(uint32_t c) {
    const uint32_t v = c >= 10u ? 255u : (uint32_t)((255ull * c + 5ull) / 10ull);
    const uint32_t a = c >= 50u ? 255u : (uint32_t)((255ull * (50ull + c) + 50ull) / 100ull);
    return v | (v << 8) | (v << 16) | (a << 24);
}

static __global__ void k_splat(int n, const float* __restrict__ x, const float* __restrict__ y,
                               int width, int height, float x0, float sx, float y0, float sy,
                               uint32_t* __restrict__ counts) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int p = render_pixel(x[i], y[i], width, height, x0, sx, y0, sy);
    if (p >= 0) atomicAdd(counts + p, 1u);
}

static __global__ void k_shade(int pixels, uint32_t* __restrict__ px) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < pixels) px[i] = render_rgba(px[i]);
}

}  // namespace ssg
