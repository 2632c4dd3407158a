// Headless point rasteriser: the reference's draw pass
// (assets/shaders/draw.wgsl:18-40: one instanced quad of half-size 0.4 world
// units per particle, white on black; MSAA 4, runners/bevy/src/render/
// pipeline.rs:52-56) as CUDA kernels writing an 8-bit framebuffer instead of
// a swapchain image.
//
// Mapping (the vertex shader's NDC transform, y up in the world, row 0 at the
// top of the image): a world point (x, y) lands on pixel coordinates
//   X = x * sx,  Y = height_px - y * sy,  sx = width_px / W, sy = height_px / H.
// A particle covers the axis-aligned square [X - hx, X + hx) x [Y - hy, Y + hy)
// with hx = 0.4 * sx, hy = 0.4 * sy; a sample is covered when it lies in that
// half-open square (the top-left fill rule of an axis-aligned quad).  Each
// pixel has the four standard MSAA sample positions.  As in a multisampled
// colour target, a sample is white once any quad covers it, so a pixel's
// value is the resolve of the union of its covered samples:
// 255 * popcount(mask) / 4, rounded down, where the 4-bit mask is OR-ed over
// every particle that touches the pixel.
#include <stdint.h>

#include "wrach_internal.cuh"
#include "wrach_kernels.h"

namespace wrach {

namespace {

// standard 4x sample positions inside a pixel
__constant__ float kSampleX[4] = {0.375f, 0.875f, 0.125f, 0.625f};
__constant__ float kSampleY[4] = {0.125f, 0.375f, 0.625f, 0.875f};

__global__ void k_raster(const float2* __restrict__ pos, uint32_t n, float sx, float sy,
                         uint32_t width_px, uint32_t height_px, uint32_t* __restrict__ cover) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 p = pos[i];
  const float X = __fmul_rn(p.x, sx);
  const float Y = __fsub_rn((float)height_px, __fmul_rn(p.y, sy));
  const float hx = __fmul_rn(0.4f, sx), hy = __fmul_rn(0.4f, sy);
  const float x0 = __fsub_rn(X, hx), x1 = __fadd_rn(X, hx);
  const float y0 = __fsub_rn(Y, hy), y1 = __fadd_rn(Y, hy);
  if (!(x1 > 0.0f) || !(y1 > 0.0f) || !(x0 < (float)width_px) || !(y0 < (float)height_px)) return;
  const int px0 = max((int)floorf(x0), 0), px1 = min((int)floorf(x1), (int)width_px - 1);
  const int py0 = max((int)floorf(y0), 0), py1 = min((int)floorf(y1), (int)height_px - 1);
  for (int py = py0; py <= py1; ++py)
    for (int px = px0; px <= px1; ++px) {
      uint32_t mask = 0;
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const float sxp = __fadd_rn((float)px, kSampleX[s]);
        const float syp = __fadd_rn((float)py, kSampleY[s]);
        mask |= (sxp >= x0 && sxp < x1 && syp >= y0 && syp < y1) ? 1u << s : 0u;
      }
      if (mask) atomicOr(&cover[(size_t)py * width_px + px], mask);
    }
}

__global__ void k_resolve(const uint32_t* __restrict__ cover, size_t npix,
                          uint8_t* __restrict__ image) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < npix) image[i] = (uint8_t)(255u * (uint32_t)__popc(cover[i]) / 4u);
}

}  // namespace

cudaError_t launch_render(const float2* pos, uint32_t n, float world_w, float world_h,
                          uint32_t width_px, uint32_t height_px, uint32_t* cover,
                          uint8_t* image, cudaStream_t st) {
  const size_t npix = (size_t)width_px * height_px;
  cudaError_t e = cudaMemsetAsync(cover, 0, npix * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  const float sx = (float)width_px / world_w, sy = (float)height_px / world_h;
  if (n) {
    k_raster<<<(n + 255) / 256, 256, 0, st>>>(pos, n, sx, sy, width_px, height_px, cover);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  k_resolve<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(cover, npix, image);
  return cudaGetLastError();
}

}  // namespace wrach
