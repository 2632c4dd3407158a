// Viewport streaming: the device side of writing a world's frame back into
// its particle store (the reference's `ParticleStore::update_from_gpu`,
// runners/bevy/src/particle_store.rs:71-85, a TODO there).  The store keeps
// the particles it holds outside the viewport, in store order; the frame's
// particles are appended after them.  This file has the stable compaction
// of the store by "outside the viewport" (key == ncells from
// k_upload_keys): per tile of 1024 items a count, one block scans the
// counts, then every tile writes its kept items in order.
#include "wrach_internal.cuh"
#include "wrach_kernels.h"

namespace wrach {

namespace {

constexpr uint32_t kThreads = 256, kPer = 4, kTile = kThreads * kPer;

// Exclusive scan of one value per thread over the block; *total receives
// the sum.
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_sum[32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sum[warp] = x;
  __syncthreads();
  uint32_t before = 0, all = 0;
  for (uint32_t w = 0; w < nw; ++w) {
    before += w < warp ? warp_sum[w] : 0u;
    all += warp_sum[w];
  }
  __syncthreads();
  *total = all;
  return before + x - v;
}

__global__ void __launch_bounds__(kThreads)
k_compact_count(const uint32_t* __restrict__ keys, uint32_t ncells, uint32_t n,
                uint32_t* __restrict__ tile_sums) {
  const uint32_t i0 = blockIdx.x * kTile + threadIdx.x * kPer;
  uint32_t c = 0;
#pragma unroll
  for (uint32_t u = 0; u < kPer; ++u) c += (i0 + u < n && keys[i0 + u] >= ncells) ? 1u : 0u;
  uint32_t total;
  block_scan(c, &total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// One block: tile_sums becomes its exclusive scan; *count = the total.
__global__ void __launch_bounds__(1024)
k_compact_scan(uint32_t* __restrict__ tile_sums, uint32_t ntiles, uint32_t* __restrict__ count) {
  uint32_t carry = 0;
  for (uint32_t b0 = 0; b0 < ntiles; b0 += blockDim.x) {
    const uint32_t b = b0 + threadIdx.x;
    const uint32_t v = b < ntiles ? tile_sums[b] : 0u;
    uint32_t total;
    const uint32_t ex = block_scan(v, &total);
    if (b < ntiles) tile_sums[b] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *count = carry;
}

__global__ void __launch_bounds__(kThreads)
k_compact_scatter(const uint32_t* __restrict__ keys, uint32_t ncells, uint32_t n,
                  const uint32_t* __restrict__ tile_offsets, const float2* __restrict__ pos,
                  const float2* __restrict__ vel, float2* __restrict__ dst_pos,
                  float2* __restrict__ dst_vel) {
  const uint32_t i0 = blockIdx.x * kTile + threadIdx.x * kPer;
  bool keep[kPer];
  uint32_t c = 0;
#pragma unroll
  for (uint32_t u = 0; u < kPer; ++u) {
    keep[u] = i0 + u < n && keys[i0 + u] >= ncells;
    c += keep[u] ? 1u : 0u;
  }
  uint32_t total;
  uint32_t d = tile_offsets[blockIdx.x] + block_scan(c, &total);
#pragma unroll
  for (uint32_t u = 0; u < kPer; ++u) {
    if (keep[u]) {
      dst_pos[d] = pos[i0 + u];
      dst_vel[d] = vel[i0 + u];
      ++d;
    }
  }
}

}  // namespace

uint32_t keep_outside_tiles(uint32_t n) { return (n + kTile - 1) / kTile; }

cudaError_t launch_keep_outside(const uint32_t* keys, uint32_t ncells, uint32_t n,
                                const float2* pos, const float2* vel, float2* dst_pos,
                                float2* dst_vel, uint32_t* tile_sums, uint32_t* count,
                                cudaStream_t st) {
  const uint32_t ntiles = keep_outside_tiles(n);
  cudaError_t e;
  if (ntiles) {
    k_compact_count<<<ntiles, kThreads, 0, st>>>(keys, ncells, n, tile_sums);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  k_compact_scan<<<1, 1024, 0, st>>>(tile_sums, ntiles, count);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (ntiles) {
    k_compact_scatter<<<ntiles, kThreads, 0, st>>>(keys, ncells, n, tile_sums, pos, vel, dst_pos,
                                                   dst_vel);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace wrach
