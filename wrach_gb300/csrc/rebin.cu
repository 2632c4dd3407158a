// Rebin: the count, scan and pack passes of a frame
// (assets/shaders/particles_per_cell.wgsl, prefix_sum.wgsl,
// pack_new_particle_data.wgsl; dispatched by runners/bevy/src/compute/
// builder.rs:86-89) as one persistent cooperative kernel.
//
// The result is a stable counting sort: a cell's particles keep their source
// order.  (The reference places them with atomicSub and so leaves the order
// inside a cell unspecified; the CPU packer's order, spatial_bin.rs:103-149,
// is the stable one.)
//
// The sort is an LSD radix sort (8-bit digits) of (cell key, source index),
// run over all co-resident blocks of one cooperative launch with grid
// barriers between its phases.  Every block owns a contiguous chunk of the
// source, split into one contiguous sub-range per warp; a warp ranks its items
// 32 at a time in source order with warp-private digit counters in shared
// memory (__match_any_sync groups equal digits inside a step), so the rank of
// every item is stable.  Per pass:
//   A  digit histogram of each block (the warps' counters summed),
//   B  per digit, the exclusive prefix over blocks (digit rows spread over the
//      blocks) and the digit totals,
//   C  each item's destination = digit offset + block offset + warp offset +
//      rank, and the scatter.
// The cost is the same for any cell occupancy and any particle displacement.
// The cell-start table comes from per-cell counts (atomics during the first
// pass): tile sums are taken between two barriers of the first pass, and after
// the gather every block scans them and writes its own tiles' starts.
#include <limits.h>

#include "wrach_internal.cuh"
#include "wrach_kernels.h"

namespace wrach {

namespace {

constexpr uint32_t T = kRebinThreads;
constexpr uint32_t CPT = kCellsPerThread;
constexpr uint32_t NW = T / 32;

struct SmemRebin {
  uint32_t warp_sum[NW];
  uint32_t epoch;
  uint32_t flags;
  uint32_t wc[2 * kTileCells / CPT];  // tile prefixes of this block (write_table)
};

// Exclusive scan of one value per thread over the block.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v,
                                                         uint32_t& total,
                                                         uint32_t* warp_sum) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < NW ? warp_sum[lane] : 0u;
#pragma unroll
    for (uint32_t o = 1; o < NW; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < NW) warp_sum[lane] = s;
  }
  __syncthreads();
  const uint32_t warp_excl = warp ? warp_sum[warp - 1] : 0u;
  total = warp_sum[NW - 1];
  __syncthreads();
  return warp_excl + x - v;
}

// Grid-wide barrier over the co-resident blocks of a cooperative launch.
// The wait is bounded: past kWaitLimitNs it raises kFlagTimeout and returns.
__device__ void grid_barrier(Ctrl* ctrl, uint32_t& flags) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t gen = ld_acquire_u32(&ctrl->bar_gen);
    __threadfence();
    const uint32_t arrived = atomicAdd(&ctrl->bar_count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(&ctrl->bar_count, 0u);
      __threadfence();
      st_release_u32(&ctrl->bar_gen, gen + 1);
    } else if (!wait_while_equal(&ctrl->bar_gen, gen, kWaitLimitNs)) {
      flags |= kFlagTimeout;
    }
    __threadfence();
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Radix sort
// ---------------------------------------------------------------------------

// Items of a warp are ranked in steps of 32 (lane order = source order); the
// loads of kSeg steps are issued before they are consumed.
constexpr uint32_t kSeg = 8;

// Sum of one tile of kTileCells per-cell counts (L2-coherent loads).
__device__ __forceinline__ uint32_t tile_count_sum(const uint32_t* counts,
                                                   uint32_t tile, uint32_t n,
                                                   SmemRebin& sm) {
  const uint32_t c0 = tile * kTileCells + threadIdx.x * CPT;
  uint32_t s = 0;
#pragma unroll
  for (uint32_t u = 0; u < CPT; ++u) s += c0 + u < n ? __ldcg(counts + c0 + u) : 0u;
  uint32_t total;
  block_exclusive_scan(s, total, sm.warp_sum);
  return total;
}

// The cell-start table from the per-cell counts: every block scans the tile
// sums (each block reads all of them) for the prefixes of its own tiles,
// then writes its tiles' starts and zeroes their counts for the next launch.
__device__ void write_table(const RebinArgs& a, SmemRebin& sm) {
  const uint32_t t = threadIdx.x, n = a.ncells;
  const uint32_t ntiles = (n + kTileCells - 1) / kTileCells;
  const uint32_t per = (ntiles + T - 1) / T;
  const uint32_t i0 = min(t * per, ntiles), i1 = min(i0 + per, ntiles);
  uint32_t s = 0;
  for (uint32_t i = i0; i < i1; ++i) s += __ldcg(a.tile_sums + i);
  uint32_t total;
  const uint32_t excl = block_exclusive_scan(s, total, sm.warp_sum);
  // this block's tiles, kOwn at a time: their prefixes into shared memory,
  // then their starts
  constexpr uint32_t kOwn = sizeof(sm.wc) / sizeof(sm.wc[0]);
  const uint32_t G = gridDim.x, mine = ntiles > blockIdx.x ? (ntiles - blockIdx.x + G - 1) / G : 0u;
  for (uint32_t o0 = 0; o0 < mine; o0 += kOwn) {
    uint32_t run = excl;
    for (uint32_t i = i0; i < i1; ++i) {
      if (i % G == blockIdx.x && i / G >= o0 && i / G < o0 + kOwn) sm.wc[i / G - o0] = run;
      run += __ldcg(a.tile_sums + i);
    }
    __syncthreads();
    for (uint32_t o = o0; o < min(mine, o0 + kOwn); ++o) {
      const uint32_t tile = blockIdx.x + o * G;
      const uint32_t c0 = tile * kTileCells + t * CPT;
      uint32_t v[CPT];
#pragma unroll
      for (uint32_t u = 0; u < CPT; ++u) v[u] = c0 + u < n ? __ldcg(a.counts + c0 + u) : 0u;
      uint32_t agg;
      uint32_t acc = sm.wc[o - o0] + block_exclusive_scan(v[0] + v[1] + v[2] + v[3], agg, sm.warp_sum);
#pragma unroll
      for (uint32_t u = 0; u < CPT; ++u) {
        if (c0 + u < n) {
          a.cs_new[c0 + u] = acc;
          a.counts[c0 + u] = 0;
        }
        acc += v[u];
      }
    }
    __syncthreads();
  }
  if (blockIdx.x == 0 && t == 0) a.cs_new[n] = total;
}

// LSD radix sort of (key, source index) by key, stable, `a.digit_bits` bits
// per pass; the warp-private digit counters live in dynamic shared memory
// (NW * 2^digit_bits words).
__device__ void radix_sort(const RebinArgs& a, SmemRebin& sm, uint32_t* wcd,
                           uint32_t& flags, uint32_t& overflow) {
  const uint32_t G = gridDim.x, b = blockIdx.x, t = threadIdx.x;
  const uint32_t lane = t & 31, warp = t >> 5;
  const uint32_t lanemask_lt = (1u << lane) - 1u;
  const uint32_t n = a.n;
  const uint32_t chunk = (n + G - 1) / G;
  const uint32_t blo = min(b * chunk, n), bhi = min(blo + chunk, n);
  const uint32_t wsz = (bhi - blo + NW - 1) / NW;
  const uint32_t wlo = min(blo + warp * wsz, bhi), whi = min(wlo + wsz, bhi);
  const uint32_t DB = a.digit_bits, RADIX = 1u << DB, MASK = RADIX - 1u;
  const uint32_t passes = (a.key_bits + DB - 1) / DB;
  const uint32_t ntiles = (a.ncells + kTileCells - 1) / kTileCells;
  uint32_t* tot = a.hist + RADIX * G;
  uint32_t* wc = wcd + warp * RADIX;

  for (uint32_t p = 0; p < passes; ++p) {
    const uint32_t shift = DB * p;
    const uint32_t* sk = p == 0 ? a.keys : ((p & 1) ? a.kA : a.kB);
    const uint32_t* si = p == 0 ? nullptr : ((p & 1) ? a.iA : a.iB);
    uint32_t* dk = (p & 1) ? a.kB : a.kA;
    uint32_t* di = (p & 1) ? a.iB : a.iA;

    // A: digit histogram (warp-private counters); on the first pass also the
    // per-cell counts of the table
    for (uint32_t k = t; k < NW * RADIX; k += T) wcd[k] = 0;
    __syncthreads();
    for (uint32_t base = wlo; base < whi; base += 32 * kSeg) {
      uint32_t key[kSeg];
#pragma unroll
      for (uint32_t u = 0; u < kSeg; ++u) {
        const uint32_t i = base + 32 * u + lane;
        key[u] = i < whi ? __ldcg(sk + i) : 0xFFFFFFFFu;
      }
#pragma unroll
      for (uint32_t u = 0; u < kSeg; ++u) {
        const bool valid = key[u] != 0xFFFFFFFFu;
        if (p == 0 && valid && key[u] < a.ncells) atomicAdd(&a.counts[key[u]], 1u);
        const uint32_t d = valid ? (key[u] >> shift) & MASK : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        if (valid && (peers & lanemask_lt) == 0) wc[d] += __popc(peers);
        __syncwarp();
      }
    }
    __syncthreads();
    for (uint32_t d = t; d < RADIX; d += T) {
      uint32_t h = 0;
      for (uint32_t w = 0; w < NW; ++w) h += wcd[w * RADIX + d];
      a.hist[d * G + b] = h;
    }
    grid_barrier(a.ctrl, flags);

    // B: per digit, exclusive prefix over the blocks and the digit total;
    // on the first pass also the tile sums of the per-cell counts
    for (uint32_t d = b; d < RADIX; d += G) {
      const uint32_t per = (G + T - 1) / T;
      const uint32_t i0 = min(t * per, G), i1 = min(i0 + per, G);
      uint32_t s = 0;
      for (uint32_t i = i0; i < i1; ++i) s += __ldcg(a.hist + d * G + i);
      uint32_t total;
      uint32_t run = block_exclusive_scan(s, total, sm.warp_sum);
      for (uint32_t i = i0; i < i1; ++i) {
        const uint32_t v = __ldcg(a.hist + d * G + i);
        a.hist[d * G + i] = run;
        run += v;
      }
      if (t == 0) tot[d] = total;
    }
    if (p == 0)
      for (uint32_t tile = b; tile < ntiles; tile += G) {
        const uint32_t s = tile_count_sum(a.counts, tile, a.ncells, sm);
        if (t == 0) a.tile_sums[tile] = s;
      }
    grid_barrier(a.ctrl, flags);

    // C: running destinations of each (warp, digit), then the stable scatter
    {
      const uint32_t dpt = (RADIX + T - 1) / T;  // digits per thread
      const uint32_t d0 = min(t * dpt, RADIX), d1 = min(d0 + dpt, RADIX);
      uint32_t s = 0;
      for (uint32_t d = d0; d < d1; ++d) s += __ldcg(tot + d);
      uint32_t total;
      uint32_t doff = block_exclusive_scan(s, total, sm.warp_sum);
      for (uint32_t d = d0; d < d1; ++d) {
        uint32_t off = doff + __ldcg(a.hist + d * G + b);
        doff += __ldcg(tot + d);
        for (uint32_t w = 0; w < NW; ++w) {
          const uint32_t c = wcd[w * RADIX + d];
          wcd[w * RADIX + d] = off;
          off += c;
        }
      }
    }
    __syncthreads();
    for (uint32_t base = wlo; base < whi; base += 32 * kSeg) {
      uint32_t key[kSeg], idx[kSeg];
#pragma unroll
      for (uint32_t u = 0; u < kSeg; ++u) {
        const uint32_t i = base + 32 * u + lane;
        key[u] = i < whi ? __ldcg(sk + i) : 0xFFFFFFFFu;
        idx[u] = i < whi ? (si ? __ldcg(si + i) : i) : 0u;
      }
#pragma unroll
      for (uint32_t u = 0; u < kSeg; ++u) {
        const bool valid = key[u] != 0xFFFFFFFFu;
        const uint32_t d = valid ? (key[u] >> shift) & MASK : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t start = valid ? wc[d] : 0u;
        __syncwarp();
        if (valid) {
          const uint32_t rank = __popc(peers & lanemask_lt);
          if ((peers >> lane) == 1u) wc[d] = start + __popc(peers);
          const uint32_t dst = start + rank;
          if (dst < n) {  // always true unless a barrier timed out
            dk[dst] = key[u];
            di[dst] = idx[u];
          }
        }
        __syncwarp();
      }
    }
    grid_barrier(a.ctrl, flags);
  }

  // gather into cell order, then the table
  const uint32_t last = passes - 1;
  const uint32_t* sk = (last & 1) ? a.kB : a.kA;
  const uint32_t* si = (last & 1) ? a.iB : a.iA;
  for (uint32_t i = b * T + t; i < n; i += G * T) {
    const uint32_t k = __ldcg(sk + i);
    if (k >= a.ncells) continue;
    const uint32_t s = __ldcg(si + i);
    if (i < a.dst_capacity && s < n) {
      a.pos_dst[i] = a.pos_src[s];
      a.vel_dst[i] = a.vel_src[s];
      a.cell_dst[i] = k;
    } else {
      ++overflow;
    }
  }
  write_table(a, sm);
}

__global__ void __launch_bounds__(T, 3) k_rebin(RebinArgs a) {
  __shared__ SmemRebin sm;
  extern __shared__ uint32_t wcd[];
  const uint32_t t = threadIdx.x;
  uint32_t flags = 0, overflow = 0;
  if (t == 0) {
    sm.epoch = ld_acquire_u32(&a.ctrl->epoch);
    sm.flags = 0;
  }
  __syncthreads();
  radix_sort(a, sm, wcd, flags, overflow);
  // flags and overflow of the block, then the exit protocol: the last block
  // out counts the launch.
  const uint32_t wf = warp_or_u32(flags);
  const uint32_t wo = __reduce_add_sync(0xffffffffu, overflow);
  if ((t & 31) == 0) {
    if (wf) atomicOr(&sm.flags, wf);
    if (wo) atomicAdd(&a.ctrl->overflow, wo);
  }
  __syncthreads();
  if (t == 0) {
    if (sm.flags) atomicOr(&a.ctrl->flags, sm.flags);
    __threadfence();
    const uint32_t done = atomicAdd(&a.ctrl->exit_count, 1u);
    if (done == gridDim.x - 1) {
      if (!a.force_general) a.ctrl->frames += 1;
      atomicExch(&a.ctrl->exit_count, 0u);
      __threadfence();
      st_release_u32(&a.ctrl->epoch, sm.epoch + 1);
    }
  }
}

}  // namespace

uint32_t rebin_digit_bits(uint32_t key_bits) {
  const uint32_t kb = key_bits ? key_bits : 1u;
  const uint32_t passes = (kb + kMaxDigitBits - 1) / kMaxDigitBits;
  return (kb + passes - 1) / passes;
}

size_t rebin_dynamic_smem(uint32_t digit_bits) {
  return (size_t)NW * ((size_t)1 << digit_bits) * sizeof(uint32_t);
}

int rebin_grid_size(int device, uint32_t digit_bits) {
  const size_t dyn = rebin_dynamic_smem(digit_bits);
  if (cudaFuncSetAttribute(k_rebin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) !=
      cudaSuccess)
    return 0;
  int sms = 0, per_sm = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rebin, T, dyn) != cudaSuccess)
    return 0;
  return sms * per_sm;
}

cudaError_t launch_rebin(const RebinArgs& a, int grid, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(T);
  cfg.dynamicSmemBytes = rebin_dynamic_smem(a.digit_bits);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_rebin, a);
}

namespace {

// SpatialBin::get_cell_coord (runners/bevy/src/spatial_bin.rs:48-64):
// Rust's f32::div_euclid then a saturating `as i32` (NaN -> 0).
__device__ __forceinline__ int32_t cell_coord_euclid(float x, uint32_t cs) {
  const float d = (float)cs;
  float q = truncf(__fdiv_rn(x, d));
  if (fmodf(x, d) < 0.0f) q = __fsub_rn(q, 1.0f);
  if (q != q) return 0;
  if (q >= 2147483648.0f) return INT_MAX;
  if (q <= -2147483648.0f) return INT_MIN;
  return (int32_t)q;
}

__global__ void k_upload_keys(const WorldDev* __restrict__ worlds, int nworlds,
                              uint32_t ncells, uint32_t target,
                              uint32_t n_keep,
                              const uint32_t* __restrict__ cell_of,
                              uint32_t n_new,
                              const float2* __restrict__ new_pos,
                              uint32_t* __restrict__ keys) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_keep) {
    const uint32_t k = cell_of[i];
    keys[i] = (uint32_t)world_of_cell(worlds, nworlds, k) == target ? ncells : k;
  } else if (i < n_keep + n_new) {
    const WorldDev w = worlds[target];
    const float2 p = new_pos[i - n_keep];
    const int64_t cx = (int64_t)cell_coord_euclid(p.x, w.cs) - w.blx;
    const int64_t cy = (int64_t)cell_coord_euclid(p.y, w.cs) - w.bly;
    keys[i] = (cx < 0 || cy < 0 || cx >= (int64_t)w.gx || cy >= (int64_t)w.gy)
                  ? ncells
                  : w.cell_off + (uint32_t)cy * w.gx + (uint32_t)cx;
  }
}

__global__ void k_world_table(const uint32_t* __restrict__ cell_start,
                              uint32_t cell_off, uint32_t cells,
                              uint32_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t base = cell_start[cell_off];
  if (i == 0) out[0] = 0;
  if (i <= cells) out[i + 1] = cell_start[cell_off + i] - base;
}

}  // namespace

namespace {

// The bounded wait on a word: out[0] = 1 if it gave up, out[1] = the
// microseconds it waited.
__global__ void k_wait_probe(const uint32_t* word, uint32_t value, uint64_t limit_ns,
                             uint32_t* out) {
  const uint64_t t0 = global_ns();
  const bool changed = wait_while_equal(word, value, limit_ns);
  out[0] = changed ? 0u : 1u;
  out[1] = (uint32_t)((global_ns() - t0) / 1000u);
}

}  // namespace

cudaError_t launch_wait_probe(const uint32_t* word, uint32_t value, uint64_t limit_ns,
                              uint32_t* out, cudaStream_t st) {
  k_wait_probe<<<1, 1, 0, st>>>(word, value, limit_ns, out);
  return cudaGetLastError();
}

cudaError_t launch_upload_keys(const WorldDev* worlds, int nworlds,
                               uint32_t ncells, uint32_t target,
                               uint32_t n_keep, const uint32_t* cell_of,
                               uint32_t n_new, const float2* new_pos,
                               uint32_t* keys, cudaStream_t st) {
  const uint32_t n = n_keep + n_new;
  if (n == 0) return cudaSuccess;
  k_upload_keys<<<(n + 255) / 256, 256, 0, st>>>(
      worlds, nworlds, ncells, target, n_keep, cell_of, n_new, new_pos, keys);
  return cudaGetLastError();
}

namespace {

__global__ void k_local_keys(const uint32_t* __restrict__ cell_of, uint32_t n, uint32_t cell_off,
                             uint32_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = cell_of[i] - cell_off;
}

}  // namespace

cudaError_t launch_local_keys(const uint32_t* cell_of, uint32_t n, uint32_t cell_off,
                              uint32_t* out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_local_keys<<<(n + 255) / 256, 256, 0, st>>>(cell_of, n, cell_off, out);
  return cudaGetLastError();
}

cudaError_t launch_world_table(const uint32_t* cell_start, uint32_t cell_off,
                               uint32_t cells, uint32_t* out, cudaStream_t st) {
  const uint32_t n = cells + 1;
  k_world_table<<<(n + 255) / 256, 256, 0, st>>>(cell_start, cell_off, cells,
                                                  out);
  return cudaGetLastError();
}

}  // namespace wrach
