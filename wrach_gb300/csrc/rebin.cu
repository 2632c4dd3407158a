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
// Windowed path (every frame whose particles moved at most kMaxWindow cells):
// the source is in old-cell order, so every particle that lands in cell k
// comes from the (2R+1)^2 old cells around k, R = the frame's largest cell
// displacement.  Walking those old cells in row-major order visits them in
// source order, which gives each destination cell its count and, on a second
// walk, each particle's stable rank.  The counts are scanned in one pass with
// decoupled look-back over tiles of kTileCells consecutive cells, so the
// table, the scan and the scatter take a single launch.
//
// General path (uploads, or a frame that moved a particle further): an LSD
// radix sort (8-bit digits) of (key, source index) over the whole grid of
// co-resident blocks with grid barriers, then a gather and a table built by
// binary search.
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
  uint32_t tile;
  uint32_t tile_excl;
  uint32_t epoch;
  uint32_t dmax;
  uint32_t flags;
  uint32_t run[256];
  uint32_t wc[NW * 256];
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
    } else {
      const uint64_t t0 = global_ns();
      while (ld_acquire_u32(&ctrl->bar_gen) == gen) {
        if (global_ns() - t0 > kWaitLimitNs) {
          flags |= kFlagTimeout;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Windowed path
// ---------------------------------------------------------------------------

// Walk the old cells within R of cells [xa, xb] of row cy (keys
// kbase .. kbase + nk - 1) in source order.  Count mode adds to cnt[];
// scatter mode uses cnt[] as the running destination of each cell.
template <bool SCATTER>
__device__ __forceinline__ void walk_row(const RebinArgs& a, const WorldDev& w,
                                         uint32_t cy, uint32_t xa, uint32_t xb,
                                         uint32_t kbase, uint32_t nk,
                                         uint32_t R, uint32_t (&cnt)[CPT],
                                         uint32_t& overflow) {
  const uint32_t xlo = xa >= R ? xa - R : 0u;
  const uint32_t xhi = min(xb + R, w.gx - 1);
  const uint32_t ylo = cy >= R ? cy - R : 0u;
  const uint32_t yhi = min(cy + R, w.gy - 1);
  for (uint32_t row = ylo; row <= yhi; ++row) {
    const uint32_t rb = w.cell_off + row * w.gx;
    // clamped so that an inconsistent table can never index past the source
    const uint32_t je = min(a.cs_old[rb + xhi + 1], a.n);
    const uint32_t js = min(a.cs_old[rb + xlo], je);
    for (uint32_t j = js; j < je; ++j) {
      const uint32_t d = a.keys[j] - kbase;
      if (d >= nk) continue;
      if (SCATTER) {
        uint32_t dst = 0;
#pragma unroll
        for (uint32_t u = 0; u < CPT; ++u)
          if (d == u) dst = cnt[u]++;
        if (dst < a.dst_capacity) {
          a.pos_dst[dst] = a.pos_src[j];
          a.vel_dst[dst] = a.vel_src[j];
          a.cell_dst[dst] = kbase + d;
        } else {
          ++overflow;
        }
      } else {
#pragma unroll
        for (uint32_t u = 0; u < CPT; ++u) cnt[u] += (d == u);
      }
    }
  }
}

template <bool SCATTER>
__device__ __forceinline__ void walk_cells(const RebinArgs& a, uint32_t c0,
                                           uint32_t ncell, uint32_t R,
                                           uint32_t (&cnt)[CPT],
                                           uint32_t& overflow) {
  const WorldDev w = a.worlds[world_of_cell(a.worlds, a.nworlds, c0)];
  const uint32_t l0 = c0 - w.cell_off;
  const uint32_t cy = l0 / w.gx, cx0 = l0 % w.gx;
  if (cx0 + ncell <= w.gx) {
    // all of this thread's cells sit in one row of one world: one walk
    walk_row<SCATTER>(a, w, cy, cx0, cx0 + ncell - 1, c0, ncell, R, cnt,
                      overflow);
    return;
  }
  // the cells straddle a row (or world) boundary: one walk per cell
#pragma unroll
  for (uint32_t u = 0; u < CPT; ++u) {
    if (u < ncell) {
      const uint32_t c = c0 + u;
      const WorldDev wu = a.worlds[world_of_cell(a.worlds, a.nworlds, c)];
      const uint32_t l = c - wu.cell_off;
      uint32_t one[CPT] = {};
      one[0] = cnt[u];
      walk_row<SCATTER>(a, wu, l / wu.gx, l % wu.gx, l % wu.gx, c, 1, R, one,
                        overflow);
      cnt[u] = one[0];
    }
  }
}

__device__ void windowed_tile(const RebinArgs& a, uint32_t tile, uint32_t R,
                              SmemRebin& sm, uint32_t& flags,
                              uint32_t& overflow) {
  const uint32_t t = threadIdx.x;
  const uint32_t c0 = tile * kTileCells + t * CPT;
  const uint32_t ncell = c0 < a.ncells ? min(CPT, a.ncells - c0) : 0u;
  uint32_t cnt[CPT] = {};
  if (ncell) walk_cells<false>(a, c0, ncell, R, cnt, overflow);
  uint32_t mine = 0;
#pragma unroll
  for (uint32_t u = 0; u < CPT; ++u) mine += cnt[u];
  uint32_t agg;
  const uint32_t excl_t = block_exclusive_scan(mine, agg, sm.warp_sum);

  // decoupled look-back (warp 0)
  if (t < 32) {
    const uint32_t lane = t;
    const uint64_t tag = (uint64_t)(sm.epoch & 0x3FFFFFFFu) << 34;
    if (lane == 0)
      st_release_u64(&a.status[tile],
                     tag | ((tile == 0 ? 2ull : 1ull) << 32) | agg);
    uint32_t excl = 0;
    if (tile > 0) {
      int64_t base = (int64_t)tile - 1;
      while (true) {
        const int64_t j = base - (int64_t)lane;
        uint32_t flag = 2u, val = 0u;
        if (j >= 0) {
          const uint64_t t0 = global_ns();
          uint64_t s;
          while (true) {
            s = ld_acquire_u64(&a.status[j]);
            if ((s >> 34) == (tag >> 34) && ((s >> 32) & 3ull) != 0) break;
            if (global_ns() - t0 > kWaitLimitNs) {
              flags |= kFlagTimeout;
              s = tag | (2ull << 32);
              break;
            }
          }
          flag = (uint32_t)((s >> 32) & 3ull);
          val = (uint32_t)s;
        }
        const uint32_t pmask = __ballot_sync(0xffffffffu, flag == 2u);
        if (pmask) {
          const uint32_t first = __ffs(pmask) - 1;
          excl += __reduce_add_sync(0xffffffffu, lane <= first ? val : 0u);
          break;
        }
        excl += __reduce_add_sync(0xffffffffu, val);
        base -= 32;
      }
      if (lane == 0)
        st_release_u64(&a.status[tile], tag | (2ull << 32) | (excl + agg));
    }
    if (lane == 0) sm.tile_excl = excl;
  }
  __syncthreads();
  const uint32_t tile_excl = sm.tile_excl;

  uint32_t run[CPT];
  uint32_t acc = tile_excl + excl_t;
#pragma unroll
  for (uint32_t u = 0; u < CPT; ++u) {
    run[u] = acc;
    acc += cnt[u];
  }
  if (ncell == CPT) {
    *reinterpret_cast<uint4*>(a.cs_new + c0) =
        make_uint4(run[0], run[1], run[2], run[3]);
  } else {
#pragma unroll
    for (uint32_t u = 0; u < CPT; ++u)
      if (u < ncell) a.cs_new[c0 + u] = run[u];
  }
  if (tile == a.ntiles - 1 && t == 0) a.cs_new[a.ncells] = tile_excl + agg;
  if (ncell) walk_cells<true>(a, c0, ncell, R, run, overflow);
  __syncthreads();  // smem reuse by the next tile
}

// ---------------------------------------------------------------------------
// General path
// ---------------------------------------------------------------------------

__device__ void block_scan_inplace(uint32_t* arr, uint32_t n, SmemRebin& sm) {
  const uint32_t t = threadIdx.x;
  const uint32_t per = (n + T - 1) / T;
  const uint32_t lo = min(t * per, n), hi = min(lo + per, n);
  uint32_t s = 0;
  for (uint32_t i = lo; i < hi; ++i) s += __ldcg(arr + i);
  uint32_t total;
  uint32_t run = block_exclusive_scan(s, total, sm.warp_sum);
  for (uint32_t i = lo; i < hi; ++i) {
    const uint32_t v = __ldcg(arr + i);
    arr[i] = run;
    run += v;
  }
}

__device__ __forceinline__ uint32_t lower_bound_cg(const uint32_t* a,
                                                   uint32_t n, uint32_t key) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldcg(a + mid) < key)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

__device__ void general_sort(const RebinArgs& a, SmemRebin& sm,
                             uint32_t& flags, uint32_t& overflow) {
  const uint32_t G = gridDim.x, b = blockIdx.x, t = threadIdx.x;
  const uint32_t lane = t & 31, warp = t >> 5;
  const uint32_t n = a.n;
  const uint32_t chunk = ((n + G - 1) / G + T - 1) / T * T;
  const uint32_t lo = min(b * chunk, n), hi = min(lo + chunk, n);
  const uint32_t passes = a.key_bits ? (a.key_bits + 7) / 8 : 1u;
  const uint32_t lanemask_lt = (1u << lane) - 1u;

  for (uint32_t p = 0; p < passes; ++p) {
    const uint32_t shift = 8 * p;
    const uint32_t* sk = p == 0 ? a.keys : ((p & 1) ? a.kA : a.kB);
    const uint32_t* si = p == 0 ? nullptr : ((p & 1) ? a.iA : a.iB);
    uint32_t* dk = (p & 1) ? a.kB : a.kA;
    uint32_t* di = (p & 1) ? a.iB : a.iA;

    // digit histogram of this block's chunk
    sm.run[t] = 0;
    __syncthreads();
    for (uint32_t i = lo + t; i < hi; i += T)
      atomicAdd(&sm.run[(__ldcg(sk + i) >> shift) & 255u], 1u);
    __syncthreads();
    a.hist[t * G + b] = sm.run[t];
    grid_barrier(a.ctrl, flags);

    // digit-major exclusive scan of all blocks' histograms
    if (b == 0) block_scan_inplace(a.hist, 256 * G, sm);
    grid_barrier(a.ctrl, flags);

    // stable scatter, sub-tiles of T items in source order
    sm.run[t] = __ldcg(a.hist + t * G + b);
    __syncthreads();
    for (uint32_t base = lo; base < hi; base += T) {
      const uint32_t i = base + t;
      const bool valid = i < hi;
      const uint32_t key = valid ? __ldcg(sk + i) : 0u;
      const uint32_t idx = valid ? (si ? __ldcg(si + i) : i) : 0u;
      const uint32_t d = valid ? (key >> shift) & 255u : 256u;
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      const uint32_t rank = __popc(peers & lanemask_lt);
      for (uint32_t k = t; k < NW * 256; k += T) sm.wc[k] = 0;
      __syncthreads();
      if (valid && rank == 0) sm.wc[warp * 256 + d] = __popc(peers);
      __syncthreads();
      {
        uint32_t run = sm.run[t];
#pragma unroll
        for (uint32_t w = 0; w < NW; ++w) {
          const uint32_t c = sm.wc[w * 256 + t];
          sm.wc[w * 256 + t] = run;
          run += c;
        }
        sm.run[t] = run;
      }
      __syncthreads();
      if (valid) {
        const uint32_t dst = sm.wc[warp * 256 + d] + rank;
        if (dst < n) {  // always true unless a barrier timed out
          dk[dst] = key;
          di[dst] = idx;
        }
      }
      __syncthreads();
    }
    grid_barrier(a.ctrl, flags);
  }

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
  for (uint32_t c = b * T + t; c <= a.ncells; c += G * T)
    a.cs_new[c] = lower_bound_cg(sk, n, c);
}

__global__ void __launch_bounds__(T) k_rebin(RebinArgs a) {
  __shared__ SmemRebin sm;
  const uint32_t t = threadIdx.x;
  uint32_t flags = 0, overflow = 0;
  if (t == 0) {
    sm.epoch = ld_acquire_u32(&a.ctrl->epoch);
    sm.dmax = ld_acquire_u32(&a.ctrl->dmax);
    sm.flags = 0;
  }
  __syncthreads();
  const uint32_t R = sm.dmax;
  const bool general = a.force_general || R > kMaxWindow;
  if (general) {
    if (!a.force_general && blockIdx.x == 0 && t == 0) {
      atomicAdd(&a.ctrl->general, 1u);
      flags |= kFlagGeneralSort;
    }
    general_sort(a, sm, flags, overflow);
  } else {
    while (true) {
      if (t == 0) sm.tile = atomicAdd(&a.ctrl->ticket, 1u);
      __syncthreads();
      const uint32_t tile = sm.tile;
      __syncthreads();
      if (tile >= a.ntiles) break;
      windowed_tile(a, tile, R, sm, flags, overflow);
    }
  }
  // flags and overflow of the block, then the exit protocol: the last block
  // out resets the per-launch counters and advances the epoch.
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
      atomicExch(&a.ctrl->ticket, 0u);
      atomicExch(&a.ctrl->dmax, 0u);
      atomicExch(&a.ctrl->exit_count, 0u);
      __threadfence();
      st_release_u32(&a.ctrl->epoch, sm.epoch + 1);
    }
  }
}

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

int rebin_grid_size(int device) {
  int sms = 0, per_sm = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) !=
      cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rebin, T, 0) !=
      cudaSuccess)
    return 0;
  return sms * per_sm;
}

cudaError_t launch_rebin(const RebinArgs& a, int grid, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(T);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_rebin, a);
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

cudaError_t launch_world_table(const uint32_t* cell_start, uint32_t cell_off,
                               uint32_t cells, uint32_t* out, cudaStream_t st) {
  const uint32_t n = cells + 1;
  k_world_table<<<(n + 255) / 256, 256, 0, st>>>(cell_start, cell_off, cells,
                                                  out);
  return cudaGetLastError();
}

}  // namespace wrach
