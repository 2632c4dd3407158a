// Rebin as a stable counting sort over the cells: the count, scan and pack
// passes of a frame (assets/shaders/particles_per_cell.wgsl, prefix_sum.wgsl,
// pack_new_particle_data.wgsl; dispatched by runners/bevy/src/compute/
// builder.rs:86-89) as a chain of five short launches.
//
//   count    per warp, the particles of one cell (__match_any_sync) take one
//            atomic on the cell's counter; each particle's ticket (its slot
//            inside the cell, arrival order) is the returned base plus its
//            rank among the warp's particles of that cell; per warp one more
//            atomic adds the particles of each tile of 2048 cells to the
//            tile's sum.  A frame of the extended physics takes the tickets
//            in its last Jacobi pass instead (the keys are computed there)
//   scan     exclusive scan of the per-cell counts, one block per tile of
//            2048 cells; a tile's prefix is the sum of the earlier tiles'
//            sums (already final, so no block waits): each block adds them
//            up itself, or, past kPrefixTiles tiles (where that sum grows
//            with the square of the grid), a one-block launch first turns
//            the tile sums into their prefixes; it writes the
//            cell-start table and (extended physics) the capped table of the
//            taking-part particles from the counts capped at the cell
//            capacity, and lists the cells of more than kSmallCell particles
//            (the pass that takes the tickets empties that list first); the
//            place steps clear the counts of the non-empty cells afterwards
//   scatter  source index and cell of every particle to table start + ticket
//            (arrival order inside a cell)
//   place    the stable order: inside a cell, a particle's rank is the number
//            of the cell's particles with a smaller source index; then the
//            gather of positions, velocities and cells into that slot, and of
//            the taking-part particles' positions, velocities and cells into
//            the compacted arrays.  Cells of up to kSmallCell particles are
//            ranked by one thread per slot
//   cells    one block per listed cell: up to kBigCell particles a bitonic
//            sort of the source indices in shared memory, more than that a
//            block-wide LSD radix sort of them in global memory; then the
//            gather.  It writes other slots than place, so the two may run
//            at the same time
//
// The result is the stable order (a cell's particles keep their source
// order), the order of the oracle's counting sort and of rebin.cu's radix
// sort.
#include "wrach_internal.cuh"
#include "wrach_kernels.h"

namespace wrach {

namespace {

constexpr uint32_t kScanThreads = 256, kScanPer = 8;
constexpr uint32_t kScanTile = kScanThreads * kScanPer;
static_assert(kScanTile == kCountScanTile, "tile size shared with the tickets' tile sums");

__global__ void __launch_bounds__(256) k_cs_count(RebinArgs a) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t lane = threadIdx.x & 31;
  if (i == 0) a.ctrl->big_count = 0u;  // the scan lists this rebin's large cells
  // whole warps walk the particles, so every lane takes part in the match
  for (uint32_t base = i - lane; base < a.n; base += stride) {
    const uint32_t j = base + lane;
    const uint32_t k = j < a.n ? a.keys[j] : a.ncells;
    const uint32_t t = warp_ticket(k, a.ncells, a.counts, a.tile_sums, kCountScanShift, a.tp_cap,
                                   a.tp_cap ? a.tile_sums_cap : nullptr);
    if (j < a.n) a.ticket[j] = t;
  }
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* red) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = __reduce_add_sync(0xffffffffu, v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  uint32_t s = 0;
#pragma unroll
  for (uint32_t w = 0; w < kScanThreads / 32; ++w) s += red[w];
  return s;
}

// One block per tile of 2048 cells.  The tile's prefix is the sum of the
// earlier tiles' counts, which the tickets' pass has already totalled, so no
// block waits for another.
// Past this many tiles of the table, the tile sums are turned into prefixes
// by k_cs_tile_prefix first.
constexpr uint32_t kPrefixTiles = 2048;

// One block of 1024 threads: the tile sums (and the capped ones) replaced by
// their exclusive prefixes, in place; each thread scans a contiguous run.
__global__ void __launch_bounds__(1024) k_cs_tile_prefix(RebinArgs a, uint32_t ntiles) {
  __shared__ uint32_t ws[32], wc[32];
  const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t per = (ntiles + 1023) / 1024;
  const uint32_t i0 = min(t * per, ntiles), i1 = min(i0 + per, ntiles);
  const bool cap = a.tp_cap != 0u;
  uint32_t s = 0, c = 0;
  for (uint32_t i = i0; i < i1; ++i) {
    s += __ldcg(a.tile_sums + i);
    if (cap) c += __ldcg(a.tile_sums_cap + i);
  }
  uint32_t x = s, y = c;
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, x, o), v = __shfl_up_sync(0xffffffffu, y, o);
    if (lane >= o) {
      x += u;
      y += v;
    }
  }
  if (lane == 31) {
    ws[warp] = x;
    wc[warp] = y;
  }
  __syncthreads();
  uint32_t bs = 0, bc = 0;
  for (uint32_t w = 0; w < warp; ++w) {
    bs += ws[w];
    bc += wc[w];
  }
  uint32_t run = bs + x - s, crun = bc + y - c;
  for (uint32_t i = i0; i < i1; ++i) {
    const uint32_t v = __ldcg(a.tile_sums + i);
    a.tile_sums[i] = run;
    run += v;
    if (cap) {
      const uint32_t w = __ldcg(a.tile_sums_cap + i);
      a.tile_sums_cap[i] = crun;
      crun += w;
    }
  }
}

__global__ void __launch_bounds__(kScanThreads) k_cs_scan(RebinArgs a) {
  __shared__ uint32_t warp_sum[kScanThreads / 32], red[kScanThreads / 32];
  __shared__ uint32_t warp_cap[kScanThreads / 32];
  const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t tile = blockIdx.x, n = a.ncells;
  if (tile == 0 && t == 0 && !a.force_general) a.ctrl->frames += 1;
  const uint32_t c0 = tile * kScanTile + t * kScanPer;
  uint32_t v[kScanPer];
  if (c0 + kScanPer <= n) {
    const uint4* src = reinterpret_cast<const uint4*>(a.counts + c0);
#pragma unroll
    for (uint32_t u = 0; u < kScanPer / 4; ++u) {
      const uint4 q = __ldcg(src + u);
      v[4 * u] = q.x; v[4 * u + 1] = q.y; v[4 * u + 2] = q.z; v[4 * u + 3] = q.w;
    }
  } else {
#pragma unroll
    for (uint32_t u = 0; u < kScanPer; ++u) v[u] = c0 + u < n ? __ldcg(a.counts + c0 + u) : 0u;
  }
  // the capped counts (the taking-part particles) when the capped table is wanted
  const uint32_t cap = a.tp_cap;
  uint32_t sum = 0, csum = 0;
#pragma unroll
  for (uint32_t u = 0; u < kScanPer; ++u) {
    sum += v[u];
    csum += min(v[u], cap);
  }
  // the earlier tiles' totals
  uint32_t prefix, cprefix;
  if (a.tiles_prefixed) {
    prefix = __ldcg(a.tile_sums + tile);
    cprefix = cap ? __ldcg(a.tile_sums_cap + tile) : 0u;
  } else {
    uint32_t pre = 0, cpre = 0;
    for (uint32_t u = t; u < tile; u += kScanThreads) {
      pre += __ldcg(a.tile_sums + u);
      if (cap) cpre += __ldcg(a.tile_sums_cap + u);
    }
    prefix = block_sum(pre, red);
    cprefix = cap ? block_sum(cpre, red) : 0u;
  }
  // block-wide exclusive scans of the per-thread sums
  uint32_t x = sum, cx = csum;
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    const uint32_t cy = __shfl_up_sync(0xffffffffu, cx, o);
    if (lane >= o) {
      x += y;
      cx += cy;
    }
  }
  if (lane == 31) {
    warp_sum[warp] = x;
    warp_cap[warp] = cx;
  }
  __syncthreads();
  uint32_t before = 0, total = 0, cbefore = 0, ctotal = 0;
#pragma unroll
  for (uint32_t w = 0; w < kScanThreads / 32; ++w) {
    before += w < warp ? warp_sum[w] : 0u;
    total += warp_sum[w];
    cbefore += w < warp ? warp_cap[w] : 0u;
    ctotal += warp_cap[w];
  }
  uint32_t run = prefix + before + x - sum;
  uint32_t crun = cprefix + cbefore + cx - csum;
  // the large cells' work list (at most n / (kSmallCell + 1) cells qualify,
  // and big_cap is larger)
#pragma unroll
  for (uint32_t u = 0; u < kScanPer; ++u) {
    if (v[u] > kSmallCell) {
      const uint32_t w = atomicAdd(&a.ctrl->big_count, 1u);
      if (w < a.big_cap) a.big_list[w] = c0 + u;
    }
  }
  if (cap) {
    // the capped table (compacted starts of the cells' taking-part particles)
    if (c0 + kScanPer <= n) {
      uint4* dst = reinterpret_cast<uint4*>(a.ct_new + c0);
#pragma unroll
      for (uint32_t u = 0; u < kScanPer / 4; ++u) {
        uint4 q;
        q.x = crun; crun += min(v[4 * u], cap);
        q.y = crun; crun += min(v[4 * u + 1], cap);
        q.z = crun; crun += min(v[4 * u + 2], cap);
        q.w = crun; crun += min(v[4 * u + 3], cap);
        dst[u] = q;
      }
    } else {
#pragma unroll
      for (uint32_t u = 0; u < kScanPer; ++u) {
        if (c0 + u < n) a.ct_new[c0 + u] = crun;
        crun += min(v[u], cap);
      }
    }
    if (t == 0 && (tile + 1) * kScanTile >= n) a.ct_new[n] = cprefix + ctotal;
  }
  if (c0 + kScanPer <= n) {
    uint4* dst = reinterpret_cast<uint4*>(a.cs_new + c0);
#pragma unroll
    for (uint32_t u = 0; u < kScanPer / 4; ++u) {
      uint4 q;
      q.x = run; run += v[4 * u];
      q.y = run; run += v[4 * u + 1];
      q.z = run; run += v[4 * u + 2];
      q.w = run; run += v[4 * u + 3];
      dst[u] = q;
    }
  } else {
#pragma unroll
    for (uint32_t u = 0; u < kScanPer; ++u) {
      if (c0 + u < n) a.cs_new[c0 + u] = run;
      run += v[u];
    }
  }
  if (t == 0 && (tile + 1) * kScanTile >= n) a.cs_new[n] = prefix + total;
}

__global__ void __launch_bounds__(256) k_cs_scatter(RebinArgs a, uint32_t ntiles) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  // the scan has read the tile sums: clear them for the next rebin
  for (uint32_t u = i; u < ntiles; u += gridDim.x * blockDim.x) {
    a.tile_sums[u] = 0u;
    if (a.tp_cap) a.tile_sums_cap[u] = 0u;
  }
  if (i >= a.n) return;
  const uint32_t k = a.keys[i];
  if (k >= a.ncells) return;
  const uint32_t dst = a.cs_new[k] + a.ticket[i];
  if (dst < a.n) {  // always true unless the scan timed out
    a.idx_tmp[dst] = i;
    a.cell_tmp[dst] = k;
  }
}

// The particle of source index `src` into `slot`, rank `rank` inside its
// cell; a taking-part one (rank < tp_cap) also into the compacted arrays.
__device__ __forceinline__ void place_one(const RebinArgs& a, uint32_t slot, uint32_t rank,
                                          uint32_t src, uint32_t cell, uint32_t& overflow) {
  if (slot < a.dst_capacity && src < a.n) {
    const float2 p = a.pos_src[src], v = a.vel_src[src];
    a.pos_dst[slot] = p;
    a.vel_dst[slot] = v;
    a.cell_dst[slot] = cell;
    if (rank < a.tp_cap) {
      const uint32_t t = a.ct_new[cell] + rank;
      if (t < a.dst_capacity) {  // always true unless the scan timed out
        a.tp_pos[t] = p;
        a.tp_vel[t] = v;
        a.tp_cell[t] = cell;
      }
    }
  } else {
    ++overflow;
  }
}

__device__ __forceinline__ void add_overflow(const RebinArgs& a, uint32_t overflow) {
  const uint32_t wo = __reduce_add_sync(0xffffffffu, overflow);
  if ((threadIdx.x & 31) == 0 && wo) atomicAdd(&a.ctrl->overflow, wo);
}

__global__ void __launch_bounds__(256) k_cs_place(RebinArgs a) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t total = a.cs_new[a.ncells];
  uint32_t overflow = 0;
  // the guards below only matter if the scan timed out (table inconsistent)
  const uint32_t k = q < total && q < a.n ? a.cell_tmp[q] : a.ncells;
  const uint32_t c0 = k < a.ncells ? a.cs_new[k] : 0u;
  const uint32_t c1 = k < a.ncells ? a.cs_new[k + 1] : 0u;
  // larger cells are the scan's work list, placed by k_cs_big
  if (k < a.ncells && c1 - c0 <= kSmallCell) {
    const uint32_t s1 = min(c1, min(total, a.n));
    const uint32_t me = a.idx_tmp[q];
    // the particle's data and its cell's compacted start do not depend on
    // its rank: their loads go out before the rank's
    const bool src_ok = me < a.n;
    const float2 p = src_ok ? a.pos_src[me] : make_float2(0.f, 0.f);
    const float2 v = src_ok ? a.vel_src[me] : make_float2(0.f, 0.f);
    const uint32_t tp0 = a.tp_cap ? a.ct_new[k] : 0u;
    uint32_t rank = 0;
    for (uint32_t m = c0; m < s1; ++m) rank += a.idx_tmp[m] < me ? 1u : 0u;
    const uint32_t slot = c0 + rank;
    if (slot < a.dst_capacity && src_ok) {
      a.pos_dst[slot] = p;
      a.vel_dst[slot] = v;
      a.cell_dst[slot] = k;
      if (rank < a.tp_cap) {
        const uint32_t t = tp0 + rank;
        if (t < a.dst_capacity) {  // always true unless the scan timed out
          a.tp_pos[t] = p;
          a.tp_vel[t] = v;
          a.tp_cell[t] = k;
        }
      }
    } else {
      ++overflow;
    }
    // the scan has read the cell's count: zero for the next rebin (only
    // non-empty cells were counted)
    if (rank == 0) a.counts[k] = 0u;
  }
  add_overflow(a, overflow);
}

constexpr uint32_t kBigThreads = 256;
static_assert(kBigThreads == 256, "one radix digit per thread");

// Stable block-wide LSD radix sort (8-bit digits) of the m values src[0..m)
// into src or alt (returned), in chunks of 256 values: inside a chunk a
// value's slot is its digit's running offset, plus the counts of its digit
// in the chunk's earlier warps, plus its rank among its warp's equal digits.
__device__ uint32_t* block_radix_sort(uint32_t* src, uint32_t* alt, uint32_t m, uint32_t key_bits) {
  __shared__ uint32_t hist[256], wcnt[kBigThreads / 32][256];
  const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t lanemask_lt = (1u << lane) - 1u;
  for (uint32_t shift = 0; shift < key_bits; shift += 8) {
    hist[t] = 0u;
    __syncthreads();
    for (uint32_t r = t; r < m; r += kBigThreads) atomicAdd(&hist[(src[r] >> shift) & 255u], 1u);
    __syncthreads();
    // exclusive scan of the 256 digit counts (thread t owns digit t)
    uint32_t cnt = hist[t], x = cnt;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wcnt[0][warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t w = 0; w < warp; ++w) before += wcnt[0][w];
    __syncthreads();
    uint32_t base = before + x - cnt;  // digit t's running offset
    for (uint32_t c0 = 0; c0 < m; c0 += kBigThreads) {
      const uint32_t r = c0 + t;
      const bool valid = r < m;
      const uint32_t v = valid ? src[r] : 0u;
      const uint32_t d = valid ? (v >> shift) & 255u : 256u;
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
#pragma unroll
      for (uint32_t w = 0; w < kBigThreads / 32; ++w) wcnt[w][t] = 0u;
      __syncthreads();
      if (valid && (peers & lanemask_lt) == 0u) wcnt[warp][d] = __popc(peers);
      __syncthreads();
      uint32_t acc = 0;
#pragma unroll
      for (uint32_t w = 0; w < kBigThreads / 32; ++w) {
        const uint32_t c = wcnt[w][t];
        wcnt[w][t] = acc;
        acc += c;
      }
      hist[t] = base;
      __syncthreads();
      if (valid) alt[hist[d] + wcnt[warp][d] + __popc(peers & lanemask_lt)] = v;
      __syncthreads();
      base += acc;
    }
    uint32_t* tmp = src;
    src = alt;
    alt = tmp;
    __syncthreads();
  }
  return src;
}

// One block per listed cell (looping over the list): up to kBigCell source
// indices sorted in shared memory (bitonic, padded to a power of two, one
// compare-exchange per pair index and stage), larger cells by the block-wide
// radix sort in global memory; then the gather.
__global__ void __launch_bounds__(kBigThreads) k_cs_big(RebinArgs a) {
  __shared__ uint32_t sv[kBigCell];
  const uint32_t nb = min(a.ctrl->big_count, a.big_cap);
  uint32_t overflow = 0;
  const uint32_t key_bits = a.n > 1 ? 32u - __clz(a.n - 1) : 1u;
  for (uint32_t w = blockIdx.x; w < nb; w += gridDim.x) {
    const uint32_t k = a.big_list[w];
    const uint32_t s0 = a.cs_new[k], s1 = min(a.cs_new[k + 1], a.n);
    if (threadIdx.x == 0) a.counts[k] = 0u;  // read by the scan; zero for the next rebin
    const uint32_t s = s1 > s0 ? s1 - s0 : 0u;
    if (s > kBigCell) {
      const uint32_t* sorted = block_radix_sort(a.idx_tmp + s0, a.idx_alt + s0, s, key_bits);
      for (uint32_t r = threadIdx.x; r < s; r += kBigThreads) place_one(a, s0 + r, r, sorted[r], k, overflow);
      if (threadIdx.x == 0) atomicAdd(&a.ctrl->huge_cells, 1u);
      __syncthreads();
      continue;
    }
    uint32_t P = 1;
    while (P < s) P <<= 1;
    for (uint32_t r = threadIdx.x; r < P; r += kBigThreads)
      sv[r] = r < s ? a.idx_tmp[s0 + r] : 0xFFFFFFFFu;
    __syncthreads();
    for (uint32_t len = 2; len <= P; len <<= 1) {
      for (uint32_t j = len >> 1; j > 0; j >>= 1) {
        for (uint32_t pi = threadIdx.x; pi < P / 2; pi += kBigThreads) {
          // j is a power of two: r = 2 j floor(pi / j) + pi mod j
          const uint32_t r = ((pi & ~(j - 1u)) << 1) | (pi & (j - 1u)), o = r + j;
          const uint32_t x = sv[r], y = sv[o];
          if ((x > y) == ((r & len) == 0)) {
            sv[r] = y;
            sv[o] = x;
          }
        }
        __syncthreads();
      }
    }
    for (uint32_t r = threadIdx.x; r < s; r += kBigThreads) place_one(a, s0 + r, r, sv[r], k, overflow);
    __syncthreads();
  }
  add_overflow(a, overflow);
}

}  // namespace

cudaError_t launch_count_sort_step(const RebinArgs& a, int step, uint32_t big_blocks,
                                   cudaStream_t st, bool* launched) {
  const uint32_t ntiles = (a.ncells + kScanTile - 1) / kScanTile;
  const uint32_t nblk = (a.n + 255) / 256;
  *launched = true;
  if (step == 0) {
    if (!nblk) {
      *launched = false;
      return cudaSuccess;
    }
    k_cs_count<<<nblk, 256, 0, st>>>(a);
  } else if (step == 1) {
    RebinArgs b = a;
    b.tiles_prefixed = ntiles > kPrefixTiles ? 1u : 0u;
    if (b.tiles_prefixed) {
      k_cs_tile_prefix<<<1, 1024, 0, st>>>(b, ntiles);
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    k_cs_scan<<<ntiles ? ntiles : 1u, kScanThreads, 0, st>>>(b);
  } else if (!nblk) {
    *launched = false;
    return cudaSuccess;
  } else if (step == 2) {
    k_cs_scatter<<<nblk, 256, 0, st>>>(a, ntiles);
  } else if (step == 3) {
    k_cs_place<<<nblk, 256, 0, st>>>(a);
  } else {
    k_cs_big<<<big_blocks ? big_blocks : 1u, kBigThreads, 0, st>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_count_sort(const RebinArgs& a, uint32_t big_blocks, cudaStream_t st) {
  for (int step = 0; step < kCountSortSteps; ++step) {
    bool launched;
    const cudaError_t e = launch_count_sort_step(a, step, big_blocks, st, &launched);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

uint32_t count_sort_steps(uint32_t n) { return n ? 5u : 1u; }

uint32_t count_sort_launches(uint32_t n, uint32_t ncells) {
  const uint32_t ntiles = (ncells + kScanTile - 1) / kScanTile;
  return count_sort_steps(n) + (ntiles > kPrefixTiles ? 1u : 0u);
}

}  // namespace wrach
