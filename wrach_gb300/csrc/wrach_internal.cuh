// Internal device-side types and helpers shared by the kernels of the wrach
// GB300 library.  Every translation unit that includes this file is compiled
// with -fmad=false and IEEE division/square root, so the arithmetic below is
// binary32 round-to-nearest with no contraction: the contract under which the
// reference's CPU known-answer test (shaders/physics/src/particles.rs:128-146)
// reproduces bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace wrach {

// One world as the kernels see it (48 bytes).  The first eight fields are the
// reference's uniform (runners/bevy/src/config_shader.rs:15-29) minus the
// particle count, which lives in the cell-start table.
struct WorldDev {
  float dim_x, dim_y;  // view_dimensions
  float ax, ay;        // view_anchor
  uint32_t gx, gy;     // grid_dimensions
  uint32_t cs;         // cell_size
  uint32_t cell_off;   // global index of the world's first cell
  float x1, y1;        // anchor + dimensions, summed in binary32 as
                       // Particle::enforce_boundaries does (particle.rs:47-52)
  int32_t blx, bly;    // cell coordinate of the grid's bottom-left cell
  uint32_t div_m;      // x / gx == (x * div_m) >> div_s for all x < 2^31
  uint32_t div_s;
};

struct PhysDev {
  uint32_t mode;        // 0 reference, 1 extended
  uint32_t iterations;  // extended only
  float gravity;
  float min_d;
  float vmax;
  uint32_t cap;         // reference cell capacity
  float skip_d2;        // smallest squared distance s with sqrt_rn(s) > min_d
};

// Device control block: counters of the persistent rebin kernel and the
// sticky flags.  Zeroed at create; every launch of the rebin kernel leaves
// exit_count at zero again.
struct Ctrl {
  uint32_t exit_count;  // rebin blocks finished in this launch
  uint32_t epoch;       // rebin launch counter, tags the tile status words
  uint32_t flags;       // sticky WRACH_FLAG_* bits
  uint32_t bar_count;   // grid barrier arrivals
  uint32_t bar_gen;     // grid barrier generation
  uint32_t overflow;    // particles dropped for lack of destination room
  uint32_t frames;      // rebin launches that were frames (not uploads)
  uint32_t never_set;   // stays 0: the word wrach_selftest_wait waits on
  uint32_t big_count;   // counting sort: cells on the large-cell work list
  uint32_t huge_cells;  // counting sort: cells sorted in global memory, since create
  uint32_t pad[6];
};

constexpr uint32_t kFlagOutOfGrid = 1u;
constexpr uint32_t kFlagNaN = 2u;
constexpr uint32_t kFlagTimeout = 4u;


// Maximum reference-mode cell capacity held in registers/local memory.
constexpr uint32_t kMaxCellCapacity = 16;

// (row, column) of a world-local cell index without a hardware division.
__device__ __forceinline__ void cell_xy(const WorldDev& w, uint32_t local,
                                        uint32_t& cx, uint32_t& cy) {
  cy = (uint32_t)(((uint64_t)local * w.div_m) >> w.div_s);
  cx = local - cy * w.gx;
}

// World of a global cell index: the last world whose cell_off <= c.
// With more than one world, the array of nworlds WorldDev is followed by
// world_tiles(ncells) + 2 u32: the world holding the first cell of each tile
// of 2^kWorldTileShift cells (the last two entries: nworlds - 1), so a
// lookup searches only the few worlds one tile can span.
constexpr uint32_t kWorldTileShift = 12;
__host__ __device__ __forceinline__ uint32_t world_tiles(uint32_t ncells) {
  return (ncells + (1u << kWorldTileShift) - 1) >> kWorldTileShift;
}

__device__ __forceinline__ int world_of_cell(const WorldDev* __restrict__ W,
                                             int nworlds, uint32_t c) {
  if (nworlds <= 1) return 0;
  const uint32_t* tile_first = reinterpret_cast<const uint32_t*>(W + nworlds);
  const uint32_t t = c >> kWorldTileShift;
  int lo = (int)__ldg(tile_first + t), hi = (int)__ldg(tile_first + t + 1);
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(&W[mid].cell_off) <= c)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Frame-time cell of one axis (assets/shaders/particles_per_cell.wgsl:14-27):
// floor((p - anchor) / cell_size).  Out-of-grid and NaN inputs, undefined in
// the WGSL, are clamped into the grid (NaN -> 0) and flagged.  A quotient by
// 1 is its dividend exactly, so cell size 1 skips the division.
__device__ __forceinline__ uint32_t axis_cell(float p, float a, uint32_t cs,
                                              uint32_t g, uint32_t& flags) {
  const float d = __fsub_rn(p, a);
  float f = floorf(cs == 1u ? d : __fdiv_rn(d, (float)cs));
  if (!(f >= 0.0f)) {
    flags |= (f != f) ? (kFlagNaN | kFlagOutOfGrid) : kFlagOutOfGrid;
    return 0u;
  }
  if (f >= (float)g) {
    flags |= kFlagOutOfGrid;
    return g - 1u;
  }
  return (uint32_t)f;
}

// Particle::enforce_boundaries + enforce_velocity
// (shaders/physics/src/particle.rs:46-77).  The clamp is Rust's f32::clamp:
// compare-and-replace, NaN passes through.
__device__ __forceinline__ void enforce_limits(const WorldDev& w, float vmax,
                                               float& px, float& py, float& vx,
                                               float& vy) {
  if (px > w.x1) { px = w.x1; vx = -vx; }
  if (px < w.ax) { px = w.ax; vx = -vx; }
  if (py > w.y1) { py = w.y1; vy = -vy; }
  if (py < w.ay) { py = w.ay; vy = -vy; }
  if (vx < -vmax) vx = -vmax;
  if (vx > vmax) vx = vmax;
  if (vy < -vmax) vy = -vmax;
  if (vy > vmax) vy = vmax;
}

// The reference's pair push factor (shaders/physics/src/particles.rs:62-93):
// returns false when the pair is farther apart than min_d, otherwise the
// force 0.5 * (min_d - d) / d with d == 0 replaced by 0.0001.
// `skip_d2` is the smallest binary32 s with sqrt_rn(s) > min_d (computed on
// the host); since sqrt_rn is monotonic, s >= skip_d2 is exactly the
// reference's `distance > MIN_DISTANCE`, decided without the square root.
__device__ __forceinline__ bool push_factor(float ex, float ey, float min_d,
                                            float skip_d2, float& f, float& dist) {
  const float s = __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
  if (s >= skip_d2) return false;
  float d = __fsqrt_rn(s);
  dist = d;
  if (d > min_d) return false;
  if (d == 0.0f) d = 0.0001f;
  f = __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(min_d, d)), d);
  return true;
}
__device__ __forceinline__ bool push_factor(float ex, float ey, float min_d,
                                            float skip_d2, float& f) {
  float d;
  return push_factor(ex, ey, min_d, skip_d2, f, d);
}
// The same force for a pair already found within reach (s < skip_d2, or s
// NaN): both tests of push_factor would pass, so they are left out.
__device__ __forceinline__ float push_factor_within(float ex, float ey, float min_d,
                                                    float& dist) {
  const float s = __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
  float d = __fsqrt_rn(s);
  dist = d;
  if (d == 0.0f) d = 0.0001f;
  return __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(min_d, d)), d);
}

// Counting-sort ticket of a particle whose next cell is k (k >= ncells: no
// cell).  All 32 lanes of the warp call it together.  Per warp, one atomic
// per cell present gives each particle its slot inside the cell (arrival
// order, lane order inside the warp), and one atomic per tile of
// 2^tile_shift cells adds the tile's particle count.  With `tile_sums_cap`
// set, the tickets below `cap` are also added to their tile's capped sum:
// a cell's tickets are 0 .. count-1, so those number min(count, cap), the
// particles of the cell that take part in the pushes.  Returns the slot, or
// 0xFFFFFFFF for no cell.
__device__ __forceinline__ uint32_t warp_ticket(uint32_t k, uint32_t ncells, uint32_t* counts,
                                                uint32_t* tile_sums, uint32_t tile_shift,
                                                uint32_t cap, uint32_t* tile_sums_cap) {
  const uint32_t lane = threadIdx.x & 31;
  const bool valid = k < ncells;
  const uint32_t peers = __match_any_sync(0xffffffffu, valid ? k : 0xFFFFFFFFu);
  const uint32_t leader = __ffs(peers) - 1;
  uint32_t first = 0;
  if (lane == leader && valid) first = atomicAdd(&counts[k], __popc(peers));
  first = __shfl_sync(0xffffffffu, first, leader);
  const uint32_t ticket = valid ? first + __popc(peers & ((1u << lane) - 1u)) : 0xFFFFFFFFu;
  const uint32_t tile = valid ? k >> tile_shift : 0xFFFFFFFFu;
  const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
  const uint32_t cmask = tile_sums_cap ? __ballot_sync(0xffffffffu, valid && ticket < cap) : 0u;
  const uint32_t t0 = __shfl_sync(0xffffffffu, tile, vmask ? __ffs(vmask) - 1 : 0);
  if (__all_sync(0xffffffffu, !valid || tile == t0)) {
    // the common case: the warp's particles fall in one tile
    if (lane == 0 && vmask) atomicAdd(&tile_sums[t0], __popc(vmask));
    if (lane == 0 && cmask) atomicAdd(&tile_sums_cap[t0], __popc(cmask));
  } else {
    const uint32_t tpeers = __match_any_sync(0xffffffffu, tile);
    if (valid && lane == (uint32_t)(__ffs(tpeers) - 1)) {
      atomicAdd(&tile_sums[tile], __popc(tpeers));
      if (cmask & tpeers) atomicAdd(&tile_sums_cap[tile], __popc(cmask & tpeers));
    }
  }
  return ticket;
}

// What the last Jacobi pass needs to take the counting sort's tickets.
struct CountDev {
  uint32_t* counts;         // ncells, zero on entry
  uint32_t* tile_sums;      // one per tile of 2^tile_shift cells, zero on entry
  uint32_t* ticket;         // n; nullptr: no tickets
  uint32_t ncells;
  uint32_t tile_shift;
  uint32_t cap;             // cell capacity of the taking-part particles
  uint32_t* tile_sums_cap;  // per tile, tickets below cap (nullptr: not counted)
};

// The taking-part particles of a frame (the first `cap` of each cell, in
// cell order) are also kept compacted: cell c's taking-part particles are
// compacted entries [ct[c], ct[c + 1]) (the capped table, ct[ncells] = their
// number), frame particle i of cell c takes part when i - cs[c] < cap, and
// its compacted index is then ct[c] + i - cs[c].  Every neighbour row of the
// 3x3 search is then one contiguous compacted range, over-full cells or not.
__device__ __forceinline__ uint32_t tp_index(const uint32_t* __restrict__ cs,
                                             const uint32_t* __restrict__ ct, uint32_t c,
                                             uint32_t i, uint32_t cap) {
  const uint32_t r = i - cs[c];
  return r < cap ? ct[c] + r : 0xFFFFFFFFu;
}

// Packed pairs of binary32 values (x in the low word, as float2 in memory)
// and sm_100-family paired arithmetic: each half rounds to nearest even on
// its own, exactly as two __fadd_rn / __fsub_rn / __fmul_rn do.  A paired
// multiply whose result feeds a paired add can be fused into one rounding
// by the compiler (measured on sm_103a despite the .rn modifiers), so chains
// that must round twice use the scalar intrinsics, which are never fused;
// f2_len2 (paired multiply, then a scalar add of the halves) measured exact.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2_pack(float x, float y) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
  return r;
}
__device__ __forceinline__ float f2_x(f32x2 v) { return __uint_as_float((uint32_t)v); }
__device__ __forceinline__ float f2_y(f32x2 v) { return __uint_as_float((uint32_t)(v >> 32)); }
__device__ __forceinline__ f32x2 f2_add(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
// Squared length of a packed (dx, dy): fl(fl(dx*dx) + fl(dy*dy)).
__device__ __forceinline__ float f2_len2(f32x2 d) {
  const f32x2 q = f2_mul(d, d);
  return __fadd_rn(f2_x(q), f2_y(q));
}

__device__ __forceinline__ uint64_t ld_acquire_u64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(uint64_t* p, uint64_t v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// A hint that the line of p will be read soon: fetched into L2.  p must be
// inside an allocation.
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded device waits give up after this many nanoseconds and raise
// kFlagTimeout instead of hanging the GPU.
constexpr uint64_t kWaitLimitNs = 1000000000ull;

// The device's only kind of wait: until *p differs from `value`, for at most
// limit_ns of %globaltimer.  Returns false if it gave up (the caller raises
// kFlagTimeout and carries on, so a lost peer never hangs the GPU).
__device__ __forceinline__ bool wait_while_equal(const uint32_t* p, uint32_t value,
                                                 uint64_t limit_ns) {
  const uint64_t t0 = global_ns();
  while (ld_acquire_u32(p) == value) {
    if (global_ns() - t0 > limit_ns) return false;
    __nanosleep(64);
  }
  return true;
}

// Warp-reduce helpers.
__device__ __forceinline__ uint32_t warp_max_u32(uint32_t v) {
  return __reduce_max_sync(0xffffffffu, v);
}
__device__ __forceinline__ uint32_t warp_or_u32(uint32_t v) {
  return __reduce_or_sync(0xffffffffu, v);
}

}  // namespace wrach
