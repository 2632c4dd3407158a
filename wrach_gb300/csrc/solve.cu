// Solve kernels: the collision/constraint pass plus the fused
// integrate + boundary + velocity-clamp epilogue, which also emits each
// particle's next cell key for the rebin.
//
// Reference-mode kernel: one thread per cell, the sequential sweep of
// World::physics_for_cell (shaders/physics/src/cell.rs:52-95).
// Extended-mode kernels: one thread per taking-part particle (compacted), a
// Jacobi iteration over the particle's 3x3 cell neighbourhood; the last
// iteration one thread per particle.
#include "wrach_internal.cuh"
#include "wrach_kernels.h"

namespace wrach {

namespace {

// Next cell of a solved particle (assets/shaders/particles_per_cell.wgsl:
// 14-27), the key the rebin sorts by.
__device__ __forceinline__ uint32_t next_key(const WorldDev& w, float px,
                                             float py, uint32_t& flags) {
  const uint32_t ncx = axis_cell(px, w.ax, w.cs, w.gx, flags);
  const uint32_t ncy = axis_cell(py, w.ay, w.cs, w.gy, flags);
  return w.cell_off + ncy * w.gx + ncx;
}

__device__ __forceinline__ void publish_flags(Ctrl* ctrl, uint32_t flags) {
  const uint32_t wf = warp_or_u32(flags);
  if ((threadIdx.x & 31) == 0 && wf) atomicOr(&ctrl->flags, wf);
}

// Reference mode, one thread per global cell.
//  - Particles::new: the first min(count, capacity) particles of the cell
//    (shaders/physics/src/particles.rs:31-59)
//  - Particles::pairs / push_close_particles_apart: Gauss-Seidel over i < j
//    (particles.rs:62-93)
//  - Particles::finish: integrate, boundaries, clamp, write (particles.rs:
//    96-107, particle.rs:40-106)
//  - handle_overflown_particles: the rest only integrate (cell.rs:79-95)
__global__ void __launch_bounds__(512)
k_solve_reference(const WorldDev* __restrict__ worlds, int nworlds,
                  PhysDev ph, uint32_t ncells,
                  const uint32_t* __restrict__ cell_start,
                  const float2* __restrict__ pin, const float2* __restrict__ vin,
                  float2* __restrict__ pout, float2* __restrict__ vout,
                  uint32_t* __restrict__ keys, Ctrl* ctrl) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t flags = 0;
  if (c < ncells) {
    const WorldDev w = worlds[world_of_cell(worlds, nworlds, c)];
    const uint32_t s = cell_start[c], e = cell_start[c + 1];
    const uint32_t m = min(e - s, ph.cap);
    float px[kMaxCellCapacity], py[kMaxCellCapacity];
    float vx[kMaxCellCapacity], vy[kMaxCellCapacity];
    for (uint32_t i = 0; i < m; ++i) {
      float2 p = pin[s + i], v = vin[s + i];
      px[i] = p.x; py[i] = p.y; vx[i] = v.x; vy[i] = v.y;
    }
    for (uint32_t i = 0; i < m; ++i)
      for (uint32_t j = i + 1; j < m; ++j) {
        float f;
        if (!push_factor(__fsub_rn(px[i], px[j]), __fsub_rn(py[i], py[j]),
                         ph.min_d, ph.skip_d2, f))
          continue;
        float dx = __fmul_rn(__fsub_rn(px[j], px[i]), f);
        float dy = __fmul_rn(__fsub_rn(py[j], py[i]), f);
        px[i] = __fsub_rn(px[i], dx); py[i] = __fsub_rn(py[i], dy);
        px[j] = __fadd_rn(px[j], dx); py[j] = __fadd_rn(py[j], dy);
      }
    for (uint32_t i = 0; i < m; ++i) {
      float qx = __fadd_rn(px[i], vx[i]), qy = __fadd_rn(py[i], vy[i]);
      float ux = vx[i], uy = vy[i];
      enforce_limits(w, ph.vmax, qx, qy, ux, uy);
      pout[s + i] = make_float2(qx, qy);
      vout[s + i] = make_float2(ux, uy);
      keys[s + i] = next_key(w, qx, qy, flags);
    }
    for (uint32_t i = s + m; i < e; ++i) {
      float2 p = pin[i], v = vin[i];
      float qx = __fadd_rn(p.x, v.x), qy = __fadd_rn(p.y, v.y);
      float ux = v.x, uy = v.y;
      enforce_limits(w, ph.vmax, qx, qy, ux, uy);
      pout[i] = make_float2(qx, qy);
      vout[i] = make_float2(ux, uy);
      keys[i] = next_key(w, qx, qy, flags);
    }
  }
  publish_flags(ctrl, flags);
}

// Extended mode (3x3 cells, Jacobi iterations, gravity).  As in the
// reference (cell.rs:29-30, 79-95) only the first `cap` particles of a cell
// take part in the pushes, as pushed particles and as neighbours; the rest of
// an over-full cell keep their position.  The neighbour order is fixed (the
// 3x3 cells in row-major order, table order inside a cell), so each
// particle's push sum is deterministic.
//
// The iterations run over the compacted taking-part particles (the capped
// table ct of the rebin): there a neighbour row of the 3x3 search is one
// contiguous range [ct[row + x0], ct[row + x1 + 1]) whatever the cells'
// occupancy, and the particles that take no part cost nothing.  Per row, the
// candidates within reach are marked with an exact squared-distance test
// (cheap, every candidate), then the reference's push (IEEE square root and
// division) is applied to the marked ones only, in candidate order, in one
// loop over the three rows' marks, so that a lane moves on to its next row
// without waiting for the warp's other lanes to finish the current one.

__device__ __forceinline__ uint32_t low_bit(uint32_t m) { return __ffs((int)m) - 1; }
__device__ __forceinline__ uint32_t low_bit(uint64_t m) { return __ffsll((long long)m) - 1; }

// The push sum (ax, ay) of the compacted particle t of cell c at q_t = qi2,
// over the compacted iterate q.  Mask holds one bit per candidate of a row:
// 3 * cap bits.  METRICS: pen = the deepest overlap min_d - distance with a
// pushing neighbour.
// The compacted ranges [rs[r], re[r]) of the three neighbour rows of cell c
// (independent loads of the capped table).
__device__ __forceinline__ void tp_rows(const WorldDev& w, const uint32_t* __restrict__ ct,
                                        uint32_t c, uint32_t (&rs)[3], uint32_t (&re)[3]) {
  uint32_t cx, cy;
  cell_xy(w, c - w.cell_off, cx, cy);
  const uint32_t x0 = cx > 0 ? cx - 1 : 0;
  const uint32_t x1 = cx + 1 < w.gx ? cx + 1 : w.gx - 1;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const int ny = (int)cy - 1 + r;
    const bool ok = ny >= 0 && ny < (int)w.gy;
    const uint32_t rb = w.cell_off + (uint32_t)(ok ? ny : 0) * w.gx;
    rs[r] = ok ? ct[rb + x0] : 0u;
    re[r] = ok ? ct[rb + x1 + 1] : 0u;
  }
}

// The push sum over the candidates of the rows [rs[r], re[r]) of the
// compacted particle t (in the middle row).
template <typename Mask, bool METRICS>
__device__ __forceinline__ void tp_push_rows(const PhysDev& ph, const f32x2* __restrict__ q,
                                             f32x2 qi2, uint32_t t, const uint32_t (&rs)[3],
                                             const uint32_t (&re)[3], float& ax, float& ay,
                                             float& pen) {
  // the candidates within reach, three per step (a short last step tests
  // its last candidate again and keeps the first result); a NaN distance
  // counts as within reach, as in the reference's test
  Mask rmask[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    Mask close = 0;
    const uint32_t s0 = rs[r], e = re[r];
    for (uint32_t j = s0; j < e; j += 3) {
      const uint32_t j1 = min(j + 1, e - 1), j2 = min(j + 2, e - 1);
      const f32x2 da = f2_sub(q[j], qi2), db = f2_sub(q[j1], qi2), dc = f2_sub(q[j2], qi2);
      const bool ca = !(f2_len2(da) >= ph.skip_d2);
      const bool cb = j + 1 < e && !(f2_len2(db) >= ph.skip_d2);
      const bool cc = j + 2 < e && !(f2_len2(dc) >= ph.skip_d2);
      close |= (Mask)((ca ? 1u : 0u) | (cb ? 2u : 0u) | (cc ? 4u : 0u)) << (j - s0);
    }
    // the particle itself (in the middle row) is not its own neighbour
    if (r == 1) close &= ~((Mask)1 << (t - s0));
    rmask[r] = close;
  }
  // the reference's push for those, in candidate order
  Mask cur = rmask[0];
  uint32_t base = rs[0];
  Mask next1 = rmask[1], next2 = rmask[2];
  for (;;) {
    if (cur == 0) {
      if (next1) {
        cur = next1;
        next1 = 0;
        base = rs[1];
      } else if (next2) {
        cur = next2;
        next2 = 0;
        base = rs[2];
      } else {
        break;
      }
    }
    const uint32_t b = low_bit(cur);
    cur &= cur - 1;
    const f32x2 dd = f2_sub(q[base + b], qi2);
    float d;
    const float f = push_factor_within(f2_x(dd), f2_y(dd), ph.min_d, d);
    if (METRICS) pen = fmaxf(pen, __fsub_rn(ph.min_d, d));
    // scalar: a paired multiply feeding a paired add may be fused
    ax = __fadd_rn(ax, __fmul_rn(f2_x(dd), f));
    ay = __fadd_rn(ay, __fmul_rn(f2_y(dd), f));
  }
}

template <typename Mask, bool METRICS>
__device__ __forceinline__ void tp_push(const WorldDev& w, const PhysDev& ph,
                                        const uint32_t* __restrict__ ct,
                                        const f32x2* __restrict__ q, f32x2 qi2, uint32_t c,
                                        uint32_t t, float& ax, float& ay, float& pen) {
  uint32_t rs[3], re[3];
  tp_rows(w, ct, c, rs, re);
  tp_push_rows<Mask, METRICS>(ph, q, qi2, t, rs, re, ax, ay, pen);
}

// One Jacobi iteration but the last, one thread per compacted (taking-part)
// particle: q' = q - push sum, over the compacted count ct[ncells] (a
// grid-stride loop; the plain frames' grid covers every particle of the
// frame, so each thread takes one or none).  A launch whose `run_if` flag
// reads 0 returns at once.
// ROWS 0: the neighbour rows from the capped table; 1: also written to
// `rows` (4 planes of `stride`); 2: read from `rows` (the cell and its
// world are then not needed).
template <typename Mask, int ROWS>
__global__ void __launch_bounds__(512)
k_jacobi_tp(const WorldDev* __restrict__ worlds, int nworlds, PhysDev ph, uint32_t ncells,
            const uint32_t* __restrict__ ct, const uint32_t* __restrict__ tp_cell,
            const float2* __restrict__ qin, float2* __restrict__ qout,
            const uint32_t* __restrict__ run_if, uint32_t* __restrict__ rows, uint32_t stride) {
  if (run_if && *run_if == 0u) return;
  const uint32_t ntp = __ldg(ct + ncells);
  const f32x2* __restrict__ q = reinterpret_cast<const f32x2*>(qin);
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntp; t += gridDim.x * blockDim.x) {
    uint32_t rs[3], re[3];
    if (ROWS == 2) {
      const uint32_t len = rows[3 * (size_t)stride + t];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        rs[r] = rows[(size_t)r * stride + t];
        re[r] = rs[r] + ((len >> (8 * r)) & 0xFFu);
      }
    } else {
      const uint32_t c = tp_cell[t];
      tp_rows(worlds[world_of_cell(worlds, nworlds, c)], ct, c, rs, re);
      if (ROWS == 1) {
#pragma unroll
        for (int r = 0; r < 3; ++r) rows[(size_t)r * stride + t] = rs[r];
        rows[3 * (size_t)stride + t] =
            (re[0] - rs[0]) | ((re[1] - rs[1]) << 8) | ((re[2] - rs[2]) << 16);
      }
    }
    const f32x2 qi2 = q[t];
    float ax = 0.f, ay = 0.f, pen = 0.f;
    tp_push_rows<Mask, false>(ph, q, qi2, t, rs, re, ax, ay, pen);
    qout[t] = make_float2(__fsub_rn(f2_x(qi2), ax), __fsub_rn(f2_y(qi2), ay));
  }
}

// The last iteration, one thread per frame particle (a grid-stride loop
// over whole blocks of particles; the plain frames' grid covers them all):
// the push (taking-part particles, from the compacted iterate q), then
// gravity, integration, boundaries, the velocity clamp and the key emission,
// and the rebin's tickets.  METRICS also writes the block's sums for the
// surrogate's fallback gate to part[blockIdx.x * 8 + k]: [0] sum and [1] max
// over taking-part particles of the deepest overlap max(0, min_d - distance)
// with a pushing neighbour (measured on the pass's input), [2] the number of
// taking-part particles, [3] the kinetic energy of the output and [4] the
// kinetic energy a plain frame gives (gravity, the clamp and wall
// reflections only change the velocity).  A launch whose `run_if` flag
// reads 0 returns at once.
template <typename Mask, bool METRICS>
__global__ void __launch_bounds__(512)
k_jacobi_final(const WorldDev* __restrict__ worlds, int nworlds, PhysDev ph, uint32_t n,
               int do_push, const uint32_t* __restrict__ cell_start,
               const uint32_t* __restrict__ ct, const uint32_t* __restrict__ cell_of,
               const float2* __restrict__ pin, const float2* __restrict__ qtp,
               float2* __restrict__ pout, const float2* __restrict__ vin,
               float2* __restrict__ vout, uint32_t* __restrict__ keys, Ctrl* ctrl,
               const uint32_t* __restrict__ run_if, float* __restrict__ part, CountDev count) {
  if (run_if && *run_if == 0u) return;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // taking the tickets: the rebin's scan lists its large cells afresh
  if (count.ticket && blockIdx.x == 0 && threadIdx.x == 0) ctrl->big_count = 0u;
  uint32_t flags = 0;
  float pen = 0.f, taking = 0.f, ke = 0.f, ke_plain = 0.f;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const bool live = i < n;
    uint32_t key = count.ncells;  // no cell
    if (live) {
      const uint32_t c = cell_of[i];
      const WorldDev w = worlds[world_of_cell(worlds, nworlds, c)];
      // the velocity and, for the tickets' atomics, the counters of the
      // particle's cell and of the cells above and below it (its next cell
      // is almost always among their lines) are fetched before the push
      const float2 v = vin[i];
      if (count.ticket) {
        prefetch_l2(count.counts + c);
        prefetch_l2(count.counts + (c >= w.gx ? c - w.gx : c));
        prefetch_l2(count.counts + min(c + w.gx, count.ncells - 1));
      }
      const uint32_t t = tp_index(cell_start, ct, c, i, ph.cap);
      float qx, qy;
      if (t != 0xFFFFFFFFu) {
        if (METRICS) taking = __fadd_rn(taking, 1.f);
        const f32x2* __restrict__ q = reinterpret_cast<const f32x2*>(qtp);
        const f32x2 qi2 = q[t];
        float ax = 0.f, ay = 0.f;
        if (do_push) tp_push<Mask, METRICS>(w, ph, ct, q, qi2, c, t, ax, ay, pen);
        qx = __fsub_rn(f2_x(qi2), ax);
        qy = __fsub_rn(f2_y(qi2), ay);
      } else {
        const float2 p = pin[i];
        qx = p.x;
        qy = p.y;
      }
      float ux = v.x, uy = __fsub_rn(v.y, ph.gravity);
      float px = __fadd_rn(qx, ux), py = __fadd_rn(qy, uy);
      enforce_limits(w, ph.vmax, px, py, ux, uy);
      pout[i] = make_float2(px, py);
      vout[i] = make_float2(ux, uy);
      key = next_key(w, px, py, flags);
      keys[i] = key;
      if (METRICS) {
        ke = __fadd_rn(ke, __fmul_rn(0.5f, __fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy))));
        const float cx = fminf(fmaxf(v.x, -ph.vmax), ph.vmax);
        const float cy = fminf(fmaxf(__fsub_rn(v.y, ph.gravity), -ph.vmax), ph.vmax);
        ke_plain = __fadd_rn(ke_plain,
                             __fmul_rn(0.5f, __fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy))));
      }
    }
    if (count.ticket) {
      // the rebin's tickets (every lane of the warp takes part)
      const uint32_t tk = warp_ticket(key, count.ncells, count.counts, count.tile_sums,
                                      count.tile_shift, count.cap, count.tile_sums_cap);
      if (live) count.ticket[i] = tk;
    }
  }
  publish_flags(ctrl, flags);
  if (METRICS) {
    // warp sums, then one thread sums the block's warps in a fixed order
    __shared__ float red[16][5];
    float v[5] = {pen, pen, taking, ke, ke_plain};
#pragma unroll
    for (uint32_t o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const float u = __shfl_xor_sync(0xffffffffu, v[k], o);
        v[k] = k == 1 ? fmaxf(v[k], u) : __fadd_rn(v[k], u);
      }
    }
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < 5; ++k) red[warp][k] = v[k];
    __syncthreads();
    if (threadIdx.x < 5) {
      const uint32_t nw = (blockDim.x + 31) >> 5;
      float acc = red[0][threadIdx.x];
      for (uint32_t wi = 1; wi < nw; ++wi)
        acc = threadIdx.x == 1 ? fmaxf(acc, red[wi][threadIdx.x]) : __fadd_rn(acc, red[wi][threadIdx.x]);
      part[blockIdx.x * 8 + threadIdx.x] = acc;
    }
  }
}

}  // namespace

cudaError_t launch_solve_reference(const SolveArgs& a, cudaStream_t st) {
  if (a.ncells == 0) return cudaSuccess;
  const uint32_t threads = a.block ? a.block : 128;
  const uint32_t blocks = (a.ncells + threads - 1) / threads;
  k_solve_reference<<<blocks, threads, 0, st>>>(
      a.worlds, a.nworlds, a.ph, a.ncells, a.cell_start, a.pos, a.vel,
      a.pos_out, a.vel_out, a.keys, a.ctrl);
  return cudaGetLastError();
}

uint32_t solve_blocks(const SolveArgs& a) {
  const uint32_t threads = a.block ? a.block : 128;
  const uint32_t per = a.per_thread ? a.per_thread : 1u;
  const uint32_t blocks = (a.n + threads * per - 1) / (threads * per);
  // a launch that usually returns at once (the surrogate's fallback) strides
  // over the frame with a few blocks per SM, so that skipping it is cheap
  const uint32_t few = (uint32_t)(a.sms > 0 ? a.sms : 1) * (1024u / threads);
  return a.run_if && blocks > few ? few : blocks;
}

cudaError_t launch_jacobi_iteration(const SolveArgs& a, const float2* qin, float2* qout,
                                    cudaStream_t st) {
  if (a.n == 0) return cudaSuccess;
  const uint32_t threads = a.block ? a.block : 128;
  const uint32_t blocks = solve_blocks(a);
  const int mode = a.rows ? a.rows_mode : 0;
#define WRACH_TP(MASK, ROWS)                                                                  \
  k_jacobi_tp<MASK, ROWS><<<blocks, threads, 0, st>>>(a.worlds, a.nworlds, a.ph, a.ncells, a.ct, \
                                                      a.tp_cell, qin, qout, a.run_if, a.rows,  \
                                                      a.rows_stride)
  if (3 * a.ph.cap <= 32) {
    if (mode == 1) WRACH_TP(uint32_t, 1);
    else if (mode == 2) WRACH_TP(uint32_t, 2);
    else WRACH_TP(uint32_t, 0);
  } else {
    if (mode == 1) WRACH_TP(uint64_t, 1);
    else if (mode == 2) WRACH_TP(uint64_t, 2);
    else WRACH_TP(uint64_t, 0);
  }
#undef WRACH_TP
  return cudaGetLastError();
}

cudaError_t launch_jacobi_final(const SolveArgs& a, const float2* qtp, int do_push,
                                cudaStream_t st) {
  if (a.n == 0) return cudaSuccess;
  const uint32_t threads = a.block ? a.block : 128;
  const uint32_t blocks = solve_blocks(a);
  const bool narrow = 3 * a.ph.cap <= 32;
#define WRACH_FINAL(MASK, METRICS, PART)                                                     \
  k_jacobi_final<MASK, METRICS><<<blocks, threads, 0, st>>>(                                 \
      a.worlds, a.nworlds, a.ph, a.n, do_push, a.cell_start, a.ct, a.cell_of, a.pos, qtp,    \
      a.pos_out, a.vel, a.vel_out, a.keys, a.ctrl, a.run_if, PART, a.count)
  if (a.part && narrow)
    WRACH_FINAL(uint32_t, true, a.part);
  else if (a.part)
    WRACH_FINAL(uint64_t, true, a.part);
  else if (narrow)
    WRACH_FINAL(uint32_t, false, nullptr);
  else
    WRACH_FINAL(uint64_t, false, nullptr);
#undef WRACH_FINAL
  return cudaGetLastError();
}

}  // namespace wrach
