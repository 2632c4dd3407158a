// Solve kernels: the collision/constraint pass plus the fused
// integrate + boundary + velocity-clamp epilogue, which also emits each
// particle's next cell key for the rebin.
//
// Reference-mode kernel: one thread per cell, the sequential sweep of
// World::physics_for_cell (shaders/physics/src/cell.rs:52-95).
// Extended-mode kernel: one thread per particle, a Jacobi iteration over the
// particle's 3x3 cell neighbourhood.
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

// Extended mode, one Jacobi iteration, one thread per particle.  As in the
// reference (cell.rs:29-30, 79-95) only the first `cap` particles of a cell
// take part in the pushes, as pushed particles and as neighbours; the rest of
// an over-full cell keep their position.  The neighbour order is fixed (3x3
// cells in row-major order, table order inside a cell), so the sum is
// deterministic.
//
// Two passes: pass 1 marks, per neighbour row, the candidates within reach
// with an exact squared-distance test (cheap, every lane); pass 2 applies
// the reference's push (IEEE square root and division) to those only, in
// candidate order, in one loop over the three rows' marks.  A row whose
// cells before the last are within capacity is one contiguous range of
// candidates, scanned in one loop; other rows keep 16 mark bits per cell.
//
// FINAL fuses gravity, integration, boundaries, the velocity clamp and the
// key emission.  METRICS (final pass only) also writes the block's sums for
// the surrogate's fallback gate to part[blockIdx.x * 8 + k]: [0] sum and [1]
// max over taking-part particles of the deepest overlap max(0, min_d -
// distance) with a pushing neighbour (measured on the pass's input), [2] the
// number of taking-part particles, [3] the kinetic energy of the output and
// [4] the kinetic energy a plain frame gives (gravity, the clamp and wall
// reflections only change the velocity).  A launch whose `run_if` flag reads
// 0 returns at once.
template <bool FINAL, bool METRICS>
__global__ void __launch_bounds__(512)
k_jacobi(const WorldDev* __restrict__ worlds, int nworlds, PhysDev ph,
         uint32_t n, int do_push, const uint32_t* __restrict__ cell_start,
         const uint32_t* __restrict__ cell_of, const float2* __restrict__ qin,
         float2* __restrict__ qout, const float2* __restrict__ vin,
         float2* __restrict__ vout, uint32_t* __restrict__ keys, Ctrl* ctrl,
         const uint32_t* __restrict__ run_if, float* __restrict__ part, CountDev count) {
  static_assert(FINAL || !METRICS, "metrics come from the final pass");
  if (run_if && *run_if == 0u) return;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  // taking the tickets: the rebin's scan lists its large cells afresh
  if (FINAL && count.ticket && i == 0) ctrl->big_count = 0u;
  const bool live = i < n;
  uint32_t flags = 0;
  float pen = 0.f, taking = 0.f, ke = 0.f, ke_plain = 0.f;
  WorldDev w;
  float2 qi = make_float2(0.f, 0.f);
  // the push sum, and the positions as packed pairs
  float ax = 0.0f, ay = 0.0f;
  const f32x2* __restrict__ q64 = reinterpret_cast<const f32x2*>(qin);
  f32x2 qi2 = 0ull;
  uint32_t key = count.ncells;  // no cell, unless the final pass computes one
  if (live) {
    const uint32_t c = cell_of[i];
    w = worlds[world_of_cell(worlds, nworlds, c)];
    uint32_t cx, cy;
    cell_xy(w, c - w.cell_off, cx, cy);
    qi2 = q64[i];
    qi = make_float2(f2_x(qi2), f2_y(qi2));
    if (do_push && i - cell_start[c] < ph.cap) {
      if (METRICS) taking = 1.f;
      // the table entries of the three neighbour rows first: independent
      // loads, so their latencies overlap
      const uint32_t x0 = cx > 0 ? cx - 1 : 0;
      const uint32_t x1 = cx + 1 < w.gx ? cx + 1 : w.gx - 1;
      uint32_t st[3][4];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const int ny = (int)cy - 1 + r;
        const bool row_ok = ny >= 0 && ny < (int)w.gy;
        const uint32_t rb = w.cell_off + (uint32_t)(row_ok ? ny : 0) * w.gx + x0;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          st[r][k] = (row_ok && x0 + k <= x1 + 1) ? cell_start[rb + k] : 0u;
      }
      const uint32_t ncol = x1 - x0 + 1;  // 2 or 3 cells per row
      static_assert(kMaxCellCapacity <= 16, "16 mask bits per cell");
      // per row: the close mask and the map from mask bit b to candidate
      // index, base + b + (b >= 16 ? adj1 : 0) + (b >= 32 ? adj2 : 0)
      uint64_t rmask[3];
      uint32_t rbase[3], radj1[3], radj2[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        // the row's taking-part candidates: up to three cells of at most
        // `cap` particles each; a NaN distance counts as within reach, as in
        // the reference's test
        const uint32_t s0 = st[r][0], s1 = st[r][1], s2 = st[r][2], s3 = st[r][3];
        const uint32_t e0 = min(s1, s0 + ph.cap);
        const uint32_t e1 = min(s2, s1 + ph.cap);
        const uint32_t e2 = ncol == 3 ? min(s3, s2 + ph.cap) : s2;
        uint64_t close = 0;
        const bool merged = e0 == s1 && (ncol == 2 || e1 == s2);
        rbase[r] = s0;
        radj1[r] = merged ? 0u : s1 - s0 - 16u;
        radj2[r] = merged ? 0u : s2 - s1 - 16u;
        if (merged) {
          // no over-full cell before the last: one contiguous range, two
          // candidates per step (an odd last step tests its one candidate
          // twice and keeps the first result)
          const uint32_t e = ncol == 3 ? e2 : e1;
          for (uint32_t j = s0; j < e; j += 2) {
            const uint32_t j1 = min(j + 1, e - 1);
            const f32x2 da = f2_sub(q64[j], qi2), db = f2_sub(q64[j1], qi2);
            const bool ca = !(f2_len2(da) >= ph.skip_d2);
            const bool cb = j + 1 < e && !(f2_len2(db) >= ph.skip_d2);
            close |= (uint64_t)((ca ? 1u : 0u) | (cb ? 2u : 0u)) << (j - s0);
          }
          // the particle itself (in the middle row) is not its own neighbour
          if (r == 1 && i >= s0 && i < e) close &= ~(1ull << (i - s0));
        } else {
          uint32_t k = 0;
          for (uint32_t j = s0; j < e0; ++j, ++k) {
            if ((r != 1 || j != i) && !(f2_len2(f2_sub(q64[j], qi2)) >= ph.skip_d2)) close |= 1ull << k;
          }
          k = 16;
          for (uint32_t j = s1; j < e1; ++j, ++k) {
            if ((r != 1 || j != i) && !(f2_len2(f2_sub(q64[j], qi2)) >= ph.skip_d2)) close |= 1ull << k;
          }
          k = 32;
          for (uint32_t j = s2; j < e2; ++j, ++k) {
            if ((r != 1 || j != i) && !(f2_len2(f2_sub(q64[j], qi2)) >= ph.skip_d2)) close |= 1ull << k;
          }
        }
        rmask[r] = close;
      }
      // pass 2: the reference's push for those, in candidate order
      // (cell.rs:79-95).  One loop over the three rows' masks, so that a
      // lane moves on to its next row without waiting for the warp's other
      // lanes to finish the current one.
      uint64_t cur = rmask[0];
      uint32_t base = rbase[0], adj1 = radj1[0], adj2 = radj2[0];
      uint64_t next1 = rmask[1], next2 = rmask[2];
      for (;;) {
        if (cur == 0) {
          if (next1) {
            cur = next1; next1 = 0;
            base = rbase[1]; adj1 = radj1[1]; adj2 = radj2[1];
          } else if (next2) {
            cur = next2; next2 = 0;
            base = rbase[2]; adj1 = radj1[2]; adj2 = radj2[2];
          } else {
            break;
          }
        }
        const uint32_t b = __ffsll((long long)cur) - 1;
        cur &= cur - 1;
        const uint32_t j = base + b + (b >= 16 ? adj1 : 0u) + (b >= 32 ? adj2 : 0u);
        const f32x2 dd = f2_sub(q64[j], qi2);
        float d;
        const float f = push_factor_within(f2_x(dd), f2_y(dd), ph.min_d, d);
        if (METRICS) pen = fmaxf(pen, __fsub_rn(ph.min_d, d));
        // scalar: a paired multiply feeding a paired add may be fused
        ax = __fadd_rn(ax, __fmul_rn(f2_x(dd), f));
        ay = __fadd_rn(ay, __fmul_rn(f2_y(dd), f));
      }
    }
  }
  if (live) {
    const float qx = __fsub_rn(qi.x, ax), qy = __fsub_rn(qi.y, ay);
    if (!FINAL) {
      qout[i] = make_float2(qx, qy);
    } else {
      const float2 v = vin[i];
      float ux = v.x, uy = __fsub_rn(v.y, ph.gravity);
      float px = __fadd_rn(qx, ux), py = __fadd_rn(qy, uy);
      enforce_limits(w, ph.vmax, px, py, ux, uy);
      qout[i] = make_float2(px, py);
      vout[i] = make_float2(ux, uy);
      key = next_key(w, px, py, flags);
      keys[i] = key;
      if (METRICS) {
        ke = __fmul_rn(0.5f, __fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy)));
        const float cx = fminf(fmaxf(v.x, -ph.vmax), ph.vmax);
        const float cy = fminf(fmaxf(__fsub_rn(v.y, ph.gravity), -ph.vmax), ph.vmax);
        ke_plain = __fmul_rn(0.5f, __fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy)));
      }
    }
  }
  if (FINAL && count.ticket) {
    // the rebin's tickets (every lane of the warp takes part)
    const uint32_t t = warp_ticket(key, count.ncells, count.counts, count.tile_sums,
                                   count.tile_shift);
    if (live) count.ticket[i] = t;
  }
  if (FINAL) publish_flags(ctrl, flags);
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

cudaError_t launch_solve_extended(const SolveArgs& a, const float2* qin,
                                  float2* qout, bool final_pass, int do_push,
                                  cudaStream_t st) {
  if (a.n == 0) return cudaSuccess;
  const uint32_t threads = a.block ? a.block : 128;
  const uint32_t blocks = (a.n + threads - 1) / threads;
  if (final_pass && a.part)
    k_jacobi<true, true><<<blocks, threads, 0, st>>>(
        a.worlds, a.nworlds, a.ph, a.n, do_push, a.cell_start, a.cell_of, qin,
        qout, a.vel, a.vel_out, a.keys, a.ctrl, a.run_if, a.part, a.count);
  else if (final_pass)
    k_jacobi<true, false><<<blocks, threads, 0, st>>>(
        a.worlds, a.nworlds, a.ph, a.n, do_push, a.cell_start, a.cell_of, qin,
        qout, a.vel, a.vel_out, a.keys, a.ctrl, a.run_if, nullptr, a.count);
  else
    k_jacobi<false, false><<<blocks, threads, 0, st>>>(
        a.worlds, a.nworlds, a.ph, a.n, do_push, a.cell_start, a.cell_of, qin,
        qout, nullptr, nullptr, nullptr, a.ctrl, a.run_if, nullptr, CountDev{});
  return cudaGetLastError();
}

}  // namespace wrach
