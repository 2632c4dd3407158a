// Solve kernels: the collision/constraint pass plus the fused
// integrate + boundary + velocity-clamp epilogue, which also emits each
// particle's next cell key for the rebin and the largest cell displacement of
// the frame (the rebin's window radius).
//
// Reference-mode kernel: one thread per cell, the sequential sweep of
// World::physics_for_cell (shaders/physics/src/cell.rs:52-95).
// Extended-mode kernel: one thread per particle, a Jacobi iteration over the
// particle's 3x3 cell neighbourhood.
#include "wrach_internal.cuh"
#include "wrach_kernels.h"

namespace wrach {

namespace {

__device__ __forceinline__ void emit_key(const WorldDev& w, uint32_t ocx,
                                         uint32_t ocy, float px, float py,
                                         uint32_t& key, uint32_t& disp,
                                         uint32_t& flags) {
  uint32_t ncx = axis_cell(px, w.ax, w.cs, w.gx, flags);
  uint32_t ncy = axis_cell(py, w.ay, w.cs, w.gy, flags);
  key = w.cell_off + ncy * w.gx + ncx;
  uint32_t dx = ncx > ocx ? ncx - ocx : ocx - ncx;
  uint32_t dy = ncy > ocy ? ncy - ocy : ocy - ncy;
  disp = max(disp, max(dx, dy));
}

__device__ __forceinline__ void publish_frame_stats(Ctrl* ctrl, uint32_t disp,
                                                    uint32_t flags) {
  uint32_t wd = warp_max_u32(disp);
  uint32_t wf = warp_or_u32(flags);
  if ((threadIdx.x & 31) == 0) {
    if (wd) atomicMax(&ctrl->dmax, wd);
    if (wf) atomicOr(&ctrl->flags, wf);
  }
}

// Reference mode, one thread per global cell.
//  - Particles::new: the first min(count, capacity) particles of the cell
//    (shaders/physics/src/particles.rs:31-59)
//  - Particles::pairs / push_close_particles_apart: Gauss-Seidel over i < j
//    (particles.rs:62-93)
//  - Particles::finish: integrate, boundaries, clamp, write (particles.rs:
//    96-107, particle.rs:40-106)
//  - handle_overflown_particles: the rest only integrate (cell.rs:79-95)
__global__ void __launch_bounds__(256)
k_solve_reference(const WorldDev* __restrict__ worlds, int nworlds,
                  PhysDev ph, uint32_t ncells,
                  const uint32_t* __restrict__ cell_start,
                  const float2* __restrict__ pin, const float2* __restrict__ vin,
                  float2* __restrict__ pout, float2* __restrict__ vout,
                  uint32_t* __restrict__ keys, Ctrl* ctrl) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t disp = 0, flags = 0;
  if (c < ncells) {
    const WorldDev w = worlds[world_of_cell(worlds, nworlds, c)];
    const uint32_t local = c - w.cell_off;
    const uint32_t ocx = local % w.gx, ocy = local / w.gx;
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
                         ph.min_d, f))
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
      emit_key(w, ocx, ocy, qx, qy, keys[s + i], disp, flags);
    }
    for (uint32_t i = s + m; i < e; ++i) {
      float2 p = pin[i], v = vin[i];
      float qx = __fadd_rn(p.x, v.x), qy = __fadd_rn(p.y, v.y);
      float ux = v.x, uy = v.y;
      enforce_limits(w, ph.vmax, qx, qy, ux, uy);
      pout[i] = make_float2(qx, qy);
      vout[i] = make_float2(ux, uy);
      emit_key(w, ocx, ocy, qx, qy, keys[i], disp, flags);
    }
  }
  publish_frame_stats(ctrl, disp, flags);
}

// Extended mode, one Jacobi iteration, one thread per particle.  The
// neighbour order is fixed (3x3 cells in row-major order, table order inside
// a row), so the sum is deterministic.  FINAL fuses gravity, integration,
// boundaries, the velocity clamp and the key emission.
template <bool FINAL>
__global__ void __launch_bounds__(256)
k_jacobi(const WorldDev* __restrict__ worlds, int nworlds, PhysDev ph,
         uint32_t n, int do_push, const uint32_t* __restrict__ cell_start,
         const uint32_t* __restrict__ cell_of, const float2* __restrict__ qin,
         float2* __restrict__ qout, const float2* __restrict__ vin,
         float2* __restrict__ vout, uint32_t* __restrict__ keys, Ctrl* ctrl) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t disp = 0, flags = 0;
  if (i < n) {
    const uint32_t c = cell_of[i];
    const WorldDev w = worlds[world_of_cell(worlds, nworlds, c)];
    const uint32_t local = c - w.cell_off;
    const uint32_t cx = local % w.gx, cy = local / w.gx;
    const float2 qi = qin[i];
    float ax = 0.0f, ay = 0.0f;
    if (do_push) {
      const uint32_t x0 = cx > 0 ? cx - 1 : 0;
      const uint32_t x1 = cx + 1 < w.gx ? cx + 1 : w.gx - 1;
      const uint32_t y0 = cy > 0 ? cy - 1 : 0;
      const uint32_t y1 = cy + 1 < w.gy ? cy + 1 : w.gy - 1;
      for (uint32_t ny = y0; ny <= y1; ++ny) {
        const uint32_t rb = w.cell_off + ny * w.gx;
        const uint32_t js = cell_start[rb + x0], je = cell_start[rb + x1 + 1];
        for (uint32_t j = js; j < je; ++j) {
          if (j == i) continue;
          const float2 qj = qin[j];
          const float dx = __fsub_rn(qj.x, qi.x), dy = __fsub_rn(qj.y, qi.y);
          float f;
          if (!push_factor(dx, dy, ph.min_d, f)) continue;
          ax = __fadd_rn(ax, __fmul_rn(dx, f));
          ay = __fadd_rn(ay, __fmul_rn(dy, f));
        }
      }
    }
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
      emit_key(w, cx, cy, px, py, keys[i], disp, flags);
    }
  }
  if (FINAL) publish_frame_stats(ctrl, disp, flags);
}

}  // namespace

cudaError_t launch_solve_reference(const SolveArgs& a, cudaStream_t st) {
  if (a.ncells == 0) return cudaSuccess;
  const uint32_t threads = 256;
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
  const uint32_t threads = 256;
  const uint32_t blocks = (a.n + threads - 1) / threads;
  if (final_pass)
    k_jacobi<true><<<blocks, threads, 0, st>>>(
        a.worlds, a.nworlds, a.ph, a.n, do_push, a.cell_start, a.cell_of, qin,
        qout, a.vel, a.vel_out, a.keys, a.ctrl);
  else
    k_jacobi<false><<<blocks, threads, 0, st>>>(
        a.worlds, a.nworlds, a.ph, a.n, do_push, a.cell_start, a.cell_of, qin,
        qout, nullptr, nullptr, nullptr, a.ctrl);
  return cudaGetLastError();
}

}  // namespace wrach
