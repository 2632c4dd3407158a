/*
 * wrach_oracle.c -- CPU restatement of wrach's per-frame particle physics step.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library and the timed CPU
 * baseline.  Never linked into the product.  Build: oracle/build_oracle.py
 * (gcc -O2 -ffp-contract=off -fno-fast-math -fopenmp).
 *
 * Table layout (the reference's `indices` buffer, C+2 u32 for C grid cells,
 * runners/bevy/src/spatial_bin.rs:103-149 and
 * runners/bevy/src/compute/builder.rs:32-33):
 *   table[0]     = 0
 *   table[c + 1] = index of the first particle of cell c   (c in 0..C-1)
 *   table[C + 1] = particles_in_frame_count
 * so cell c holds the particles [table[c + 1], table[c + 2]).
 */
#include "wrach_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int wo_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void wo_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* Rust's saturating `f32 as i32` (NaN -> 0). */
static int32_t sat_i32(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT32_MAX;
  if (f <= -2147483648.0f) return INT32_MIN;
  return (int32_t)f;
}

/* SpatialBin::get_cell_coord (runners/bevy/src/spatial_bin.rs:48-64):
 * `x.div_euclid(cell_size) as i32`, with Rust's f32::div_euclid
 * (q = trunc(x / d); if x % d < 0 then q - 1) and saturating cast. */
int32_t wo_cell_coord(float x, uint32_t cell_size) {
  float d = (float)cell_size;
  float q = truncf(x / d);
  if (fmodf(x, d) < 0.0f) q = q - 1.0f;
  return sat_i32(q);
}

/* SpatialBin::get_active_cells / update_grid_size
 * (runners/bevy/src/spatial_bin.rs:68-95): the grid spans the cells of the
 * viewport's bottom-left and top-right corners, inclusive.  The viewport is
 * (anchor, anchor + dimensions) as in WrachState::new (state.rs:65-80). */
static void world_corners(const wo_world *w, int32_t bl[2], int32_t tr[2]) {
  float x1 = w->view_anchor[0] + w->view_dimensions[0];
  float y1 = w->view_anchor[1] + w->view_dimensions[1];
  bl[0] = wo_cell_coord(w->view_anchor[0], w->cell_size);
  bl[1] = wo_cell_coord(w->view_anchor[1], w->cell_size);
  tr[0] = wo_cell_coord(x1, w->cell_size);
  tr[1] = wo_cell_coord(y1, w->cell_size);
}

void wo_world_init(wo_world *w, float width, float height, float anchor_x,
                   float anchor_y, uint32_t cell_size) {
  int32_t bl[2], tr[2];
  memset(w, 0, sizeof(*w));
  w->view_dimensions[0] = width;
  w->view_dimensions[1] = height;
  w->view_anchor[0] = anchor_x;
  w->view_anchor[1] = anchor_y;
  w->cell_size = cell_size;
  world_corners(w, bl, tr);
  w->grid_dimensions[0] = tr[0] >= bl[0] ? (uint32_t)(tr[0] - bl[0] + 1) : 0u;
  w->grid_dimensions[1] = tr[1] >= bl[1] ? (uint32_t)(tr[1] - bl[1] + 1) : 0u;
}

/* The active cell list in row-major order (spatial_bin.rs:78-86). */
uint32_t wo_active_cells(const wo_world *w, int32_t *cells_xy) {
  int32_t bl[2], tr[2];
  uint32_t n = 0;
  world_corners(w, bl, tr);
  for (int64_t y = bl[1]; y <= tr[1]; ++y)
    for (int64_t x = bl[0]; x <= tr[0]; ++x) {
      if (cells_xy) {
        cells_xy[2 * n] = (int32_t)x;
        cells_xy[2 * n + 1] = (int32_t)y;
      }
      ++n;
    }
  return n;
}

/* ParticleStore::max_particles_per_frame
 * (runners/bevy/src/particle_store.rs:116-133): cells * cs^2 plus 10 percent,
 * the percent rounded up. */
uint32_t wo_max_particles_per_frame(const wo_world *w) {
  uint32_t cells = w->grid_dimensions[0] * w->grid_dimensions[1];
  uint32_t cs2 = (uint32_t)(uint16_t)(w->cell_size * w->cell_size);
  uint32_t normal = cells * cs2;
  uint32_t one_percent = (normal + 99u) / 100u;
  return normal + 10u * one_percent;
}

/* ParticleStore::add_particle + SpatialBin::create_packed_data
 * (runners/bevy/src/particle_store.rs:54-59, spatial_bin.rs:103-149):
 * particles are grouped by the cell of their position, cells are walked in
 * row-major order, and inside a cell particles keep insertion order.  Cells
 * outside the viewport grid are dropped.  Returns the packed count, or -1 when
 * it exceeds `capacity`. */
int64_t wo_pack(const wo_world *w, uint32_t n, const float *pos,
                const float *vel, uint32_t capacity, uint32_t *table,
                float *out_pos, float *out_vel) {
  int32_t bl[2], tr[2];
  uint32_t gx = w->grid_dimensions[0], gy = w->grid_dimensions[1];
  uint32_t C = gx * gy;
  uint32_t *key = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
  uint32_t *cursor = (uint32_t *)calloc((size_t)C + 1, sizeof(uint32_t));
  uint32_t count = 0;
  world_corners(w, bl, tr);
  for (uint32_t i = 0; i < n; ++i) {
    int32_t cx = wo_cell_coord(pos[2 * i], w->cell_size);
    int32_t cy = wo_cell_coord(pos[2 * i + 1], w->cell_size);
    if (cx < bl[0] || cx > tr[0] || cy < bl[1] || cy > tr[1]) {
      key[i] = UINT32_MAX;
      continue;
    }
    key[i] = (uint32_t)((int64_t)(cy - bl[1]) * gx + (cx - bl[0]));
    cursor[key[i]]++;
    count++;
  }
  if (count > capacity) {
    free(key);
    free(cursor);
    return -1;
  }
  /* exclusive prefix -> table */
  table[0] = 0;
  uint32_t run = 0;
  for (uint32_t c = 0; c < C; ++c) {
    uint32_t k = cursor[c];
    table[c + 1] = run;
    cursor[c] = run;
    run += k;
  }
  table[C + 1] = run;
  for (uint32_t i = 0; i < n; ++i) {
    if (key[i] == UINT32_MAX) continue;
    uint32_t d = cursor[key[i]]++;
    out_pos[2 * d] = pos[2 * i];
    out_pos[2 * d + 1] = pos[2 * i + 1];
    out_vel[2 * d] = vel[2 * i];
    out_vel[2 * d + 1] = vel[2 * i + 1];
  }
  free(key);
  free(cursor);
  return count;
}

/* Frame-time cell key (assets/shaders/particles_per_cell.wgsl:14-27 and
 * pack_new_particle_data.wgsl:22-40): floor((p - anchor) / cell_size) per
 * axis, key = cy * gx + cx.  The WGSL leaves out-of-grid and NaN inputs
 * undefined; here they are clamped into the grid (NaN -> 0) and flagged. */
static uint32_t axis_cell(float p, float a, uint32_t cs, uint32_t g,
                          uint32_t *flags) {
  float f = floorf((p - a) / (float)cs);
  if (!(f >= 0.0f)) {
    *flags |= (f != f) ? (WO_FLAG_NAN | WO_FLAG_OUT_OF_GRID)
                       : WO_FLAG_OUT_OF_GRID;
    return 0u;
  }
  if (f >= (float)g) {
    *flags |= WO_FLAG_OUT_OF_GRID;
    return g - 1u;
  }
  return (uint32_t)f;
}

uint32_t wo_frame_key(const wo_world *w, float x, float y, uint32_t *flags) {
  uint32_t gx = w->grid_dimensions[0], gy = w->grid_dimensions[1];
  uint32_t cx = axis_cell(x, w->view_anchor[0], w->cell_size, gx, flags);
  uint32_t cy = axis_cell(y, w->view_anchor[1], w->cell_size, gy, flags);
  return cy * gx + cx;
}

/* ------------------------------------------------------------------------ */
/* Physics.  Generated for float and for double (the FP64 re-run).          */
/* ------------------------------------------------------------------------ */

/* Particle::enforce_boundaries (shaders/physics/src/particle.rs:46-70),
 * Particle::enforce_velocity with Rust's f32::clamp (particle.rs:73-77;
 * NaN passes through). */
#define DEFINE_LIMITS(T, SUF)                                                  \
  static void limits_##SUF(const wo_world *w, T vmax, T *px, T *py, T *vx,     \
                           T *vy) {                                            \
    T x0 = (T)w->view_anchor[0], y0 = (T)w->view_anchor[1];                    \
    T x1 = (T)(w->view_anchor[0] + w->view_dimensions[0]);                     \
    T y1 = (T)(w->view_anchor[1] + w->view_dimensions[1]);                     \
    if (*px > x1) { *px = x1; *vx = -*vx; }                                    \
    if (*px < x0) { *px = x0; *vx = -*vx; }                                    \
    if (*py > y1) { *py = y1; *vy = -*vy; }                                    \
    if (*py < y0) { *py = y0; *vy = -*vy; }                                    \
    if (*vx < -vmax) *vx = -vmax;                                              \
    if (*vx > vmax) *vx = vmax;                                                \
    if (*vy < -vmax) *vy = -vmax;                                              \
    if (*vy > vmax) *vy = vmax;                                                \
  }

DEFINE_LIMITS(float, f32)
DEFINE_LIMITS(double, f64)

/* Mode 0, one cell: World::physics_for_cell (shaders/physics/src/cell.rs:52-75)
 *  - Particles::new copies min(count, capacity) particles
 *    (shaders/physics/src/particles.rs:31-59);
 *  - Particles::pairs: i < j in order, distance = |p_i - p_j| (glam
 *    Vec2::distance), skip when > min_distance, 0 -> 0.0001, then
 *    push_close_particles_apart: force = 0.5 * (min - d) / d,
 *    dv = (p_j - p_i) * force, p_i -= dv, p_j += dv (particles.rs:62-93);
 *  - Particles::finish: integrate, boundaries, velocity clamp, write back to
 *    the same index (particles.rs:96-107, particle.rs:40-106);
 *  - handle_overflown_particles: particles past the capacity are only
 *    integrated and limited (cell.rs:79-95).
 * The index clear of cell.rs:116-131 belongs to the reference's in-place
 * table reuse and has no counterpart here (the rebin writes a fresh table). */
#define DEFINE_SOLVE_R(T, SUF, SQRT)                                           \
  static void solve_r_##SUF(const wo_world *w, const wo_physics *ph,           \
                            const uint32_t *table, const T *pin,               \
                            const T *vin, T *pout, T *vout) {                  \
    uint32_t C = w->grid_dimensions[0] * w->grid_dimensions[1];                \
    uint32_t cap = ph->cell_capacity;                                          \
    T mind = (T)ph->min_distance, vmax = (T)ph->max_velocity;                  \
    _Pragma("omp parallel for schedule(dynamic, 4096)")                        \
    for (int64_t c = 0; c < (int64_t)C; ++c) {                                 \
      uint32_t s = table[c + 1], e = table[c + 2];                             \
      uint32_t cnt = e - s, m = cnt < cap ? cnt : cap;                         \
      T px[64], py[64], vx[64], vy[64];                                        \
      T *Px = px, *Py = py, *Vx = vx, *Vy = vy;                                \
      if (m > 64) {                                                            \
        Px = (T *)malloc(sizeof(T) * 4 * m);                                   \
        Py = Px + m; Vx = Py + m; Vy = Vx + m;                                 \
      }                                                                        \
      for (uint32_t i = 0; i < m; ++i) {                                       \
        Px[i] = pin[2 * (s + i)]; Py[i] = pin[2 * (s + i) + 1];                \
        Vx[i] = vin[2 * (s + i)]; Vy[i] = vin[2 * (s + i) + 1];                \
      }                                                                        \
      for (uint32_t i = 0; i < m; ++i)                                         \
        for (uint32_t j = i + 1; j < m; ++j) {                                 \
          T ex = Px[i] - Px[j], ey = Py[i] - Py[j];                            \
          T d = SQRT(ex * ex + ey * ey);                                       \
          if (d > mind) continue;                                              \
          if (d == (T)0) d = (T)0.0001f;                                       \
          T f = ((T)0.5 * (mind - d)) / d;                                     \
          T dx = (Px[j] - Px[i]) * f, dy = (Py[j] - Py[i]) * f;                \
          Px[i] = Px[i] - dx; Py[i] = Py[i] - dy;                              \
          Px[j] = Px[j] + dx; Py[j] = Py[j] + dy;                              \
        }                                                                      \
      for (uint32_t i = 0; i < m; ++i) {                                       \
        T qx = Px[i] + Vx[i], qy = Py[i] + Vy[i], ux = Vx[i], uy = Vy[i];      \
        limits_##SUF(w, vmax, &qx, &qy, &ux, &uy);                             \
        pout[2 * (s + i)] = qx; pout[2 * (s + i) + 1] = qy;                    \
        vout[2 * (s + i)] = ux; vout[2 * (s + i) + 1] = uy;                    \
      }                                                                        \
      for (uint32_t i = s + m; i < e; ++i) {                                   \
        T ux = vin[2 * i], uy = vin[2 * i + 1];                                \
        T qx = pin[2 * i] + ux, qy = pin[2 * i + 1] + uy;                      \
        limits_##SUF(w, vmax, &qx, &qy, &ux, &uy);                             \
        pout[2 * i] = qx; pout[2 * i + 1] = qy;                                \
        vout[2 * i] = ux; vout[2 * i + 1] = uy;                                \
      }                                                                        \
      if (m > 64) free(Px);                                                    \
    }                                                                          \
  }

/* Mode 1 (extended physics; not in the reference, parity unpinned by it).
 * The reference's per-cell physics widened to the 3x3 cell neighbourhood and
 * iterated, with gravity.  As in the reference (cell.rs:29-30, 79-95) only
 * the first `cell_capacity` particles of a cell (in table order) take part in
 * the pair pushes; the rest of an over-full cell only integrate.
 *   q = p
 *   repeat `iterations` times (Jacobi: every particle reads the previous q):
 *     for each taking-part particle i of cell (cx, cy):
 *       acc = 0; for the 3x3 cells around (cx, cy) in row-major order, for
 *       each taking-part particle j != i of that cell in table order:
 *         d = |q_i - q_j|; skip if d > min; if d == 0: d = 0.0001
 *         f = 0.5 * (min - d) / d          (the reference's pair push)
 *         acc += (q_j - q_i) * f
 *       q_i' = q_i - acc
 *   then v.y -= gravity; p = q + v; boundaries; velocity clamp.
 * Velocities change only at the walls and the clamp, as in the reference.
 * Every pair's contributions to i and j are exact negatives, so the push is
 * momentum-conserving; the fixed summation order makes it deterministic under
 * any parallel schedule. */
#define DEFINE_SOLVE_X(T, SUF, SQRT)                                           \
  static void solve_x_##SUF(const wo_world *w, const wo_physics *ph,           \
                            const uint32_t *table, const T *pin,               \
                            const T *vin, T *pout, T *vout) {                  \
    int64_t gx = w->grid_dimensions[0], gy = w->grid_dimensions[1];            \
    uint32_t n = table[gx * gy + 1], cap = ph->cell_capacity;                  \
    T mind = (T)ph->min_distance, vmax = (T)ph->max_velocity;                  \
    T *qa = (T *)malloc(sizeof(T) * 2 * (n ? n : 1));                          \
    T *qb = (T *)malloc(sizeof(T) * 2 * (n ? n : 1));                          \
    memcpy(qa, pin, sizeof(T) * 2 * n);                                        \
    for (uint32_t it = 0; it < ph->iterations; ++it) {                         \
      _Pragma("omp parallel for schedule(dynamic, 64)")                        \
      for (int64_t cy = 0; cy < gy; ++cy)                                      \
        for (int64_t cx = 0; cx < gx; ++cx) {                                  \
          uint32_t s = table[cy * gx + cx + 1], e = table[cy * gx + cx + 2];   \
          uint32_t m = e - s < cap ? e - s : cap;                              \
          for (uint32_t i = s; i < s + m; ++i) {                               \
            T qx = qa[2 * i], qy = qa[2 * i + 1], ax = 0, ay = 0;              \
            for (int64_t ny = cy - 1; ny <= cy + 1; ++ny) {                    \
              if (ny < 0 || ny >= gy) continue;                                \
              for (int64_t nx = cx - 1; nx <= cx + 1; ++nx) {                  \
                if (nx < 0 || nx >= gx) continue;                              \
                uint32_t js = table[ny * gx + nx + 1];                         \
                uint32_t je = table[ny * gx + nx + 2];                         \
                if (je - js > cap) je = js + cap;                              \
                for (uint32_t j = js; j < je; ++j) {                           \
                  if (j == i) continue;                                        \
                  T dx = qa[2 * j] - qx, dy = qa[2 * j + 1] - qy;              \
                  T d = SQRT(dx * dx + dy * dy);                               \
                  if (d > mind) continue;                                      \
                  if (d == (T)0) d = (T)0.0001f;                               \
                  T f = ((T)0.5 * (mind - d)) / d;                             \
                  ax = ax + dx * f;                                            \
                  ay = ay + dy * f;                                            \
                }                                                              \
              }                                                                \
            }                                                                  \
            qb[2 * i] = qx - ax;                                               \
            qb[2 * i + 1] = qy - ay;                                           \
          }                                                                    \
          for (uint32_t i = s + m; i < e; ++i) {                               \
            qb[2 * i] = qa[2 * i];                                             \
            qb[2 * i + 1] = qa[2 * i + 1];                                     \
          }                                                                    \
        }                                                                      \
      T *t = qa; qa = qb; qb = t;                                              \
    }                                                                          \
    T g = (T)ph->gravity;                                                      \
    _Pragma("omp parallel for schedule(static)")                               \
    for (int64_t i = 0; i < (int64_t)n; ++i) {                                 \
      T ux = vin[2 * i], uy = vin[2 * i + 1] - g;                              \
      T qx = qa[2 * i] + ux, qy = qa[2 * i + 1] + uy;                          \
      limits_##SUF(w, vmax, &qx, &qy, &ux, &uy);                               \
      pout[2 * i] = qx; pout[2 * i + 1] = qy;                                  \
      vout[2 * i] = ux; vout[2 * i + 1] = uy;                                  \
    }                                                                          \
    free(qa);                                                                  \
    free(qb);                                                                  \
  }

DEFINE_SOLVE_R(float, f32, sqrtf)
DEFINE_SOLVE_R(double, f64, sqrt)
DEFINE_SOLVE_X(float, f32, sqrtf)
DEFINE_SOLVE_X(double, f64, sqrt)

void wo_solve(const wo_world *w, const wo_physics *ph, const uint32_t *table,
              const float *pin, const float *vin, float *pout, float *vout) {
  if (ph->mode == 0)
    solve_r_f32(w, ph, table, pin, vin, pout, vout);
  else
    solve_x_f32(w, ph, table, pin, vin, pout, vout);
}

void wo_solve_f64(const wo_world *w, const wo_physics *ph,
                  const uint32_t *table, const double *pin, const double *vin,
                  double *pout, double *vout) {
  if (ph->mode == 0)
    solve_r_f64(w, ph, table, pin, vin, pout, vout);
  else
    solve_x_f64(w, ph, table, pin, vin, pout, vout);
}

/* Rebin after the solve: the count pass (particles_per_cell.wgsl:7-30), the
 * exclusive scan over the table (prefix_sum.wgsl:17-123) and the pack pass
 * (pack_new_particle_data.wgsl:10-45).  The reference places particles inside
 * a cell with atomicSub, so its order there is unspecified (its own test
 * sorts within a cell, runners/bevy/src/compute/04_pack_particle_data.rs:
 * 127-134).  The order defined here is the stable one: a cell's particles keep
 * the order they had in the solve output, which is also what
 * create_packed_data produces when the frame's particles are re-added in
 * buffer order.  Returns the flag bits. */
uint32_t wo_rebin(const wo_world *w, uint32_t n, const float *pout,
                  const float *vout, uint32_t *keys, uint32_t *table,
                  float *pin, float *vin) {
  uint32_t C = w->grid_dimensions[0] * w->grid_dimensions[1];
  uint32_t flags = 0;
#pragma omp parallel for schedule(static) reduction(| : flags)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    uint32_t f = 0;
    keys[i] = wo_frame_key(w, pout[2 * i], pout[2 * i + 1], &f);
    flags |= f;
  }
  uint32_t *cursor = (uint32_t *)calloc((size_t)C + 1, sizeof(uint32_t));
  for (uint32_t i = 0; i < n; ++i) cursor[keys[i]]++;
  table[0] = 0;
  uint32_t run = 0;
  for (uint32_t c = 0; c < C; ++c) {
    uint32_t k = cursor[c];
    table[c + 1] = run;
    cursor[c] = run;
    run += k;
  }
  table[C + 1] = run;
  for (uint32_t i = 0; i < n; ++i) {
    uint32_t d = cursor[keys[i]]++;
    pin[2 * d] = pout[2 * i];
    pin[2 * d + 1] = pout[2 * i + 1];
    vin[2 * d] = vout[2 * i];
    vin[2 * d + 1] = vout[2 * i + 1];
  }
  free(cursor);
  return flags;
}

/* One frame = solve on the binned state, then rebin (the pass order of
 * runners/bevy/src/compute/builder.rs:86-89).  `table`, `pos` and `vel` hold
 * the binned state and are updated in place.  Returns the OR of the flags. */
uint32_t wo_step(const wo_world *w, const wo_physics *ph, uint32_t nsteps,
                 uint32_t *table, float *pos, float *vel) {
  uint32_t C = w->grid_dimensions[0] * w->grid_dimensions[1];
  uint32_t n = table[C + 1];
  float *po = (float *)malloc(sizeof(float) * 2 * (n ? n : 1));
  float *vo = (float *)malloc(sizeof(float) * 2 * (n ? n : 1));
  uint32_t *keys = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
  uint32_t flags = 0;
  for (uint32_t s = 0; s < nsteps; ++s) {
    wo_solve(w, ph, table, pos, vel, po, vo);
    flags |= wo_rebin(w, n, po, vo, keys, table, pos, vel);
  }
  free(po);
  free(vo);
  free(keys);
  return flags;
}
