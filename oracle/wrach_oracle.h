/*
 * wrach_oracle.h -- CPU restatement of wrach's per-frame particle physics step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the CUDA library is
 * compared against (tests/, the smoke check and bench.py's CPU baseline leg).
 * Nothing in the product path links, loads or calls it.
 *
 * Parity anchor: the reference is a Rust/rust-gpu + WGSL code base that cannot
 * be compiled here (no Rust toolchain, no graphics adapter), so this file
 * restates its algorithm in plain C, citing the reference file:line each
 * function follows, and is pinned against the known-answer tests that the
 * reference's own test modules hold (see tests/test_oracle_golden.py).
 *
 * Arithmetic contract (shared with the CUDA kernels): IEEE-754 binary32,
 * round-to-nearest, no FMA contraction (-ffp-contract=off), correctly rounded
 * sqrt and division, denormals preserved.  Under that contract the reference's
 * own CPU known-answer test (shaders/physics/src/particles.rs:128-146)
 * reproduces bit for bit.
 */
#ifndef WRACH_ORACLE_H
#define WRACH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-world settings.  Same 32-byte layout as the reference's uniform
 * (runners/bevy/src/config_shader.rs:15-29, shaders/shared/src/lib.rs:19-31,
 * assets/shaders/types.wgsl:3-15). */
typedef struct {
  float view_dimensions[2];
  float view_anchor[2];
  uint32_t grid_dimensions[2];
  uint32_t cell_size;
  uint32_t particles_in_frame_count;
} wo_world;

/* Physics parameters.  mode 0 = the reference's physics (same-cell
 * Gauss-Seidel sweep, cell capacity 9, no gravity); mode 1 = the extended
 * physics (3x3-cell Jacobi iterations with gravity). */
typedef struct {
  uint32_t mode;
  uint32_t iterations;    /* mode 1 only; mode 0 always sweeps once */
  float gravity;          /* mode 1 only; v.y -= gravity every frame */
  float min_distance;     /* 1.0 (shaders/physics/src/particles.rs:18) */
  float max_velocity;     /* 1.0 (shaders/physics/src/particle.rs:74) */
  uint32_t cell_capacity; /* 9 (shaders/physics/src/cell.rs:29-30) */
} wo_physics;

/* flag bits reported by the frame functions */
#define WO_FLAG_OUT_OF_GRID 1u /* a key had to be clamped into the grid */
#define WO_FLAG_NAN 2u         /* a non-finite position was binned */

int32_t wo_cell_coord(float x, uint32_t cell_size);
void wo_world_init(wo_world *w, float width, float height, float anchor_x,
                   float anchor_y, uint32_t cell_size);
uint32_t wo_active_cells(const wo_world *w, int32_t *cells_xy);
uint32_t wo_max_particles_per_frame(const wo_world *w);
int64_t wo_pack(const wo_world *w, uint32_t n, const float *pos,
                const float *vel, uint32_t capacity, uint32_t *table,
                float *out_pos, float *out_vel);
uint32_t wo_frame_key(const wo_world *w, float x, float y, uint32_t *flags);
void wo_solve(const wo_world *w, const wo_physics *ph, const uint32_t *table,
              const float *pin, const float *vin, float *pout, float *vout);
void wo_solve_f64(const wo_world *w, const wo_physics *ph,
                  const uint32_t *table, const double *pin, const double *vin,
                  double *pout, double *vout);
uint32_t wo_rebin(const wo_world *w, uint32_t n, const float *pout,
                  const float *vout, uint32_t *keys, uint32_t *table,
                  float *pin, float *vin);
uint32_t wo_step(const wo_world *w, const wo_physics *ph, uint32_t nsteps,
                 uint32_t *table, float *pos, float *vel);
int wo_num_threads(void);
void wo_set_num_threads(int n);

#ifdef __cplusplus
}
#endif

#endif
