/*
 * wrach.h -- C ABI of the GB300 (sm_103a) CUDA implementation of wrach's
 * per-frame particle physics step.
 *
 * This boundary replaces the reference's `WrachAPI` surface
 * (runners/api/src/lib.rs:17-88) and the wgpu compute pipeline behind it
 * (runners/bevy/src/compute/builder.rs:24-92, runners/bevy/src/plugin/
 * build.rs:88-158).  Plain pointers and sizes only; every call returns a
 * status code (WRACH_OK == 0) where the reference panics.
 *
 * Threading: a context is owned by one thread at a time (the reference's
 * `&mut self`).  All device work of a context runs in order on the context's
 * own CUDA stream; wrach_read and wrach_sync block until it is done.
 *
 * Data layout (the reference's, runners/bevy/src/spatial_bin.rs:20-33):
 *   positions, velocities: `capacity` float pairs (x, y), in cell order;
 *     wrach_read writes the first particles_in_frame_count of them and
 *     leaves the rest as they were (the reference's readback returns
 *     whatever its buffers hold there);
 *   indices: grid cells + 2 u32, indices[0] = 0, indices[c + 1] = first
 *     particle of cell c, indices[cells + 1] = particles_in_frame_count.
 */
#ifndef WRACH_H
#define WRACH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WRACH_OK 0
#define WRACH_ERR_INVALID_ARGUMENT 1 /* null pointer, zero size, bad enum */
#define WRACH_ERR_CAPACITY 2         /* more particles than the frame holds */
#define WRACH_ERR_CUDA 3             /* a CUDA call failed; see last_error */
#define WRACH_ERR_OUT_OF_MEMORY 4    /* device allocation failed */
#define WRACH_ERR_DEVICE 5           /* a device-side check fired (flags) */
#define WRACH_ERR_UNSUPPORTED 6      /* no sm_103a device / feature absent */

/* Physics modes. */
#define WRACH_MODE_REFERENCE 0u /* the reference's same-cell sweep */
#define WRACH_MODE_EXTENDED 1u  /* 3x3-cell Jacobi iterations + gravity */

/* Sticky device flags (wrach_flags). */
#define WRACH_FLAG_OUT_OF_GRID 1u /* a key was clamped into the grid */
#define WRACH_FLAG_NAN 2u         /* a non-finite position was binned */
#define WRACH_FLAG_TIMEOUT 4u     /* a bounded device wait gave up */
#define WRACH_FLAG_OVERFLOW 8u    /* particles did not fit the output
                                     (wrach_pack_noalloc's status only) */

/* The reference's 32-byte shader uniform, field for field
 * (runners/bevy/src/config_shader.rs:15-29, shaders/shared/src/lib.rs:19-31,
 * assets/shaders/types.wgsl:3-15). */
typedef struct WrachWorldSettings {
  float view_dimensions[2];
  float view_anchor[2];
  uint32_t grid_dimensions[2];
  uint32_t cell_size;
  uint32_t particles_in_frame_count;
} WrachWorldSettings;

/* WrachConfig (runners/bevy/src/config_app.rs:10-36) plus the physics knobs
 * the reference hard-codes (shaders/physics/src/particles.rs:18,
 * particle.rs:74, cell.rs:29-30). */
typedef struct WrachConfig {
  float width;             /* dimensions.0 (default 480) */
  float height;            /* dimensions.1 (default 352) */
  float anchor_x;          /* view_anchor (always 0 in the reference) */
  float anchor_y;
  uint32_t cell_size;      /* default 3 (shaders/shared/src/lib.rs:34) */
  uint32_t mode;           /* WRACH_MODE_* (default REFERENCE) */
  uint32_t iterations;     /* EXTENDED only (default 4) */
  float gravity;           /* EXTENDED only, px/frame^2 (default 0) */
  float min_distance;      /* default 1.0 */
  float max_velocity;      /* default 1.0 */
  uint32_t cell_capacity;  /* particles of a cell that interact, 1..16,
                              default 9 */
  uint32_t capacity;       /* 0 = max_particles_per_frame of the grid */
  int32_t device;          /* CUDA ordinal (default 0) */
  uint32_t rebin_blocks;   /* blocks of the rebin's large-cell sort (cells of
                              more than 64 particles), 0 = 8 per SM */
  uint32_t solve_block;    /* threads per block of the solve kernels, a
                              multiple of 32 up to 512, 0 = 128 */
  uint32_t solve_per_thread; /* particles each thread of the extended solve
                              takes in turn (the grid shrinks accordingly;
                              32 x this = particles per warp), 0 = 1 */
  uint32_t reserved[4];
} WrachConfig;

typedef struct WrachContext WrachContext;

/* Defaults of WrachConfig::default() (config_app.rs:23-36). */
int wrach_config_default(WrachConfig *config);

/* WrachAPI::new + PhysicsComputeWorker::build (runners/api/src/lib.rs:30-45,
 * runners/bevy/src/compute/builder.rs:24-92): sizes the grid from the
 * viewport (spatial_bin.rs:68-95) and allocates the device buffers. */
int wrach_create(const WrachConfig *config, WrachContext **out);

/* Many independent worlds stepped together.  `dims` holds 2*nworlds floats
 * (width, height per world); every other setting comes from `config`.
 * World w's data is addressed with the `world` argument of the calls below.
 * No counterpart in the reference (one world per app). */
int wrach_create_batch(const WrachConfig *config, uint32_t nworlds,
                       const float *dims, WrachContext **out);

int wrach_destroy(WrachContext *ctx);

/* WrachAPI::add_particles / WrachState::add_particles
 * (runners/api/src/lib.rs:78-81, runners/bevy/src/state.rs:90-101): appends
 * n particles (host arrays of n float pairs) to the world's store and re-packs
 * the whole store into the frame on the device: the cell-ordered layout of
 * SpatialBin::create_packed_data (spatial_bin.rs:103-149), insertion order
 * inside a cell, particles outside the viewport grid kept in the store but
 * left out of the frame.  Like the reference, a re-pack restarts the frame
 * from the store's particles. */
int wrach_add_particles(WrachContext *ctx, uint32_t world, const float *pos,
                        const float *vel, uint32_t n);

/* Replaces the world's store with these n particles and re-packs the frame
 * from them (ParticleStore::add_particles_to_cell followed by
 * create_packed_data, runners/bevy/src/particle_store.rs:62-65,103-149,
 * for the whole store at once).  The host arrays are read before the call
 * returns (pinned memory makes the copies faster).  With one world and no
 * more particles than the frame capacity, the last steps of the re-pack may
 * still be running on the context's stream when it returns; every later call
 * on the context is ordered after them. */
int wrach_set_particles(WrachContext *ctx, uint32_t world, const float *pos,
                        const float *vel, uint32_t n);

/* As wrach_add_particles with device-resident input arrays. */
int wrach_add_particles_device(WrachContext *ctx, uint32_t world,
                               const float *d_pos, const float *d_vel,
                               uint32_t n);

/* Packs n particles (device arrays of n float pairs, any order) into the
 * cell order of the world `config` describes (width, height, anchor,
 * cell_size, device), writing d_pos_out/d_vel_out (out_capacity float pairs
 * each) and d_indices (grid cells + 2 u32, the reference's table; its last
 * entry is the number of particles in the frame).  The same result as
 * wrach_set_particles followed by wrach_read, for callers that cannot
 * allocate GPU memory (code inside a host callback or a real-time loop that
 * must not wait on the allocator, a plugin whose host owns all device memory,
 * a process with no memory to spare): this call allocates nothing and
 * calls no allocating routine.  Its temporaries live in one static device
 * array sized for at most 131,072 particles and 524,288 grid cells (about
 * 6.3 MB on every GPU that loads the library, until exit); larger inputs
 * return WRACH_ERR_CAPACITY.  Particles past out_capacity are not written
 * (d_indices still counts them).  The first call on a device looks up that
 * array's device address (cudaGetSymbolAddress), so make it before any
 * stream capture.  Every call shares the array: calls that overlap on the GPU
 * race, so keep them on one stream.  Asynchronous on `stream` (a
 * cudaStream_t, NULL = the legacy default stream): the return code covers
 * the arguments and the launches only.  What only the device knows goes to
 * d_status (optional, NULL = not wanted; 2 u32 of device memory), written
 * after the call's kernels: d_status[0] = WRACH_FLAG_* bits
 * (WRACH_FLAG_TIMEOUT if a bounded grid barrier of the sort gave up, the
 * output then being unreliable; WRACH_FLAG_OVERFLOW if particles did not fit
 * out_capacity), d_status[1] = the number that did not fit.  No counterpart
 * in the reference. */
int wrach_pack_noalloc(const WrachConfig *config, const float *d_pos,
                       const float *d_vel, uint32_t n, float *d_pos_out,
                       float *d_vel_out, uint32_t out_capacity,
                       uint32_t *d_indices, uint32_t *d_status, void *stream);

/* nsteps frames of the physics pass list (builder.rs:86-89): solve, count,
 * scan, pack.  Asynchronous on the context's stream. */
int wrach_step(WrachContext *ctx, uint32_t nsteps);

/* WrachAPI::tick's readback (runners/bevy/src/plugin/build.rs:135-158,
 * runners/api/src/lib.rs:58-74): copies the world's frame into host arrays.
 * positions/velocities take 2*capacity floats, indices cells+2 u32; any of
 * the three may be NULL.  `capacity` must be at least the world's frame
 * capacity (wrach_capacity).  Blocks until the copies are done. */
int wrach_read(WrachContext *ctx, uint32_t world, float *positions,
               float *velocities, uint32_t *indices, uint32_t capacity);

/* WrachAPI::tick (runners/api/src/lib.rs:49-52): one step then a read. */
int wrach_tick(WrachContext *ctx, uint32_t world, float *positions,
               float *velocities, uint32_t *indices, uint32_t capacity);

/* The draw pass (assets/shaders/draw.wgsl:18-40, MSAA 4 from
 * runners/bevy/src/render/pipeline.rs:52-56) without a graphics API: each
 * particle of the world's frame as a white square of half-size 0.4 world
 * units on black, 4 samples per pixel, into `image` (height_px rows of
 * width_px bytes, row 0 at the top, y up in the world).  Blocks. */
int wrach_render(WrachContext *ctx, uint32_t world, uint32_t width_px,
                 uint32_t height_px, uint8_t *image);

/* Settings of a world (the uniform, with particles_in_frame_count). */
int wrach_get_settings(WrachContext *ctx, uint32_t world,
                       WrachWorldSettings *out);

/* ParticleStore::max_particles_per_frame (particle_store.rs:116-133) for a
 * grid of `cells` cells of size `cell_size`. */
uint32_t wrach_max_particles_per_frame(uint32_t cells, uint32_t cell_size);

/* The frame capacity of a world (the length of its readback arrays). */
uint32_t wrach_capacity(WrachContext *ctx, uint32_t world);
uint32_t wrach_num_worlds(WrachContext *ctx);

int wrach_sync(WrachContext *ctx);

/* The cell key of each of the world's frame particles, in frame order:
 * cy * gx + cx, the key the reference's count pass computes
 * (particles_per_cell.wgsl:14-27), world-local.  `keys` takes at least the
 * frame's particle count (particles_in_frame_count) entries.  Blocks. */
int wrach_read_keys(WrachContext *ctx, uint32_t world, uint32_t *keys,
                    uint32_t capacity);

/* Sticky device flags (WRACH_FLAG_*) seen since create; blocks. */
int wrach_flags(WrachContext *ctx, uint32_t *flags);

/* Counters of the device side (no counterpart in the reference). */
typedef struct WrachStats {
  uint32_t flags;             /* sticky WRACH_FLAG_* bits */
  uint32_t frames;            /* frames stepped since create */
  uint32_t overflow;          /* particles without destination room */
  uint32_t rebin_blocks;      /* blocks of the rebin's large-cell sort */
  uint32_t tiles;             /* tiles of the cell table */
  uint32_t particles;         /* particles in the frame, all worlds */
  uint32_t cells;             /* grid cells, all worlds */
  uint32_t huge_cells;        /* cells of more than 2048 particles the rebin
                                 sorted in global memory, since create */
  uint32_t reserved[8];
} WrachStats;

/* --- Viewport streaming ---------------------------------------------------
 * Each world keeps a device-resident particle store, the counterpart of the
 * reference's ParticleStore (runners/bevy/src/particle_store.rs:13-27):
 * every particle added to the world, inside the viewport or not.  The frame
 * is packed from the store's particles inside the viewport, as
 * create_packed_data does (spatial_bin.rs:103-149); the others stay in the
 * store, unsimulated.  Adding particles re-packs the world's frame from the
 * store, as the reference does. */

/* Writes the world's frame back into its store (the reference's TODO
 * update_from_gpu, particle_store.rs:71-85): the store becomes its particles
 * outside the viewport (store order) followed by the frame's particles (frame
 * order).  Blocks.  No counterpart in the reference. */
int wrach_write_back(WrachContext *ctx, uint32_t world);
/* Moves the world's viewport to the same-size rectangle anchored at
 * (anchor_x, anchor_y): writes the frame back, then packs the frame from the
 * store under the new viewport (its walls move with it).  The grid size must
 * stay the same (always so for a move by whole cells, or for a viewport whose
 * sides are multiples of the cell size); otherwise
 * WRACH_ERR_INVALID_ARGUMENT.  Blocks.  No counterpart in the reference. */
int wrach_set_viewport(WrachContext *ctx, uint32_t world, float anchor_x,
                       float anchor_y);
/* Number of particles in the world's store. */
int wrach_store_size(WrachContext *ctx, uint32_t world, uint32_t *count);
/* Copies the world's store (positions, velocities as float pairs; either may
 * be NULL) to host buffers of at least `capacity` >= store size entries.
 * Blocks. */
int wrach_read_store(WrachContext *ctx, uint32_t world, float *positions,
                     float *velocities, uint32_t capacity);

/* Reads the counters; blocks. */
int wrach_stats(WrachContext *ctx, WrachStats *out);

/* Self-test of the device's bounded wait, the one every device-side wait of
 * the library uses (grid barriers): a one-thread kernel waits on a device
 * word that nothing sets for limit_us microseconds (at most 1,000,000),
 * then reports *timed_out = 1 and how long it waited.  The context stays
 * usable; its sticky flags are not touched.  Blocks.  No counterpart in the
 * reference. */
int wrach_selftest_wait(WrachContext *ctx, uint32_t limit_us,
                        uint32_t *timed_out, uint32_t *waited_us);

/* The last error message of the context ("" if none). */
const char *wrach_last_error(WrachContext *ctx);

/* --- The learned solver surrogate (no counterpart in the reference) -------
 * A per-particle MLP (64 -> 64 -> 64 -> 2, GELU, BF16 weights on the tensor
 * cores, FP32 accumulation) reads the relative positions and velocities of
 * each particle's 12 nearest neighbours in its 3x3 cells (the candidates of
 * its Jacobi iterations) plus its own velocity and predicts the
 * position correction of the first iterations-1 Jacobi iterations of the
 * extended solve.  A surrogate frame applies that correction, runs the last
 * plain iteration (with integration, walls and clamp) and falls back to the
 * plain solve of the same frame when its gate fails.  The gate is decided on
 * the device (no host synchronisation per frame) from metrics the last
 * iteration computes on its input: the mean over taking-part particles of
 * the deepest overlap max(0, min_distance - distance) with a neighbour, and
 * the kinetic energy of the output.  A frame falls back when that mean
 * exceeds the same measure of the latest plain frame by more than
 * max_penetration (px), or when its kinetic energy deviates from the plain
 * frame's by more than max_energy_drift (relative).  Every 32nd frame, the
 * first included, is a plain calibration frame that refreshes the
 * reference.  Extended mode with iterations >= 2 only. */
typedef struct WrachSurrogateStats {
  uint32_t frames;         /* frames run, calibration frames included */
  uint32_t fallbacks;      /* surrogate frames replaced by the plain solve */
  float mean_penetration;  /* mean over frames of the mean deepest overlap
                              before the last iteration (px) */
  float max_penetration;   /* deepest such overlap in an accepted frame (px) */
  float max_energy_drift;  /* largest relative kinetic-energy deviation */
  uint32_t calibrations;   /* plain calibration frames */
  float reference_penetration; /* the latest plain frame's mean overlap */
  uint32_t reserved[9];
} WrachSurrogateStats;

/* Parameters: w1 [64][64], b1 [64], w2 [64][64], b2 [64], w3 [64][8],
 * b3 [8] (FP32, row = input, column = output; outputs 2..7 are padding). */
uint32_t wrach_surrogate_param_count(void);
/* Allocates the network (seeded Glorot-uniform init) and room for
 * max_samples training rows; clears collected samples. */
int wrach_surrogate_init(WrachContext *ctx, uint32_t seed,
                         uint32_t max_samples);
int wrach_surrogate_get_params(WrachContext *ctx, float *params,
                               uint32_t count);
int wrach_surrogate_set_params(WrachContext *ctx, const float *params,
                               uint32_t count);
/* Features of the current frame (BF16 rows of 64) into a device buffer of
 * at least particles_in_frame rows. */
int wrach_surrogate_features(WrachContext *ctx, uint16_t *d_x, uint32_t rows);
/* Network outputs (n float pairs) of n device feature rows, on the tcgen05
 * tensor cores (operands in shared memory, accumulators in tensor memory).
 * Asynchronous; a bounded device wait that gives up raises
 * WRACH_FLAG_TIMEOUT (wrach_flags). */
int wrach_surrogate_forward(WrachContext *ctx, const uint16_t *d_x,
                            uint32_t n, float *d_y);
/* The same on the warp-level mma.sync tensor-core instructions (the kernel
 * the fused correction of surrogate frames and the training run on). */
int wrach_surrogate_forward_mma(WrachContext *ctx, const uint16_t *d_x,
                                uint32_t n, float *d_y);
/* Gradients (host, param_count floats) and loss of 0.5 * mean over the n
 * rows of the squared error against d_t (n float pairs). */
int wrach_surrogate_gradients(WrachContext *ctx, const uint16_t *d_x,
                              const float *d_t, uint32_t n, float *grad,
                              float *loss);
/* Appends features and plain-solver targets of the current frame's
 * taking-part particles to the training set (the frame does not advance):
 * every stride-th of them (0 = 1), from an offset that turns with each call;
 * *total = rows collected.  Blocks. */
int wrach_surrogate_collect(WrachContext *ctx, uint32_t stride, uint32_t *total);
/* `steps` Adam steps on batches of `batch` collected rows; *loss = the last
 * batch's loss. */
int wrach_surrogate_train(WrachContext *ctx, uint32_t steps, uint32_t batch,
                          float lr, float *loss);
/* For the current frame (which does not advance): the mean squared error,
 * over particles that take part in the solve, of the network's correction
 * against the plain solver's first-iterations correction, and the same for
 * a zero correction (the frame without the network). */
int wrach_surrogate_evaluate(WrachContext *ctx, float *mse_network,
                             float *mse_zero);
/* Metrics of the current (binned) frame: over the particles that take part
 * in the solve, the mean and the largest deepest overlap with a neighbour of
 * the 3x3 cells (min_distance - distance, if positive), and the total
 * kinetic energy.  Blocks.  No counterpart in the reference. */
int wrach_frame_metrics(WrachContext *ctx, float *mean_penetration,
                        float *max_penetration, float *kinetic_energy);
/* The network's correction of the current binned frame, computed by the
 * fused kernel of surrogate frames (features, network and correction in one
 * pass), into d_corr (device, (n, 2) FP32; zero for particles that do not
 * take part).  Asynchronous on the context's stream. */
int wrach_surrogate_correction(WrachContext *ctx, float *d_corr);
/* nsteps frames with the surrogate and its fallback gate; blocks once, at
 * the end. */
int wrach_surrogate_step(WrachContext *ctx, uint32_t nsteps,
                         float max_penetration, float max_energy_drift,
                         WrachSurrogateStats *stats);

/* Runs one frame eagerly with a CUDA event between its kernel launches and
 * writes each launch's duration in milliseconds to ms[0 .. *count - 1]
 * (launch order: the solve launches, then the rebin).  The launches run one
 * at a time on the context's stream, including the large cells' sort, which
 * wrach_step runs beside the small cells' pass.  Same results as
 * wrach_step.  Blocks.  No counterpart in the reference (which has no GPU
 * timers). */
int wrach_profile_frame(WrachContext *ctx, float *ms, uint32_t cap,
                        uint32_t *count);

/* Number of kernel launches issued by this context since create. */
uint64_t wrach_kernel_launches(WrachContext *ctx);

/* The CUDA stream the context runs on (a cudaStream_t). */
void *wrach_stream(WrachContext *ctx);

#ifdef __cplusplus
}
#endif

#endif
