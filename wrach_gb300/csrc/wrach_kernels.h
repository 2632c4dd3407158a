// Host-side declarations of the kernel launchers (internal to the library).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "wrach_internal.cuh"

namespace wrach {

struct SolveArgs {
  const WorldDev* worlds;
  int nworlds;
  PhysDev ph;
  uint32_t ncells;              // cells over all worlds
  uint32_t n;                   // particles over all worlds
  const uint32_t* cell_start;   // ncells + 1
  const uint32_t* cell_of;      // n, cell of each binned particle
  const float2* pos;            // binned state
  const float2* vel;
  float2* pos_out;              // solve output, same order
  float2* vel_out;
  uint32_t* keys;               // next cell of each output particle
  Ctrl* ctrl;
  uint32_t block;               // threads per block of the solve kernels (<= 512)
  uint32_t per_thread;          // extended solve: particles per thread in turn (0 = 1)
  const uint32_t* run_if;       // extended solve: skip the launch when *run_if == 0 (optional)
  float* part;                  // final extended pass: per-block metrics, 8 floats a block (optional)
  CountDev count;               // final extended pass: take the rebin's tickets (count.ticket set)
  // the frame's taking-part particles, compacted (extended physics)
  const uint32_t* ct;           // ncells + 1: capped table
  const uint32_t* tp_cell;      // cell of each compacted particle
  const float2* tp_pos;         // compacted positions of the binned state
  const float2* tp_vel;         // compacted velocities of the binned state
  int sms;                      // SMs of the device
  // extended iterations (optional): each compacted taking-part particle's
  // three neighbour rows, as 4 planes of rows_stride u32 (the rows' compacted
  // starts, then their lengths packed one byte each); rows_mode 0 computes
  // the rows from the capped table, 1 also writes them, 2 reads them
  uint32_t* rows;
  uint32_t rows_stride;
  int rows_mode;
};

cudaError_t launch_solve_reference(const SolveArgs& a, cudaStream_t st);
// One extended-mode iteration but the last, over the compacted taking-part
// particles: qin and qout are compacted (the first iteration reads
// a.tp_pos).
cudaError_t launch_jacobi_iteration(const SolveArgs& a, const float2* qin, float2* qout,
                                    cudaStream_t st);
// The last iteration over every frame particle, from the compacted iterate
// qtp (a.tp_pos when there is one iteration), into a.pos_out / a.vel_out /
// a.keys (and the tickets and metrics when a.count / a.part are set);
// do_push == 0 integrates only (no iterations).
cudaError_t launch_jacobi_final(const SolveArgs& a, const float2* qtp, int do_push,
                                cudaStream_t st);

// Rebin: stable sort of `n` source particles by key into cell order, writing
// a fresh cell-start table.  Persistent cooperative kernel.
struct RebinArgs {
  const WorldDev* worlds;
  int nworlds;
  uint32_t ncells;
  uint32_t n;                   // source particles
  uint32_t dst_capacity;        // room in pos_dst/vel_dst/cell_dst
  const uint32_t* keys;         // n source keys, ncells = leave out
  const float2* pos_src;
  const float2* vel_src;
  uint32_t* cs_new;             // ncells + 1
  float2* pos_dst;
  float2* vel_dst;
  uint32_t* cell_dst;
  uint32_t* tile_sums;          // one word per tile of kTileCells cells
  uint32_t* kA;                 // radix sort ping-pong buffers, n each
  uint32_t* kB;
  uint32_t* iA;
  uint32_t* iB;
  uint32_t* hist;               // 2^digit_bits * (grid + 1)
  uint32_t key_bits;
  uint32_t digit_bits;          // rebin_digit_bits(key_bits)
  int force_general;            // set for uploads (not counted as frames)
  uint32_t* counts;             // ncells + 1 zeros on entry and on exit
  Ctrl* ctrl;
  // the counting sort (count_sort.cu); unused by the radix sort
  uint32_t* ticket;             // n: slot of each particle inside its cell (arrival order)
  uint32_t* idx_tmp;            // n: source index per slot, arrival order
  uint32_t* cell_tmp;           // n: cell per slot
  uint32_t* idx_alt;            // n: scratch of the in-memory sort of very large cells
  uint32_t* big_list;           // big_cap: cells of more than kSmallCell particles
  uint32_t big_cap;
  // the taking-part particles, compacted (extended physics; tp_cap == 0: none)
  uint32_t tp_cap;              // cell capacity: the first tp_cap of a cell take part
  uint32_t* tile_sums_cap;      // per scan tile, its taking-part particles (zero between rebins)
  uint32_t* ct_new;             // ncells + 1: capped table (compacted start of each cell)
  float2* tp_pos;               // compacted positions
  float2* tp_vel;               // compacted velocities
  uint32_t* tp_cell;            // compacted cells
  uint32_t tiles_prefixed;      // scan step: tile sums already turned into prefixes (set by it)
};

constexpr uint32_t kRebinThreads = 256;
constexpr uint32_t kCellsPerThread = 4;
constexpr uint32_t kTileCells = kRebinThreads * kCellsPerThread;

// Radix digits of at most kMaxDigitBits bits, as few passes as that allows
// (8-bit digits measured faster than 11-bit ones on the 1M-particle frame:
// the per-digit scans and offsets grow with the radix).
constexpr uint32_t kMaxDigitBits = 8;
uint32_t rebin_digit_bits(uint32_t key_bits);
size_t rebin_dynamic_smem(uint32_t digit_bits);
// Blocks the cooperative rebin kernel launches with on `device`.
int rebin_grid_size(int device, uint32_t digit_bits);
cudaError_t launch_rebin(const RebinArgs& a, int grid, cudaStream_t st);

// The same rebin as a stable counting sort over the cells (count_sort.cu),
// five plain launches: cells of up to kSmallCell particles are ranked per
// slot, cells of up to kBigCell in shared memory, larger ones in global
// memory by one block each.
constexpr uint32_t kCountScanShift = 11;
constexpr uint32_t kCountScanTile = 1u << kCountScanShift;  // cells per scan tile (tile_sums entry)
constexpr uint32_t kSmallCell = 64;
constexpr uint32_t kBigCell = 2048;
// big_blocks: the grid of the large-cell step (its blocks loop over the
// listed cells); kBigBlocksPerSm per SM unless a config sets it.
constexpr uint32_t kBigBlocksPerSm = 8;
cudaError_t launch_count_sort(const RebinArgs& a, uint32_t big_blocks, cudaStream_t st);
// The same, one step at a time (steps 0 .. kCountSortSteps - 1: count, scan,
// scatter, place, large cells); *launched is false for a step that has
// nothing to do.  Step 0 may be left out when the tickets were taken by the
// last Jacobi pass (SolveArgs::count).
constexpr int kCountSortSteps = 5;
cudaError_t launch_count_sort_step(const RebinArgs& a, int step, uint32_t big_blocks,
                                   cudaStream_t st, bool* launched);
// Steps of one rebin (count, scan, scatter, place, large cells; the scan
// alone when there are no particles) and its kernel launches (a large grid's
// scan step is two launches).
uint32_t count_sort_steps(uint32_t n);
uint32_t count_sort_launches(uint32_t n, uint32_t ncells);

// Keys for an upload re-pack: the first n_keep sources are particles of the
// current frame (their cell, or `ncells` if they belong to world `target`),
// the next n_new are store particles of world `target` binned as
// SpatialBin::get_cell_coord does (ncells if outside the grid).
cudaError_t launch_upload_keys(const WorldDev* worlds, int nworlds,
                               uint32_t ncells, uint32_t target,
                               uint32_t n_keep, const uint32_t* cell_of,
                               uint32_t n_new, const float2* new_pos,
                               uint32_t* keys, cudaStream_t st);

// One thread waits (bounded) while *word == value: out[0] = 1 if the wait
// gave up, out[1] = microseconds waited.  The wait every device-side wait
// of the library uses (wait_while_equal).
cudaError_t launch_wait_probe(const uint32_t* word, uint32_t value, uint64_t limit_ns,
                              uint32_t* out, cudaStream_t st);

// World-local cell keys (cell_of - cell_off) of n frame particles.
cudaError_t launch_local_keys(const uint32_t* cell_of, uint32_t n, uint32_t cell_off,
                              uint32_t* out, cudaStream_t st);

// Reference-layout table of one world (cells + 2 entries) from the global
// cell-start table.
cudaError_t launch_world_table(const uint32_t* cell_start, uint32_t cell_off,
                               uint32_t cells, uint32_t* out, cudaStream_t st);

// The surrogate network (surrogate.cu): FP32 master parameters in the order
// w1 [64 in][64 out], b1 [64], w2 [64][64], b2 [64], w3 [64][8], b3 [8]
// (outputs 2..7 of the last layer are padding), and BF16 copies of the
// weights in two layouts.
constexpr uint32_t kMlpIn = 64, kMlpHidden = 64, kMlpOutPad = 8;
constexpr uint32_t kMlpParams =
    kMlpIn * kMlpHidden + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden +
    kMlpHidden * kMlpOutPad + kMlpOutPad;
constexpr uint32_t kKnn = 12;

struct MlpDev {
  float* params;           // kMlpParams
  float* b1;               // into params
  float* b2;
  float* b3;
  uint16_t* w1;            // BF16 [in][out]
  uint16_t* w1t;           // BF16 [out][in]
  uint16_t* w2;
  uint16_t* w2t;
  uint16_t* w3;            // BF16 [in][8]
  uint16_t* w3t;           // BF16 [8][in]
};

// Device-side state of the surrogate's fallback gate (k_gate).
struct GateState {
  float tol;          // allowed excess of the mean overlap over the reference (px)
  float max_drift;    // allowed relative kinetic-energy deviation
  float pen_ref;      // mean overlap before the last iteration, latest plain frame
  uint32_t fallback;  // the current frame falls back to the plain solve
  uint32_t frames, fallbacks, calibrations;
  float pen_sum, pen_max, drift_max;
  uint32_t pad[6];
};

cudaError_t launch_knn_features(const SolveArgs& a, uint16_t* x, cudaStream_t st);
// Training rows of the binned frame: the features of the taking-part
// particles t = phase + k * stride into rows k of x (at most `rows`) and
// their targets q_t - p_t from the compacted iterate q.
cudaError_t launch_samples(const SolveArgs& a, const float2* q, uint32_t stride, uint32_t phase,
                           uint32_t rows, uint16_t* x, float2* target, cudaStream_t st);
// Fused surrogate correction of the binned frame: the compacted iterate
// q_t = p + network(features) of each taking-part particle; `corr` optional
// (per frame particle).
cudaError_t launch_surrogate_correct(const MlpDev& m, const SolveArgs& a, float2* q, float2* corr,
                                     int blocks, cudaStream_t st);
// One-time set-up of the fused correction kernel on `device` (its shared
// memory size); returns its grid (one wave of co-resident blocks), 0 if the
// set-up failed.
int surrogate_correct_blocks(int device);
cudaError_t launch_gate(const float* part, uint32_t nparts, GateState* gs, int mode,
                        cudaStream_t st);
// Number of blocks (and so of gate partials) of an extended solve launch:
// one thread per particle, or, for a launch with a run_if flag, a few
// blocks per SM striding over the frame.
uint32_t solve_blocks(const SolveArgs& a);
cudaError_t launch_mlp_forward(const MlpDev& m, const uint16_t* x, uint32_t n, float2* y,
                               int blocks, cudaStream_t st);
// The same forward pass on the tcgen05 tensor cores (mlp_tc.cu): operands in
// shared memory, accumulators in TMEM; a bounded wait that gives up raises
// kFlagTimeout in *flags.
cudaError_t launch_mlp_forward_tc(const MlpDev& m, const uint16_t* x, uint32_t n, float2* y,
                                  uint32_t* flags, int sms, cudaStream_t st);
cudaError_t launch_mlp_backward(const MlpDev& m, const uint16_t* x, const float2* target,
                                uint32_t n, float inv_rows, float* grad, float* loss,
                                int blocks, cudaStream_t st);
cudaError_t launch_adam(const MlpDev& m, const float* grad, float* mom1, float* mom2, float lr,
                        uint32_t step, cudaStream_t st);
// target[i] = q_t - p_i for the first n frame particles, q compacted (zero
// for a particle that takes no part).
cudaError_t launch_target(const SolveArgs& a, uint32_t n, const float2* q, float2* target,
                          cudaStream_t st);
cudaError_t launch_errors(const SolveArgs& a, const float2* corr, const float2* target, float* out,
                          cudaStream_t st);
// Report-only frame metrics: per-block partials into `part` (8 floats per
// 256 particles), their sums into out[0..4].
cudaError_t launch_penetration(const SolveArgs& a, const float2* pos, const float2* vel,
                               float* part, float* out, cudaStream_t st);

// Viewport streaming (viewport.cu): the n items whose key is >= ncells
// (outside the viewport), in order, into dst; *count receives how many.
// `tile_sums` holds keep_outside_tiles(n) words of scratch.
uint32_t keep_outside_tiles(uint32_t n);
cudaError_t launch_keep_outside(const uint32_t* keys, uint32_t ncells, uint32_t n,
                                const float2* pos, const float2* vel, float2* dst_pos,
                                float2* dst_vel, uint32_t* tile_sums, uint32_t* count,
                                cudaStream_t st);

// Headless point rasteriser (render.cu): `cover` holds width_px * height_px
// u32 scratch, `image` the 8-bit result.
cudaError_t launch_render(const float2* pos, uint32_t n, float world_w, float world_h,
                          uint32_t width_px, uint32_t height_px, uint32_t* cover,
                          uint8_t* image, cudaStream_t st);

}  // namespace wrach
