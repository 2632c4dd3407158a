// The C ABI (include/wrach.h): context lifetime, uploads, the frame loop,
// viewport streaming and readback.  Host orchestration of the kernels in
// solve.cu, count_sort.cu, rebin.cu and viewport.cu; the learned surrogate's
// entry points are in surrogate_host.cu.
//
// Device layout of a context (all worlds concatenated; world w owns the
// global cells [cell_off_w, cell_off_w + gx_w * gy_w) and, in the frame, the
// particles [cell_start[cell_off_w], cell_start[cell_off_w + cells_w])):
//   pos, vel          binned state, float2 x capacity        (cell order)
//   pos_o, vel_o      solve output, float2 x capacity        (same order)
//   q1, q2            extended-mode Jacobi iterates
//   rows              the iterations' neighbour-row ranges per compacted particle (4 planes)
//   cell_of[2]        cell of each binned particle (u32)
//   cs[2]             cell-start table, cells + 1 u32 (ping-pong per frame)
//   ct[2], tp_pos[2], tp_vel[2], tp_cell[2]
//                     extended physics: the capped table (start of each
//                     cell's taking-part particles among them all) and those
//                     particles' positions, velocities and cells, compacted in
//                     cell order
//   keys              next cell of each solve output (u32)
//   kA kB iA iB       rebin scratch (tickets, slot cells, slot sources, sort ping-pong)
//   tile_sums         rebin: particles per tile of 2048 cells (zero between frames)
//   ctrl              counters and sticky flags
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "context_internal.h"

using wrach::Ctrl;
using wrach::PhysDev;
using wrach::WorldDev;
using namespace wrach::host;

namespace {

// Rust's saturating `f32 as i32` (NaN -> 0).
int32_t sat_i32(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT32_MAX;
  if (f <= -2147483648.0f) return INT32_MIN;
  return (int32_t)f;
}

// SpatialBin::get_cell_coord (runners/bevy/src/spatial_bin.rs:48-64).
int32_t cell_coord(float x, uint32_t cs) {
  volatile float d = (float)cs;  // keep the binary32 division
  float q = std::trunc(x / d);
  if (std::fmod(x, (float)d) < 0.0f) q = q - 1.0f;
  return sat_i32(q);
}

__global__ void k_gather_u32(const uint32_t* __restrict__ src,
                             const uint32_t* __restrict__ idx, uint32_t n,
                             uint32_t* __restrict__ out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = src[idx[i]];
}

// The smallest binary32 s with sqrt_rn(s) > min_d.  Correctly rounded
// square roots are monotonic, so for every s: s >= skip_threshold(min_d)
// exactly when sqrtf(s) > min_d.
float skip_threshold(float min_d) {
  volatile float s = min_d * min_d;
  while (s > 0.0f && std::sqrt((float)std::nextafter((float)s, 0.0f)) > min_d)
    s = std::nextafter((float)s, 0.0f);
  while (!(std::sqrt((float)s) > min_d)) s = std::nextafter((float)s, INFINITY);
  return s;
}

uint32_t bits_for(uint32_t v) {
  uint32_t b = 0;
  while (b < 32 && (v >> b) != 0) ++b;
  return b;
}

}  // namespace


namespace {

void drop_graphs(WrachContext* ctx) {
  for (auto& g : ctx->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  for (auto& row : ctx->sur.graph)
    for (auto& g : row)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
}

void release(WrachContext* ctx) {
  drop_graphs(ctx);
  {
    void* sp[] = {ctx->sur.params, ctx->sur.grad, ctx->sur.mom1, ctx->sur.mom2, ctx->sur.loss,
                  ctx->sur.metrics, ctx->sur.bf16, ctx->sur.x, ctx->sur.corr, ctx->sur.tx,
                  ctx->sur.tt, ctx->sur.part, ctx->sur.gate};
    for (void* p : sp) dfree(p);
  }
  void* ptrs[] = {ctx->worlds_d, ctx->pos, ctx->vel, ctx->pos_o, ctx->vel_o,
                  ctx->q1, ctx->q2, ctx->rows, ctx->cell_of[0], ctx->cell_of[1],
                  ctx->cs[0], ctx->cs[1], ctx->keys, ctx->kA, ctx->kB,
                  ctx->iA, ctx->iB, ctx->tile_sums, ctx->ctrl, ctx->big_list,
                  ctx->ct[0], ctx->ct[1], ctx->tp_pos[0], ctx->tp_pos[1], ctx->tp_cell[0],
                  ctx->tp_cell[1], ctx->tile_sums_cap, ctx->tp_vel[0], ctx->tp_vel[1],
                  ctx->stage_pos, ctx->stage_vel, ctx->table_tmp, ctx->counts, ctx->render_cover, ctx->render_image,
                  ctx->gather_idx, ctx->gather_out, ctx->compact_sums};
  for (void* p : ptrs) dfree(p);
  for (auto& s : ctx->stores) {
    dfree(s.pos);
    dfree(s.vel);
  }
  if (ctx->gather_h) cudaFreeHost(ctx->gather_h);
  if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
  if (ctx->join_ev) cudaEventDestroy(ctx->join_ev);
  if (ctx->counts_ev) cudaEventDestroy(ctx->counts_ev);
  if (ctx->aux) cudaStreamDestroy(ctx->aux);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
}

// The buffers below may still be in use by work queued on the context's
// streams (a frame, or the last steps of an upload), so a reallocation waits
// for that work before freeing them.
int ensure_sort_capacity(WrachContext* ctx, size_t need) {
  if (need <= ctx->sort_cap) return WRACH_OK;
  size_t cap = std::max(need, ctx->sort_cap * 2);
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaStreamSynchronize(ctx->aux));
  uint32_t** bufs[] = {&ctx->keys, &ctx->kA, &ctx->kB, &ctx->iA, &ctx->iB};
  for (auto b : bufs) {
    dfree(*b);
    *b = nullptr;
  }
  for (auto b : bufs) CK(dalloc(b, cap));
  dfree(ctx->big_list);
  ctx->big_list = nullptr;
  // at most cap / (kSmallCell + 1) cells can be larger than kSmallCell
  ctx->big_cap = (uint32_t)(cap / (wrach::kSmallCell + 1) + 2);
  CK(dalloc(&ctx->big_list, ctx->big_cap));
  ctx->sort_cap = cap;
  drop_graphs(ctx);
  return WRACH_OK;
}

int ensure_stage(WrachContext* ctx, size_t need) {
  if (need <= ctx->stage_cap) return WRACH_OK;
  size_t cap = std::max(need, ctx->stage_cap * 2);
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaStreamSynchronize(ctx->aux));
  dfree(ctx->stage_pos);
  dfree(ctx->stage_vel);
  ctx->stage_pos = ctx->stage_vel = nullptr;
  CK(dalloc(&ctx->stage_pos, cap));
  CK(dalloc(&ctx->stage_vel, cap));
  ctx->stage_cap = cap;
  return WRACH_OK;
}

int ensure_store(WrachContext* ctx, Store& s, size_t need) {
  if (need <= s.cap) return WRACH_OK;
  size_t cap = std::max<size_t>(need, (size_t)s.cap * 2);
  if (cap > 0xFFFFFFF0ull) return fail(ctx, WRACH_ERR_CAPACITY, "store too large");
  float2 *np = nullptr, *nv = nullptr;
  CK(dalloc(&np, cap));
  CK(dalloc(&nv, cap));
  if (s.n) {
    CK(cudaMemcpyAsync(np, s.pos, s.n * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(nv, s.vel, s.n * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaStreamSynchronize(ctx->aux));
  dfree(s.pos);
  dfree(s.vel);
  s.pos = np;
  s.vel = nv;
  s.cap = (uint32_t)cap;
  return WRACH_OK;
}

}  // namespace

namespace wrach {
namespace host {

int fail(WrachContext* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

void dfree(void* p) {
  if (p) cudaFree(p);
}

wrach::SolveArgs solve_args(WrachContext* ctx) {
  wrach::SolveArgs a{};
  a.worlds = ctx->worlds_d;
  a.nworlds = (int)ctx->nworlds;
  a.ph = ctx->ph;
  a.ncells = ctx->ncells;
  a.n = ctx->n;
  a.cell_start = ctx->cs[ctx->cur];
  a.cell_of = ctx->cell_of[ctx->cur];
  a.pos = ctx->pos;
  a.vel = ctx->vel;
  a.pos_out = ctx->pos_o;
  a.vel_out = ctx->vel_o;
  a.keys = ctx->keys;
  a.ctrl = ctx->ctrl;
  a.block = ctx->cfg.solve_block;
  a.per_thread = ctx->cfg.solve_per_thread;
  a.ct = ctx->ct[ctx->cur];
  a.tp_cell = ctx->tp_cell[ctx->cur];
  a.tp_pos = ctx->tp_pos[ctx->cur];
  a.tp_vel = ctx->tp_vel[ctx->cur];
  a.sms = ctx->sms;
  a.rows = ctx->rows;
  a.rows_stride = ctx->total_cap;
  return a;
}

wrach::CountDev ticket_args(WrachContext* ctx) {
  return wrach::CountDev{ctx->counts, ctx->tile_sums, ctx->kA, ctx->ncells, wrach::kCountScanShift,
                         ctx->ph.cap, ctx->tile_sums_cap};
}

wrach::RebinArgs rebin_args(WrachContext* ctx) {
  wrach::RebinArgs r{};
  r.worlds = ctx->worlds_d;
  r.nworlds = (int)ctx->nworlds;
  r.ncells = ctx->ncells;
  r.tile_sums = ctx->tile_sums;
  r.kA = ctx->kA;
  r.kB = ctx->kB;
  r.iA = ctx->iA;
  r.iB = ctx->iB;
  r.keys = ctx->keys;
  r.counts = ctx->counts;
  r.ctrl = ctx->ctrl;
  r.ticket = ctx->kA;
  r.idx_tmp = ctx->iA;
  r.cell_tmp = ctx->kB;
  r.idx_alt = ctx->iB;
  r.big_list = ctx->big_list;
  r.big_cap = ctx->big_cap;
  // every rebin writes the next table parity; extended physics also the
  // compacted taking-part particles
  if (ctx->ph.mode == WRACH_MODE_EXTENDED) {
    r.tp_cap = ctx->ph.cap;
    r.tile_sums_cap = ctx->tile_sums_cap;
    r.ct_new = ctx->ct[ctx->cur ^ 1];
    r.tp_pos = ctx->tp_pos[ctx->cur ^ 1];
    r.tp_vel = ctx->tp_vel[ctx->cur ^ 1];
    r.tp_cell = ctx->tp_cell[ctx->cur ^ 1];
  }
  return r;
}

}  // namespace host
}  // namespace wrach

namespace {

void mark(WrachContext* ctx) {
  if (ctx->event_hook) cudaEventRecord(ctx->event_hook[ctx->event_count++], ctx->stream);
}

// One frame: solve (1 or `iterations` launches) then the rebin launch.
int enqueue_frame(WrachContext* ctx) {
  wrach::SolveArgs a = solve_args(ctx);
  cudaStream_t st = ctx->stream;
  mark(ctx);
  if (ctx->ph.mode == WRACH_MODE_REFERENCE) {
    CK(wrach::launch_solve_reference(a, st));
    mark(ctx);
    ctx->launches += 1;
  } else {
    // the last pass takes the rebin's tickets (it computes the keys)
    wrach::SolveArgs fin = a;
    fin.count = ticket_args(ctx);
    const uint32_t K = ctx->ph.iterations;
    const float2* q = nullptr;
    CK(enqueue_iterations(ctx, a, K > 0 ? K - 1 : 0, st, &q, [&]() { mark(ctx); }));
    CK(wrach::launch_jacobi_final(fin, q, K > 0 ? 1 : 0, st));
    mark(ctx);
    ctx->launches += ctx->n ? std::max<uint32_t>(K, 1) : 0u;
  }
  const bool tickets_taken = ctx->ph.mode != WRACH_MODE_REFERENCE;
  wrach::RebinArgs r = rebin_args(ctx);
  r.n = ctx->n;
  r.dst_capacity = ctx->total_cap;
  r.pos_src = ctx->pos_o;
  r.vel_src = ctx->vel_o;
  r.cs_new = ctx->cs[ctx->cur ^ 1];
  r.pos_dst = ctx->pos;
  r.vel_dst = ctx->vel;
  r.cell_dst = ctx->cell_of[ctx->cur ^ 1];
  r.force_general = 0;
  // the large cells' sort (the last step) writes other slots than the small
  // cells' pass before it, so outside per-launch profiling it runs on the
  // auxiliary stream at the same time, joined back before the frame ends
  const bool fork = !ctx->event_hook && r.n;
  for (int step = tickets_taken ? 1 : 0; step < wrach::kCountSortSteps; ++step) {
    bool launched;
    if (fork && step == wrach::kCountSortSteps - 2) {
      CK(cudaEventRecord(ctx->fork_ev, st));
      CK(cudaStreamWaitEvent(ctx->aux, ctx->fork_ev, 0));
      CK(wrach::launch_count_sort_step(r, step + 1, ctx->big_blocks, ctx->aux, &launched));
      CK(cudaEventRecord(ctx->join_ev, ctx->aux));
      CK(wrach::launch_count_sort_step(r, step, ctx->big_blocks, st, &launched));
      CK(cudaStreamWaitEvent(st, ctx->join_ev, 0));
      break;
    }
    CK(wrach::launch_count_sort_step(r, step, ctx->big_blocks, st, &launched));
    if (launched) mark(ctx);
  }
  ctx->launches += wrach::count_sort_launches(r.n, ctx->ncells) - (tickets_taken && r.n ? 1 : 0);
  ctx->cur ^= 1;
  return WRACH_OK;
}

// Steps wrach_profile_frame times in one frame: each solve launch, then
// each rebin launch (an empty frame's extended solve launches nothing, but
// still marks its steps).
uint32_t frame_steps(const WrachContext* ctx) {
  const uint32_t rebin = wrach::count_sort_steps(ctx->n);
  if (ctx->ph.mode == WRACH_MODE_REFERENCE) return 1 + rebin;
  return std::max<uint32_t>(ctx->ph.iterations, 1) + rebin - (ctx->n ? 1 : 0);
}

// Kernel launches of one frame.
uint32_t frame_launches(const WrachContext* ctx) {
  const uint32_t extra = wrach::count_sort_launches(ctx->n, ctx->ncells) - wrach::count_sort_steps(ctx->n);
  if (ctx->ph.mode == WRACH_MODE_EXTENDED && !ctx->n) return wrach::count_sort_launches(0, ctx->ncells);
  return frame_steps(ctx) + extra;
}

// One frame captured as a CUDA graph, instantiated once per table parity
// (the frame reads cs[parity] and writes cs[parity ^ 1]).
int build_graph(WrachContext* ctx) {
  const int parity = ctx->cur;
  const uint64_t launches = ctx->launches;
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    ctx->graph_ok = false;
    return WRACH_OK;
  }
  int rc = enqueue_frame(ctx);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  ctx->cur = parity;
  ctx->launches = launches;
  if (rc != WRACH_OK || e != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    ctx->graph_ok = false;
    ctx->err.clear();
    return WRACH_OK;
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ctx->graph_ok = false;
    return WRACH_OK;
  }
  ctx->graph[parity] = exec;
  ctx->graph_n[parity] = ctx->n;
  return WRACH_OK;
}

int world_settings_init(WorldDev& w, float width, float height, float ax,
                        float ay, uint32_t cs) {
  std::memset(&w, 0, sizeof(w));
  w.dim_x = width;
  w.dim_y = height;
  w.ax = ax;
  w.ay = ay;
  w.cs = cs;
  volatile float x1 = ax + width, y1 = ay + height;
  w.x1 = x1;
  w.y1 = y1;
  const int32_t blx = cell_coord(ax, cs), bly = cell_coord(ay, cs);
  const int32_t trx = cell_coord(x1, cs), try_ = cell_coord(y1, cs);
  if (trx < blx || try_ < bly) return 1;
  const int64_t gx = (int64_t)trx - blx + 1, gy = (int64_t)try_ - bly + 1;
  if (gx * gy > 0x7FFFFFFFll) return 1;
  w.gx = (uint32_t)gx;
  w.gy = (uint32_t)gy;
  w.blx = blx;
  w.bly = bly;
  // x / gx for every x < 2^31 as (x * m) >> (31 + l), l = ceil(log2 gx),
  // m = floor(2^(31 + l) / gx) + 1 < 2^32 (Granlund & Montgomery, 1994)
  uint32_t l = 0;
  while ((1ull << l) < w.gx) ++l;
  w.div_m = (uint32_t)((1ull << (31 + l)) / w.gx + 1);
  w.div_s = 31 + l;
  return 0;
}

int create_impl(const WrachConfig* config, uint32_t nworlds, const float* dims,
                WrachContext** out) {
  if (!config || !out || nworlds == 0) return WRACH_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  WrachContext* ctx = new (std::nothrow) WrachContext();
  if (!ctx) return WRACH_ERR_OUT_OF_MEMORY;
  ctx->cfg = *config;
  const WrachConfig& c = ctx->cfg;
  auto bad = [&](const char* m) {
    int rc = fail(ctx, WRACH_ERR_INVALID_ARGUMENT, m);
    delete ctx;
    return rc;
  };
  if (c.cell_size == 0) return bad("cell_size must be positive");
  if (c.mode != WRACH_MODE_REFERENCE && c.mode != WRACH_MODE_EXTENDED) return bad("unknown mode");
  if (c.cell_capacity == 0 || c.cell_capacity > wrach::kMaxCellCapacity)
    return bad("cell_capacity must be in 1..16");
  if (!(c.min_distance > 0.0f) || !(c.max_velocity >= 0.0f)) return bad("bad physics constants");
  if (c.iterations > 64) return bad("iterations must be at most 64");
  if (c.solve_block && (c.solve_block > 512 || c.solve_block % 32))
    return bad("solve_block must be a multiple of 32 up to 512");
  if (c.solve_per_thread > 64) return bad("solve_per_thread must be at most 64");

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    int rc = fail(ctx, WRACH_ERR_UNSUPPORTED, "no CUDA device");
    delete ctx;
    return rc;
  }
  if (c.device < 0 || c.device >= ndev) return bad("device ordinal out of range");
  ctx->device = c.device;
  DeviceGuard guard(ctx->device);
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, ctx->device) != cudaSuccess ||
      !(prop.major == 10 && prop.minor == 3)) {
    int rc = fail(ctx, WRACH_ERR_UNSUPPORTED,
                  std::string("this build targets sm_103a; device is ") + prop.name);
    delete ctx;
    return rc;
  }

  ctx->ph.mode = c.mode;
  ctx->ph.iterations = c.mode == WRACH_MODE_REFERENCE ? 1u : c.iterations;
  ctx->ph.gravity = c.mode == WRACH_MODE_REFERENCE ? 0.0f : c.gravity;
  ctx->ph.min_d = c.min_distance;
  ctx->ph.vmax = c.max_velocity;
  ctx->ph.cap = c.cell_capacity;
  ctx->ph.skip_d2 = skip_threshold(c.min_distance);

  ctx->nworlds = nworlds;
  ctx->worlds_h.resize(nworlds);
  ctx->cap_h.resize(nworlds);
  ctx->n_h.assign(nworlds, 0);
  ctx->poff_h.assign(nworlds, 0);
  ctx->stores.resize(nworlds);
  uint64_t cells = 0, cap = 0;
  for (uint32_t w = 0; w < nworlds; ++w) {
    const float wd = dims ? dims[2 * w] : c.width;
    const float ht = dims ? dims[2 * w + 1] : c.height;
    if (!(wd >= 0.0f) || !(ht >= 0.0f)) return bad("world dimensions must be non-negative");
    if (world_settings_init(ctx->worlds_h[w], wd, ht, c.anchor_x, c.anchor_y, c.cell_size))
      return bad("grid too large");
    WorldDev& wd_ = ctx->worlds_h[w];
    wd_.cell_off = (uint32_t)cells;
    const uint64_t wc = (uint64_t)wd_.gx * wd_.gy;
    cells += wc;
    ctx->max_world_cells = std::max<uint32_t>(ctx->max_world_cells, (uint32_t)wc);
    const uint32_t wcap = c.capacity ? c.capacity
                                     : wrach_max_particles_per_frame((uint32_t)wc, c.cell_size);
    ctx->cap_h[w] = wcap;
    cap += wcap;
    // keys carry a flag in bit 31, so cell indices stay below 2^31
    if (cells > 0x7FFFFFF0ull || cap > 0x7FFFFFFFull) return bad("grid or capacity too large");
  }
  ctx->ncells = (uint32_t)cells;
  ctx->total_cap = (uint32_t)cap;

  auto oom = [&](cudaError_t e) {
    int rc = fail(ctx, e == cudaErrorMemoryAllocation ? WRACH_ERR_OUT_OF_MEMORY : WRACH_ERR_CUDA,
                  std::string("allocation: ") + cudaGetErrorString(e));
    cudaGetLastError();
    release(ctx);
    delete ctx;
    return rc;
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) return oom(e);
  if ((e = cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking)) != cudaSuccess) return oom(e);
  if ((e = cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming)) != cudaSuccess) return oom(e);
  if ((e = cudaEventCreateWithFlags(&ctx->join_ev, cudaEventDisableTiming)) != cudaSuccess) return oom(e);
  if ((e = cudaEventCreateWithFlags(&ctx->counts_ev, cudaEventDisableTiming)) != cudaSuccess) return oom(e);
  const size_t tc = ctx->total_cap;
  // the worlds, then (batches) the first world of each tile of cells
  const size_t tiles_words = nworlds > 1 ? (size_t)wrach::world_tiles(ctx->ncells) + 2 : 0;
  const size_t worlds_words = (nworlds * sizeof(WorldDev) + 3) / 4 + tiles_words;
  {
    uint32_t* raw = nullptr;
    if ((e = dalloc(&raw, worlds_words)) != cudaSuccess) return oom(e);
    ctx->worlds_d = reinterpret_cast<WorldDev*>(raw);
  }
  if ((e = dalloc(&ctx->pos, tc)) != cudaSuccess) return oom(e);
  if ((e = dalloc(&ctx->vel, tc)) != cudaSuccess) return oom(e);
  if ((e = dalloc(&ctx->pos_o, tc)) != cudaSuccess) return oom(e);
  if ((e = dalloc(&ctx->vel_o, tc)) != cudaSuccess) return oom(e);
  if (c.mode == WRACH_MODE_EXTENDED && ctx->ph.iterations >= 2) {
    if ((e = dalloc(&ctx->q1, tc)) != cudaSuccess) return oom(e);
    if ((e = dalloc(&ctx->q2, tc)) != cudaSuccess) return oom(e);
  }
  if (c.mode == WRACH_MODE_EXTENDED && ctx->ph.iterations >= 3)
    if ((e = dalloc(&ctx->rows, 4 * tc)) != cudaSuccess) return oom(e);
  if (c.mode == WRACH_MODE_EXTENDED) {
    for (int i = 0; i < 2; ++i) {
      if ((e = dalloc(&ctx->ct[i], (size_t)ctx->ncells + 1)) != cudaSuccess) return oom(e);
      if ((e = cudaMemset(ctx->ct[i], 0, ((size_t)ctx->ncells + 1) * 4)) != cudaSuccess) return oom(e);
      if ((e = dalloc(&ctx->tp_pos[i], tc)) != cudaSuccess) return oom(e);
      if ((e = dalloc(&ctx->tp_vel[i], tc)) != cudaSuccess) return oom(e);
      if ((e = dalloc(&ctx->tp_cell[i], tc)) != cudaSuccess) return oom(e);
    }
  }
  for (int i = 0; i < 2; ++i) {
    if ((e = dalloc(&ctx->cell_of[i], tc)) != cudaSuccess) return oom(e);
    if ((e = dalloc(&ctx->cs[i], (size_t)ctx->ncells + 1)) != cudaSuccess) return oom(e);
    if ((e = cudaMemset(ctx->cs[i], 0, ((size_t)ctx->ncells + 1) * 4)) != cudaSuccess) return oom(e);
  }
  // one sum per tile of kTileCells cells of the table
  ctx->ntiles = (ctx->ncells + wrach::kTileCells - 1) / wrach::kTileCells;
  if ((e = dalloc(&ctx->tile_sums, ctx->ntiles)) != cudaSuccess) return oom(e);
  // the counting sort's tile sums reuse the table tile sums (kTileCells <= 2048)
  static_assert(wrach::kTileCells <= wrach::kCountScanTile, "tile sums buffer large enough");
  if ((e = cudaMemset(ctx->tile_sums, 0, (size_t)ctx->ntiles * 4)) != cudaSuccess) return oom(e);
  if (c.mode == WRACH_MODE_EXTENDED) {
    if ((e = dalloc(&ctx->tile_sums_cap, ctx->ntiles)) != cudaSuccess) return oom(e);
    if ((e = cudaMemset(ctx->tile_sums_cap, 0, (size_t)ctx->ntiles * 4)) != cudaSuccess) return oom(e);
  }
  if ((e = cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, ctx->device)) != cudaSuccess)
    return oom(e);
  ctx->big_blocks = c.rebin_blocks ? c.rebin_blocks : wrach::kBigBlocksPerSm * (uint32_t)ctx->sms;
  if ((e = dalloc(&ctx->ctrl, 1)) != cudaSuccess) return oom(e);
  if ((e = cudaMemset(ctx->ctrl, 0, sizeof(Ctrl))) != cudaSuccess) return oom(e);
  if ((e = dalloc(&ctx->table_tmp, (size_t)ctx->max_world_cells + 2)) != cudaSuccess) return oom(e);
  if ((e = dalloc(&ctx->counts, (size_t)ctx->ncells + 1)) != cudaSuccess) return oom(e);
  if ((e = cudaMemset(ctx->counts, 0, ((size_t)ctx->ncells + 1) * 4)) != cudaSuccess) return oom(e);
  if ((e = dalloc(&ctx->gather_idx, nworlds + 1)) != cudaSuccess) return oom(e);
  if ((e = dalloc(&ctx->gather_out, nworlds + 1)) != cudaSuccess) return oom(e);
  if ((e = cudaMallocHost(reinterpret_cast<void**>(&ctx->gather_h), (nworlds + 1) * sizeof(uint32_t))) !=
      cudaSuccess)
    return oom(e);
  {
    std::vector<uint32_t> idx(nworlds + 1);
    for (uint32_t w = 0; w < nworlds; ++w) idx[w] = ctx->worlds_h[w].cell_off;
    idx[nworlds] = ctx->ncells;
    if ((e = cudaMemcpy(ctx->gather_idx, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return oom(e);
  }
  if ((e = cudaMemcpy(ctx->worlds_d, ctx->worlds_h.data(), nworlds * sizeof(WorldDev),
                      cudaMemcpyHostToDevice)) != cudaSuccess)
    return oom(e);
  if (tiles_words) {
    static_assert(sizeof(WorldDev) % 4 == 0, "the tile table follows the worlds word-aligned");
    std::vector<uint32_t> first(tiles_words);
    uint32_t wi = 0;
    for (size_t t = 0; t < tiles_words; ++t) {
      const uint64_t c = std::min<uint64_t>((uint64_t)t << wrach::kWorldTileShift, ctx->ncells - 1);
      while (wi + 1 < nworlds && ctx->worlds_h[wi + 1].cell_off <= c) ++wi;
      first[t] = wi;
    }
    first[tiles_words - 2] = first[tiles_words - 1] = nworlds - 1;
    if ((e = cudaMemcpy(reinterpret_cast<uint32_t*>(ctx->worlds_d + nworlds), first.data(),
                        tiles_words * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
      return oom(e);
  }
  if (ensure_sort_capacity(ctx, tc) != WRACH_OK) {
    int rc = WRACH_ERR_OUT_OF_MEMORY;
    release(ctx);
    delete ctx;
    return rc;
  }
  *out = ctx;
  return WRACH_OK;
}

int upload_impl(WrachContext* ctx, uint32_t world, const float* pos,
                const float* vel, uint32_t n_add, cudaMemcpyKind kind,
                bool replace) {
  if (!ctx) return WRACH_ERR_INVALID_ARGUMENT;
  if (world >= ctx->nworlds) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "world out of range");
  if (n_add && (!pos || !vel)) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "null particle arrays");
  DeviceGuard guard(ctx->device);
  Store& s = ctx->stores[world];
  const uint32_t old_n = s.n;
  if (replace) s.n = 0;
  int rc = ensure_store(ctx, s, (size_t)s.n + n_add);
  if (rc) return rc;
  // One world re-packed from a store that holds no more particles than its
  // frame: the capacity check below cannot fail, so the sort places straight
  // into the frame buffers, and the velocities are copied on the second
  // stream while the positions' keys are counted, scanned and scattered
  // (only the place steps read them).
  const bool direct = ctx->nworlds == 1 && replace && n_add <= ctx->cap_h[world];
  const bool vel_aside = direct && n_add;
  if (n_add) {
    CK(cudaMemcpyAsync(s.pos + s.n, pos, (size_t)n_add * sizeof(float2), kind, ctx->stream));
    if (vel_aside) {
      CK(cudaEventRecord(ctx->fork_ev, ctx->stream));
      CK(cudaStreamWaitEvent(ctx->aux, ctx->fork_ev, 0));
      CK(cudaMemcpyAsync(s.vel + s.n, vel, (size_t)n_add * sizeof(float2), kind, ctx->aux));
      CK(cudaEventRecord(ctx->join_ev, ctx->aux));
    } else {
      CK(cudaMemcpyAsync(s.vel + s.n, vel, (size_t)n_add * sizeof(float2), kind, ctx->stream));
    }
  }
  s.n += n_add;

  // the frame's particles of other worlds are kept; with one world they all
  // belong to the world being re-packed from its store, so none are
  const uint32_t n_keep = ctx->nworlds > 1 ? ctx->n : 0u, n_new = s.n;
  const size_t nsrc = (size_t)n_keep + n_new;
  if (nsrc > 0xFFFFFFF0ull) {
    s.n = old_n;
    return fail(ctx, WRACH_ERR_CAPACITY, "too many particles");
  }
  if ((rc = ensure_stage(ctx, nsrc))) return rc;
  if ((rc = ensure_sort_capacity(ctx, nsrc))) return rc;
  // the sort's source: [kept frame particles, store]; without kept
  // particles the store itself
  const float2* src_pos = s.pos;
  const float2* src_vel = s.vel;
  if (n_keep) {
    CK(cudaMemcpyAsync(ctx->stage_pos, ctx->pos, n_keep * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->stage_vel, ctx->vel, n_keep * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
    if (n_new) {
      CK(cudaMemcpyAsync(ctx->stage_pos + n_keep, s.pos, n_new * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
      CK(cudaMemcpyAsync(ctx->stage_vel + n_keep, s.vel, n_new * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    src_pos = ctx->stage_pos;
    src_vel = ctx->stage_vel;
  }
  CK(wrach::launch_upload_keys(ctx->worlds_d, (int)ctx->nworlds, ctx->ncells, world, n_keep,
                               ctx->cell_of[ctx->cur], n_new, s.pos, ctx->keys, ctx->stream));
  ctx->launches += nsrc ? 1 : 0;
  wrach::RebinArgs r = rebin_args(ctx);
  r.n = (uint32_t)nsrc;
  r.dst_capacity = ctx->total_cap;
  r.pos_src = src_pos;
  r.vel_src = src_vel;
  r.cs_new = ctx->cs[ctx->cur ^ 1];
  r.pos_dst = direct ? ctx->pos : ctx->pos_o;
  r.vel_dst = direct ? ctx->vel : ctx->vel_o;
  r.cell_dst = ctx->cell_of[ctx->cur ^ 1];
  r.force_general = 1;
  // per-world counts from the new table, read back as soon as the scan has
  // written it
  const uint32_t nw = ctx->nworlds;
  for (int step = 0; step < wrach::kCountSortSteps; ++step) {
    // the place steps (3, 4) are the first to read the velocities
    if (vel_aside && step == 3) CK(cudaStreamWaitEvent(ctx->stream, ctx->join_ev, 0));
    bool launched;
    CK(wrach::launch_count_sort_step(r, step, ctx->big_blocks, ctx->stream, &launched));
    if (step == 1) {
      k_gather_u32<<<(nw + 1 + 255) / 256, 256, 0, ctx->stream>>>(ctx->cs[ctx->cur ^ 1],
                                                                   ctx->gather_idx, nw + 1,
                                                                   ctx->gather_out);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(ctx->gather_h, ctx->gather_out, (nw + 1) * 4, cudaMemcpyDeviceToHost,
                         ctx->stream));
      CK(cudaEventRecord(ctx->counts_ev, ctx->stream));
    }
  }
  ctx->launches += wrach::count_sort_launches(r.n, ctx->ncells) + 1;
  if (direct) {
    // the call returns once the counts are known and both host arrays have
    // been read; the place steps are still running, ahead of whatever the
    // caller enqueues next on the context's stream
    CK(cudaEventSynchronize(ctx->counts_ev));
    if (vel_aside) CK(cudaEventSynchronize(ctx->join_ev));
  } else {
    CK(cudaStreamSynchronize(ctx->stream));
  }
  const std::vector<uint32_t> starts(ctx->gather_h, ctx->gather_h + nw + 1);
  for (uint32_t w = 0; w < nw; ++w) {
    const uint32_t cnt = starts[w + 1] - starts[w];
    if (cnt > ctx->cap_h[w]) {
      s.n = old_n;
      return fail(ctx, WRACH_ERR_CAPACITY,
                  "world " + std::to_string(w) + ": " + std::to_string(cnt) +
                      " particles in the frame exceed its capacity " + std::to_string(ctx->cap_h[w]));
    }
  }
  const uint32_t total = starts[nw];
  if (total && !direct) {
    CK(cudaMemcpyAsync(ctx->pos, ctx->pos_o, (size_t)total * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->vel, ctx->vel_o, (size_t)total * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
  }
  ctx->cur ^= 1;
  ctx->n = total;
  for (uint32_t w = 0; w < nw; ++w) {
    ctx->n_h[w] = starts[w + 1] - starts[w];
    ctx->poff_h[w] = starts[w];
  }
  ctx->graph_ok = true;
  if (!direct) CK(cudaStreamSynchronize(ctx->stream));
  return WRACH_OK;
}

// ---------------------------------------------------------------------------
// Viewport streaming
// ---------------------------------------------------------------------------

// The world's store becomes: its particles outside the viewport (store
// order), then the world's frame particles (frame order) -- per cell the
// reference's write-back of the GPU's particles into its store
// (particle_store.rs:71-85, a TODO there).
int write_back_impl(WrachContext* ctx, uint32_t world) {
  Store& s = ctx->stores[world];
  const uint32_t nf = ctx->n_h[world], off = ctx->poff_h[world];
  int rc;
  if ((rc = ensure_sort_capacity(ctx, (size_t)s.n + 1))) return rc;
  if ((rc = ensure_stage(ctx, (size_t)s.n + nf))) return rc;
  const uint32_t ntiles = wrach::keep_outside_tiles(s.n);
  if (ntiles + 1 > ctx->compact_cap) {
    dfree(ctx->compact_sums);
    ctx->compact_sums = nullptr;
    ctx->compact_cap = 0;
    CK(dalloc(&ctx->compact_sums, (size_t)ntiles + 1));
    ctx->compact_cap = (size_t)ntiles + 1;
  }
  uint32_t kept = 0;
  if (s.n) {
    CK(wrach::launch_upload_keys(ctx->worlds_d, (int)ctx->nworlds, ctx->ncells, world, 0, nullptr,
                                 s.n, s.pos, ctx->keys, ctx->stream));
    CK(wrach::launch_keep_outside(ctx->keys, ctx->ncells, s.n, s.pos, s.vel, ctx->stage_pos,
                                  ctx->stage_vel, ctx->compact_sums, ctx->compact_sums + ntiles,
                                  ctx->stream));
    ctx->launches += ntiles ? 4 : 2;
    CK(cudaMemcpyAsync(&kept, ctx->compact_sums + ntiles, 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  if (nf) {
    CK(cudaMemcpyAsync(ctx->stage_pos + kept, ctx->pos + off, (size_t)nf * sizeof(float2),
                       cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->stage_vel + kept, ctx->vel + off, (size_t)nf * sizeof(float2),
                       cudaMemcpyDeviceToDevice, ctx->stream));
  }
  if ((rc = ensure_store(ctx, s, (size_t)kept + nf))) return rc;
  if (kept + nf) {
    CK(cudaMemcpyAsync(s.pos, ctx->stage_pos, ((size_t)kept + nf) * sizeof(float2),
                       cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(s.vel, ctx->stage_vel, ((size_t)kept + nf) * sizeof(float2),
                       cudaMemcpyDeviceToDevice, ctx->stream));
  }
  s.n = kept + nf;
  CK(cudaStreamSynchronize(ctx->stream));
  return WRACH_OK;
}

}  // namespace

extern "C" {

int wrach_config_default(WrachConfig* c) {
  if (!c) return WRACH_ERR_INVALID_ARGUMENT;
  std::memset(c, 0, sizeof(*c));
  c->width = 480.0f;
  c->height = 352.0f;
  c->cell_size = 3;
  c->mode = WRACH_MODE_REFERENCE;
  c->iterations = 4;
  c->gravity = 0.0f;
  c->min_distance = 1.0f;
  c->max_velocity = 1.0f;
  c->cell_capacity = 9;
  c->capacity = 0;
  c->device = 0;
  return WRACH_OK;
}

uint32_t wrach_max_particles_per_frame(uint32_t cells, uint32_t cell_size) {
  const uint32_t cs2 = (uint32_t)(uint16_t)(cell_size * cell_size);
  const uint32_t normal = cells * cs2;
  const uint32_t one_percent = (normal + 99u) / 100u;
  return normal + 10u * one_percent;
}

int wrach_create(const WrachConfig* config, WrachContext** out) {
  return create_impl(config, 1, nullptr, out);
}

int wrach_create_batch(const WrachConfig* config, uint32_t nworlds, const float* dims,
                       WrachContext** out) {
  if (!dims) return WRACH_ERR_INVALID_ARGUMENT;
  return create_impl(config, nworlds, dims, out);
}

int wrach_destroy(WrachContext* ctx) {
  if (!ctx) return WRACH_ERR_INVALID_ARGUMENT;
  {
    DeviceGuard guard(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    // a frame's work on `aux` is joined into `stream`, unless its enqueue
    // failed between the fork and the join
    if (ctx->aux) cudaStreamSynchronize(ctx->aux);
    release(ctx);
  }
  delete ctx;
  return WRACH_OK;
}

int wrach_add_particles(WrachContext* ctx, uint32_t world, const float* pos, const float* vel,
                        uint32_t n) {
  return upload_impl(ctx, world, pos, vel, n, cudaMemcpyHostToDevice, false);
}

int wrach_set_particles(WrachContext* ctx, uint32_t world, const float* pos, const float* vel,
                        uint32_t n) {
  return upload_impl(ctx, world, pos, vel, n, cudaMemcpyHostToDevice, true);
}

int wrach_add_particles_device(WrachContext* ctx, uint32_t world, const float* d_pos,
                               const float* d_vel, uint32_t n) {
  return upload_impl(ctx, world, d_pos, d_vel, n, cudaMemcpyDeviceToDevice, false);
}

int wrach_step(WrachContext* ctx, uint32_t nsteps) {
  if (!ctx) return WRACH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(ctx->device);
  for (uint32_t s = 0; s < nsteps; ++s) {
    // a graph holds the particle count (grid sizes) it was captured with;
    // buffer reallocations drop the graphs
    if (ctx->graph[ctx->cur] && ctx->graph_n[ctx->cur] != ctx->n) {
      cudaGraphExecDestroy(ctx->graph[ctx->cur]);
      ctx->graph[ctx->cur] = nullptr;
    }
    if (ctx->graph_ok && !ctx->graph[ctx->cur]) {
      int rc = build_graph(ctx);
      if (rc) return rc;
    }
    if (ctx->graph_ok && ctx->graph[ctx->cur]) {
      CK(cudaGraphLaunch(ctx->graph[ctx->cur], ctx->stream));
      ctx->launches += frame_launches(ctx);
      ctx->cur ^= 1;
    } else {
      int rc = enqueue_frame(ctx);
      if (rc) return rc;
    }
  }
  return WRACH_OK;
}

int wrach_profile_frame(WrachContext* ctx, float* ms, uint32_t cap, uint32_t* count) {
  if (!ctx || !count) return WRACH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(ctx->device);
  const uint32_t nl = frame_steps(ctx);
  *count = nl;
  if (!ms || cap < nl) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "profile buffer too small");
  std::vector<cudaEvent_t> ev(nl + 1);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  ctx->event_hook = ev.data();
  ctx->event_count = 0;
  int rc = enqueue_frame(ctx);
  ctx->event_hook = nullptr;
  if (rc == WRACH_OK) {
    CK(cudaStreamSynchronize(ctx->stream));
    for (uint32_t i = 0; i < nl; ++i) CK(cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]));
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return rc;
}

int wrach_read(WrachContext* ctx, uint32_t world, float* positions, float* velocities,
               uint32_t* indices, uint32_t capacity) {
  if (!ctx) return WRACH_ERR_INVALID_ARGUMENT;
  if (world >= ctx->nworlds) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "world out of range");
  DeviceGuard guard(ctx->device);
  const uint32_t n = ctx->n_h[world], off = ctx->poff_h[world];
  if ((positions || velocities) && capacity < ctx->cap_h[world])
    return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "capacity smaller than the world's frame capacity");
  if (positions && n)
    CK(cudaMemcpyAsync(positions, ctx->pos + off, (size_t)n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  if (velocities && n)
    CK(cudaMemcpyAsync(velocities, ctx->vel + off, (size_t)n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  const WorldDev& w = ctx->worlds_h[world];
  const uint32_t cells = w.gx * w.gy;
  if (indices) {
    if (ctx->nworlds == 1) {
      CK(cudaMemcpyAsync(indices + 1, ctx->cs[ctx->cur], ((size_t)cells + 1) * 4,
                         cudaMemcpyDeviceToHost, ctx->stream));
    } else {
      CK(wrach::launch_world_table(ctx->cs[ctx->cur], w.cell_off, cells, ctx->table_tmp, ctx->stream));
      ctx->launches += 1;
      CK(cudaMemcpyAsync(indices, ctx->table_tmp, ((size_t)cells + 2) * 4, cudaMemcpyDeviceToHost,
                         ctx->stream));
    }
  }
  CK(cudaStreamSynchronize(ctx->stream));
  if (indices && ctx->nworlds == 1) indices[0] = 0;
  return WRACH_OK;
}

int wrach_tick(WrachContext* ctx, uint32_t world, float* positions, float* velocities,
               uint32_t* indices, uint32_t capacity) {
  int rc = wrach_step(ctx, 1);
  if (rc) return rc;
  return wrach_read(ctx, world, positions, velocities, indices, capacity);
}

int wrach_get_settings(WrachContext* ctx, uint32_t world, WrachWorldSettings* out) {
  if (!ctx || !out || world >= ctx->nworlds) return WRACH_ERR_INVALID_ARGUMENT;
  const WorldDev& w = ctx->worlds_h[world];
  out->view_dimensions[0] = w.dim_x;
  out->view_dimensions[1] = w.dim_y;
  out->view_anchor[0] = w.ax;
  out->view_anchor[1] = w.ay;
  out->grid_dimensions[0] = w.gx;
  out->grid_dimensions[1] = w.gy;
  out->cell_size = w.cs;
  out->particles_in_frame_count = ctx->n_h[world];
  return WRACH_OK;
}

int wrach_read_keys(WrachContext* ctx, uint32_t world, uint32_t* keys, uint32_t capacity) {
  if (!ctx) return WRACH_ERR_INVALID_ARGUMENT;
  if (world >= ctx->nworlds) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "world out of range");
  const uint32_t n = ctx->n_h[world], off = ctx->poff_h[world];
  if (n && (!keys || capacity < n)) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "key buffer too small");
  DeviceGuard guard(ctx->device);
  if (n) {
    // the keys land in the scratch the sort uses between frames
    int rc = ensure_sort_capacity(ctx, (size_t)n);
    if (rc) return rc;
    CK(wrach::launch_local_keys(ctx->cell_of[ctx->cur] + off, n, ctx->worlds_h[world].cell_off,
                                ctx->iB, ctx->stream));
    ctx->launches += 1;
    CK(cudaMemcpyAsync(keys, ctx->iB, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return WRACH_OK;
}

int wrach_write_back(WrachContext* ctx, uint32_t world) {
  if (!ctx) return WRACH_ERR_INVALID_ARGUMENT;
  if (world >= ctx->nworlds) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "world out of range");
  DeviceGuard guard(ctx->device);
  return write_back_impl(ctx, world);
}

int wrach_set_viewport(WrachContext* ctx, uint32_t world, float anchor_x, float anchor_y) {
  if (!ctx) return WRACH_ERR_INVALID_ARGUMENT;
  if (world >= ctx->nworlds) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "world out of range");
  DeviceGuard guard(ctx->device);
  const WorldDev old = ctx->worlds_h[world];
  WorldDev w;
  if (world_settings_init(w, old.dim_x, old.dim_y, anchor_x, anchor_y, old.cs) || w.gx != old.gx ||
      w.gy != old.gy)
    return fail(ctx, WRACH_ERR_INVALID_ARGUMENT,
                "the viewport at this anchor has a different grid size; move it by whole cells "
                "or use a size that is a multiple of the cell size");
  int rc = write_back_impl(ctx, world);
  if (rc) return rc;
  w.cell_off = old.cell_off;
  ctx->worlds_h[world] = w;
  CK(cudaMemcpyAsync(ctx->worlds_d + world, &ctx->worlds_h[world], sizeof(WorldDev),
                     cudaMemcpyHostToDevice, ctx->stream));
  // the frame, packed from the store under the new viewport
  return upload_impl(ctx, world, nullptr, nullptr, 0, cudaMemcpyDeviceToDevice, false);
}

int wrach_selftest_wait(WrachContext* ctx, uint32_t limit_us, uint32_t* timed_out,
                        uint32_t* waited_us) {
  if (!ctx || !timed_out || !waited_us) return WRACH_ERR_INVALID_ARGUMENT;
  if (limit_us > 1000000u) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "limit above 1 s");
  DeviceGuard guard(ctx->device);
  CK(wrach::launch_wait_probe(&ctx->ctrl->never_set, 0u, (uint64_t)limit_us * 1000u,
                              ctx->gather_out, ctx->stream));
  ctx->launches += 1;
  uint32_t h[2];
  CK(cudaMemcpyAsync(h, ctx->gather_out, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *timed_out = h[0];
  *waited_us = h[1];
  return WRACH_OK;
}

int wrach_store_size(WrachContext* ctx, uint32_t world, uint32_t* count) {
  if (!ctx || !count || world >= ctx->nworlds) return WRACH_ERR_INVALID_ARGUMENT;
  *count = ctx->stores[world].n;
  return WRACH_OK;
}

int wrach_read_store(WrachContext* ctx, uint32_t world, float* positions, float* velocities,
                     uint32_t capacity) {
  if (!ctx || world >= ctx->nworlds) return WRACH_ERR_INVALID_ARGUMENT;
  const Store& s = ctx->stores[world];
  if (capacity < s.n) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "capacity smaller than the store");
  DeviceGuard guard(ctx->device);
  if (positions && s.n)
    CK(cudaMemcpyAsync(positions, s.pos, (size_t)s.n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  if (velocities && s.n)
    CK(cudaMemcpyAsync(velocities, s.vel, (size_t)s.n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return WRACH_OK;
}

uint32_t wrach_capacity(WrachContext* ctx, uint32_t world) {
  if (!ctx || world >= ctx->nworlds) return 0;
  return ctx->cap_h[world];
}

uint32_t wrach_num_worlds(WrachContext* ctx) { return ctx ? ctx->nworlds : 0; }

int wrach_render(WrachContext* ctx, uint32_t world, uint32_t width_px, uint32_t height_px,
                 uint8_t* image) {
  if (!ctx || !image || !width_px || !height_px) return WRACH_ERR_INVALID_ARGUMENT;
  if (world >= ctx->nworlds) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "world out of range");
  DeviceGuard guard(ctx->device);
  const size_t npix = (size_t)width_px * height_px;
  if (npix > ctx->render_cap) {
    dfree(ctx->render_cover);
    dfree(ctx->render_image);
    ctx->render_cover = nullptr;
    ctx->render_image = nullptr;
    ctx->render_cap = 0;
    CK(dalloc(&ctx->render_cover, npix));
    CK(dalloc(&ctx->render_image, npix));
    ctx->render_cap = npix;
  }
  const WorldDev& w = ctx->worlds_h[world];
  CK(wrach::launch_render(ctx->pos + ctx->poff_h[world], ctx->n_h[world], w.dim_x, w.dim_y, width_px,
                          height_px, ctx->render_cover, ctx->render_image, ctx->stream));
  ctx->launches += ctx->n_h[world] ? 2 : 1;
  CK(cudaMemcpyAsync(image, ctx->render_image, npix, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return WRACH_OK;
}

int wrach_sync(WrachContext* ctx) {
  if (!ctx) return WRACH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(ctx->device);
  CK(cudaStreamSynchronize(ctx->stream));
  return WRACH_OK;
}

int wrach_flags(WrachContext* ctx, uint32_t* flags) {
  if (!ctx || !flags) return WRACH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(ctx->device);
  Ctrl h{};
  CK(cudaMemcpyAsync(&h, ctx->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *flags = h.flags;
  return WRACH_OK;
}

int wrach_stats(WrachContext* ctx, WrachStats* out) {
  if (!ctx || !out) return WRACH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(ctx->device);
  Ctrl h{};
  CK(cudaMemcpyAsync(&h, ctx->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  std::memset(out, 0, sizeof(*out));
  out->flags = h.flags;
  out->frames = h.frames;
  out->overflow = h.overflow;
  out->rebin_blocks = ctx->big_blocks;
  out->tiles = ctx->ntiles;
  out->particles = ctx->n;
  out->cells = ctx->ncells;
  out->huge_cells = h.huge_cells;
  return WRACH_OK;
}

const char* wrach_last_error(WrachContext* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

uint64_t wrach_kernel_launches(WrachContext* ctx) { return ctx ? ctx->launches : 0; }

void* wrach_stream(WrachContext* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

}  // extern "C"
