// Host-side state of a context and the helpers shared by the files of the C
// ABI: context.cu (lifetime, uploads, frames, viewport streaming, readback)
// and surrogate_host.cu (the learned surrogate).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/wrach.h"
#include "wrach_kernels.h"

namespace wrach {
namespace host {

// A world's device-resident particle store.
struct Store {
  float2* pos = nullptr;
  float2* vel = nullptr;
  uint32_t n = 0;
  uint32_t cap = 0;
};

}  // namespace host
}  // namespace wrach

struct WrachContext {
  int device = 0;
  cudaStream_t stream = nullptr;
  // a frame's large-cell sort runs on `aux`, beside the small cells' pass
  cudaStream_t aux = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  // uploads: the per-world counts read back (the call waits for them only)
  cudaEvent_t counts_ev = nullptr;
  WrachConfig cfg{};
  wrach::PhysDev ph{};
  uint32_t nworlds = 0;
  std::vector<wrach::WorldDev> worlds_h;
  std::vector<uint32_t> cap_h;   // frame capacity per world
  std::vector<uint32_t> n_h;     // frame particles per world
  std::vector<uint32_t> poff_h;  // first frame particle of each world
  uint32_t ncells = 0;
  uint32_t total_cap = 0;
  uint32_t n = 0;
  uint32_t max_world_cells = 0;
  wrach::WorldDev* worlds_d = nullptr;
  float2 *pos = nullptr, *vel = nullptr, *pos_o = nullptr, *vel_o = nullptr;
  float2 *q1 = nullptr, *q2 = nullptr;
  uint32_t* rows = nullptr;  // the iterations' neighbour rows: 4 planes of total_cap u32
  uint32_t* cell_of[2] = {nullptr, nullptr};
  uint32_t* cs[2] = {nullptr, nullptr};
  int cur = 0;
  uint32_t* keys = nullptr;
  uint32_t *kA = nullptr, *kB = nullptr, *iA = nullptr, *iB = nullptr;
  size_t sort_cap = 0;
  uint32_t* tile_sums = nullptr;  // one word per tile of the cell table
  // extended physics: the taking-part particles compacted (ping-pong with cs)
  uint32_t* ct[2] = {nullptr, nullptr};       // capped table, cells + 1
  float2* tp_pos[2] = {nullptr, nullptr};     // compacted positions
  float2* tp_vel[2] = {nullptr, nullptr};     // compacted velocities
  uint32_t* tp_cell[2] = {nullptr, nullptr};  // compacted cells
  uint32_t* tile_sums_cap = nullptr;          // per scan tile, taking-part particles
  uint32_t ntiles = 0;
  uint32_t* big_list = nullptr;               // counting sort: large-cell work list
  uint32_t big_cap = 0;
  int sms = 0;
  wrach::Ctrl* ctrl = nullptr;
  uint32_t big_blocks = 0;  // grid of the rebin's large-cell sort
  std::vector<wrach::host::Store> stores;
  float2 *stage_pos = nullptr, *stage_vel = nullptr;
  size_t stage_cap = 0;
  uint32_t* compact_sums = nullptr;   // viewport streaming: tile sums + 1 count word
  size_t compact_cap = 0;
  uint32_t* counts = nullptr;     // per-cell counts of the rebin (ncells + 1)
  uint32_t* table_tmp = nullptr;  // one world's reference-layout table
  uint32_t* gather_idx = nullptr; // nworlds + 1
  uint32_t* gather_out = nullptr;
  uint32_t* gather_h = nullptr;   // pinned host copy of gather_out (nworlds + 1)
  std::string err;
  uint64_t launches = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  uint32_t graph_n[2] = {0, 0};       // particle count each graph was captured with
  bool graph_ok = true;
  uint32_t* render_cover = nullptr;   // wrach_render scratch and image
  uint8_t* render_image = nullptr;
  size_t render_cap = 0;
  cudaEvent_t* event_hook = nullptr;  // wrach_profile_frame: one event per launch boundary
  uint32_t event_count = 0;
  // the learned surrogate (wrach_surrogate_*)
  struct {
    bool ready = false;
    wrach::MlpDev m{};
    float *params = nullptr, *grad = nullptr, *mom1 = nullptr, *mom2 = nullptr;
    float *loss = nullptr, *metrics = nullptr;
    float* part = nullptr;           // per-block metrics of a solve launch (8 floats a block)
    wrach::GateState* gate = nullptr;
    uint16_t* bf16 = nullptr;        // the six BF16 weight arrays
    uint16_t* x = nullptr;           // features of the frame (capacity rows)
    float2* corr = nullptr;          // the network's output (capacity)
    uint16_t* tx = nullptr;          // training features (max_samples rows)
    float2* tt = nullptr;            // training targets
    uint32_t nsamples = 0, max_samples = 0, step = 0;
    uint32_t collects = 0;           // wrach_surrogate_collect calls since init
    int blocks = 0;
    int correct_blocks = 0;          // grid of the fused correction kernel (one wave)
    // surrogate frames as CUDA graphs: [table parity][calibration frame]
    cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    uint32_t graph_n[2][2] = {{0, 0}, {0, 0}};         // particle count at capture
    uint32_t graph_launches[2][2] = {{0, 0}, {0, 0}};  // kernel launches per graph
  } sur;
};

namespace wrach {
namespace host {

// Records `msg` as the context's last error and returns `code`.
int fail(WrachContext* c, int code, const std::string& msg);

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void**)p, count * sizeof(T));
}

void dfree(void* p);

// Makes `dev` current for the scope of a C ABI call.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int now = -1;
    if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev)
      cudaSetDevice(prev);
  }
};

// The launch arguments of the context's current binned frame.
wrach::SolveArgs solve_args(WrachContext* ctx);
wrach::RebinArgs rebin_args(WrachContext* ctx);
// What a frame's last extended pass needs to take the rebin's tickets.
wrach::CountDev ticket_args(WrachContext* ctx);

// The first `count` extended iterations of the binned frame over the
// compacted taking-part particles, from a.tp_pos through the iterates q1 and
// q2 in turn; *q receives the last iterate (a.tp_pos when count is 0).
// `after` runs after each launch.
template <typename After>
cudaError_t enqueue_iterations(WrachContext* ctx, const wrach::SolveArgs& a, uint32_t count,
                               cudaStream_t st, const float2** q, After after) {
  const float2* src = a.tp_pos;
  for (uint32_t it = 0; it < count; ++it) {
    float2* dst = (it & 1) ? ctx->q2 : ctx->q1;
    // the first iteration writes the particles' neighbour rows, the later
    // ones read them
    wrach::SolveArgs ai = a;
    ai.rows_mode = count > 1 ? (it == 0 ? 1 : 2) : 0;
    const cudaError_t e = wrach::launch_jacobi_iteration(ai, src, dst, st);
    if (e != cudaSuccess) return e;
    after();
    src = dst;
  }
  *q = src;
  return cudaSuccess;
}

}  // namespace host
}  // namespace wrach

// Returns a status from the enclosing C ABI function (with `ctx` in scope)
// when a CUDA call fails.
#define CK(call)                                                             \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      return wrach::host::fail(ctx,                                          \
                               e_ == cudaErrorMemoryAllocation               \
                                   ? WRACH_ERR_OUT_OF_MEMORY                 \
                                   : WRACH_ERR_CUDA,                         \
                               std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
