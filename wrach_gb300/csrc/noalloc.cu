// wrach_pack_noalloc: the device-side packing of particles into cell order
// (the upload binning behind wrach_add_particles) for callers that cannot
// allocate GPU memory.
//
// Who needs it: code that runs where cudaMalloc is off limits, for instance
// inside a host callback or a real-time frame loop that must never stall on
// the allocator, a plugin whose host application owns all device memory
// through its own pool, or a process that has already committed every byte
// it may use.  Such a caller brings the input and output arrays; every
// temporary this call needs lives in one file-scope device array, sized for
// at most kNoAllocMaxParticles particles and kNoAllocMaxCells grid cells
// (about 6.3 MB, held by every GPU that loads this library until the process
// exits).
//
// The array's name, used in host code, is only a host-side stand-in for the
// device symbol: its device address is obtained with cudaGetSymbolAddress,
// once per device, on the first call made with that device current, and the
// kernels get that address.  That first call therefore does a little set-up
// work; make it before any stream capture.  All calls share the one array,
// so calls whose work overlaps on the GPU (other streams, other threads)
// race with each other; serialise them on one stream.
//
// The call returns before its kernels run, so what can only be known on the
// device (a grid barrier of the rebin that gave up, particles that did not
// fit out_capacity) is written, once the kernels are done, to the caller's
// optional two-word device status array.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/wrach.h"
#include "wrach_kernels.h"

namespace {

using wrach::Ctrl;

constexpr uint32_t kNoAllocMaxParticles = 131072;  // 2^17
constexpr uint32_t kNoAllocMaxCells = 524288;      // 2^19
constexpr uint32_t kNoAllocMaxBlocks = 1024;       // rebin grid the digit table holds
constexpr uint32_t kNoAllocMaxDevices = 64;

// Word offsets of the regions of the scratch array.
constexpr size_t kCtrlWords = 128;  // >= sizeof(Ctrl) / 4
constexpr size_t kOffCtrl = 0;
constexpr size_t kOffKeys = kOffCtrl + kCtrlWords;
constexpr size_t kOffKA = kOffKeys + kNoAllocMaxParticles;
constexpr size_t kOffKB = kOffKA + kNoAllocMaxParticles;
constexpr size_t kOffIA = kOffKB + kNoAllocMaxParticles;
constexpr size_t kOffIB = kOffIA + kNoAllocMaxParticles;
constexpr size_t kOffCell = kOffIB + kNoAllocMaxParticles;
constexpr size_t kOffCounts = kOffCell + kNoAllocMaxParticles;
constexpr size_t kOffTiles = kOffCounts + kNoAllocMaxCells + 64;
constexpr size_t kOffHist = kOffTiles + kNoAllocMaxCells / wrach::kTileCells + 64;
constexpr size_t kScratchWords = kOffHist + 256 * (kNoAllocMaxBlocks + 1);
static_assert(sizeof(Ctrl) <= kCtrlWords * 4, "control block fits its region");

static __device__ __align__(256) uint32_t wrach_noalloc_scratch[kScratchWords];

std::mutex g_setup_mutex;
uint32_t* g_scratch[kNoAllocMaxDevices] = {};

// SpatialBin::get_cell_coord (runners/bevy/src/spatial_bin.rs:48-64):
// Rust's f32::div_euclid, then a saturating `as i32` (NaN -> 0).
__device__ __forceinline__ int32_t noalloc_cell_coord(float x, uint32_t cs) {
  const float d = (float)cs;
  float q = truncf(__fdiv_rn(x, d));
  if (fmodf(x, d) < 0.0f) q = __fsub_rn(q, 1.0f);
  if (q != q) return 0;
  if (q >= 2147483648.0f) return 2147483647;
  if (q <= -2147483648.0f) return -2147483647 - 1;
  return (int32_t)q;
}

// Cell key of each input particle in the world's grid, `ncells` for the
// particles outside it (left out of the frame, as create_packed_data does).
__global__ void k_noalloc_keys(wrach::WorldDev w, uint32_t ncells, uint32_t n,
                               const float2* __restrict__ pos,
                               uint32_t* __restrict__ keys) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 p = pos[i];
  const int64_t cx = (int64_t)noalloc_cell_coord(p.x, w.cs) - w.blx;
  const int64_t cy = (int64_t)noalloc_cell_coord(p.y, w.cs) - w.bly;
  keys[i] = (cx < 0 || cy < 0 || cx >= (int64_t)w.gx || cy >= (int64_t)w.gy)
                ? ncells
                : (uint32_t)cy * w.gx + (uint32_t)cx;
}

int32_t host_cell_coord(float x, uint32_t cs) {
  volatile float d = (float)cs;
  float q = std::trunc(x / d);
  if (std::fmod(x, (float)d) < 0.0f) q = q - 1.0f;
  if (q != q) return 0;
  if (q >= 2147483648.0f) return INT32_MAX;
  if (q <= -2147483648.0f) return INT32_MIN;
  return (int32_t)q;
}

// Makes `dev` the current device for the lifetime of the object (ok is false
// if that failed) and restores the caller's device afterwards.
struct CurrentDevice {
  int prev = -1;
  bool ok = false;
  explicit CurrentDevice(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev && cudaSetDevice(dev) != cudaSuccess) return;
    int now = -1;
    ok = cudaGetDevice(&now) == cudaSuccess && now == dev;
  }
  ~CurrentDevice() {
    int now = -1;
    if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
  }
};

// The call's device-side outcome for the caller: status[0] = the WRACH_FLAG_*
// bits the rebin raised (WRACH_FLAG_TIMEOUT: a grid barrier gave up), plus
// WRACH_FLAG_OVERFLOW when particles did not fit out_capacity; status[1] =
// how many did not fit.
__global__ void k_noalloc_status(const Ctrl* __restrict__ ctrl, uint32_t* __restrict__ status) {
  const uint32_t overflow = ctrl->overflow;
  status[0] = ctrl->flags | (overflow ? WRACH_FLAG_OVERFLOW : 0u);
  status[1] = overflow;
}

// One launch whose own return code is checked: an error left behind by the
// caller's earlier CUDA calls is neither reported nor cleared here.
template <typename... Params, typename... Args>
cudaError_t launch(void (*kernel)(Params...), uint32_t blocks, uint32_t threads,
                   cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(threads);
  cfg.stream = st;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace

extern "C" int wrach_pack_noalloc(const WrachConfig* config, const float* d_pos,
                                  const float* d_vel, uint32_t n, float* d_pos_out,
                                  float* d_vel_out, uint32_t out_capacity,
                                  uint32_t* d_indices, uint32_t* d_status, void* stream) {
  if (!config || (n && (!d_pos || !d_vel)) || !d_pos_out || !d_vel_out || !d_indices)
    return WRACH_ERR_INVALID_ARGUMENT;
  if (config->cell_size == 0 || config->device < 0 ||
      config->device >= (int32_t)kNoAllocMaxDevices)
    return WRACH_ERR_INVALID_ARGUMENT;
  if (n > kNoAllocMaxParticles) return WRACH_ERR_CAPACITY;  // more than the scratch holds

  // the grid, as SpatialBin::get_active_cells sizes it (spatial_bin.rs:68-95)
  wrach::WorldDev w;
  std::memset(&w, 0, sizeof(w));
  w.dim_x = config->width;
  w.dim_y = config->height;
  w.ax = config->anchor_x;
  w.ay = config->anchor_y;
  w.cs = config->cell_size;
  volatile float x1 = w.ax + w.dim_x, y1 = w.ay + w.dim_y;
  w.x1 = x1;
  w.y1 = y1;
  w.blx = host_cell_coord(w.ax, w.cs);
  w.bly = host_cell_coord(w.ay, w.cs);
  const int64_t gx = (int64_t)host_cell_coord(x1, w.cs) - w.blx + 1;
  const int64_t gy = (int64_t)host_cell_coord(y1, w.cs) - w.bly + 1;
  if (gx <= 0 || gy <= 0) return WRACH_ERR_INVALID_ARGUMENT;
  if (gx * gy > (int64_t)kNoAllocMaxCells) return WRACH_ERR_CAPACITY;  // grid beyond the scratch
  w.gx = (uint32_t)gx;
  w.gy = (uint32_t)gy;
  const uint32_t ncells = w.gx * w.gy;

  CurrentDevice current(config->device);
  if (!current.ok) return WRACH_ERR_CUDA;  // the address below must be this device's
  uint32_t* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch[config->device]) {
      void* ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, wrach_noalloc_scratch) != cudaSuccess || !ptr)
        return WRACH_ERR_CUDA;
      g_scratch[config->device] = static_cast<uint32_t*>(ptr);
    }
    base = g_scratch[config->device];
  }

  uint32_t key_bits = 0;
  while (key_bits < 32 && (ncells >> key_bits) != 0) ++key_bits;
  const uint32_t digit_bits = wrach::rebin_digit_bits(key_bits);
  int grid = wrach::rebin_grid_size(config->device, digit_bits);
  if (grid <= 0) return WRACH_ERR_CUDA;
  if (grid > (int)kNoAllocMaxBlocks) grid = (int)kNoAllocMaxBlocks;
  if (((size_t)1 << digit_bits) * (grid + 1) > 256 * (kNoAllocMaxBlocks + 1))
    return WRACH_ERR_UNSUPPORTED;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the control block and the per-cell counts must start at zero; every
  // other region is written before it is read
  if (cudaMemsetAsync(base + kOffCtrl, 0, kCtrlWords * 4, st) != cudaSuccess ||
      cudaMemsetAsync(base + kOffCounts, 0, ((size_t)ncells + 1) * 4, st) != cudaSuccess ||
      cudaMemsetAsync(d_indices, 0, 4, st) != cudaSuccess)
    return WRACH_ERR_CUDA;
  if (n && launch(k_noalloc_keys, (n + 255) / 256, 256, st, w, ncells, n,
                  reinterpret_cast<const float2*>(d_pos), base + kOffKeys) != cudaSuccess)
    return WRACH_ERR_CUDA;

  wrach::RebinArgs r{};
  r.worlds = nullptr;
  r.nworlds = 1;
  r.ncells = ncells;
  r.n = n;
  r.dst_capacity = out_capacity;
  r.keys = base + kOffKeys;
  r.pos_src = reinterpret_cast<const float2*>(d_pos);
  r.vel_src = reinterpret_cast<const float2*>(d_vel);
  r.cs_new = d_indices + 1;  // the reference layout: indices[c + 1] = start of cell c
  r.pos_dst = reinterpret_cast<float2*>(d_pos_out);
  r.vel_dst = reinterpret_cast<float2*>(d_vel_out);
  r.cell_dst = base + kOffCell;
  r.tile_sums = base + kOffTiles;
  r.kA = base + kOffKA;
  r.kB = base + kOffKB;
  r.iA = base + kOffIA;
  r.iB = base + kOffIB;
  r.hist = base + kOffHist;
  r.key_bits = key_bits;
  r.digit_bits = digit_bits;
  r.force_general = 1;
  r.counts = base + kOffCounts;
  r.ctrl = reinterpret_cast<Ctrl*>(base + kOffCtrl);
  if (wrach::launch_rebin(r, grid, st) != cudaSuccess) return WRACH_ERR_CUDA;
  if (d_status && launch(k_noalloc_status, 1, 1, st, r.ctrl, d_status) != cudaSuccess)
    return WRACH_ERR_CUDA;
  return WRACH_OK;
}
