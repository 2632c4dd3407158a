// The surrogate network's forward pass on the 5th-generation tensor cores
// (tcgen05): the same network as surrogate.cu's k_mlp_forward (64 -> 64 ->
// 64 -> 2, tanh-form GELU after the hidden layers on packed FP16 pairs,
// BF16 weights and activations, FP32 accumulation) with the operands in
// shared memory and the accumulators in tensor memory (TMEM) instead of
// registers.
//
// One CTA of 256 threads takes tiles of 128 rows (M = 128), persistent over
// the rows, two tiles at a time in two slots, each with its own operand
// buffer, 64 TMEM columns and mbarrier.  Per tile and layer: one thread
// issues the layer's tcgen05.mma (K = 64 as four K = 16 steps) into the
// slot's columns and commits them to the slot's mbarrier; the threads wait
// on it, read their part of the accumulator from TMEM (tcgen05.ld: warp w
// reads TMEM lanes 32 (w % 4) .. + 31, the tile's rows, and columns
// 32 (w / 4) .. + 31 of the layer), add the bias, apply the GELU, round to
// BF16 and write them back into the slot's operand buffer for the next
// layer.  The slots alternate, so one tile's MMAs run while the threads work
// on the other tile's epilogue; the next tiles' features are copied into the
// freed buffers with cp.async while the outputs are written.  Several CTAs
// share an SM as well.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, element (r, k) of a [rows][64] BF16 matrix at
// byte (r / 8) * 1024 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2, so the
// descriptors' K-direction core-matrix offset (leading byte offset) is 128 B
// and the row-direction one (stride byte offset) 1024 B.  A weight matrix is
// the B operand as [out][in], K-major: D[row][out] = sum_in X[row][in] W[in][out].
//
// Every wait on the mbarrier is bounded (kWaitLimitNs): past it the kernel
// raises kFlagTimeout, waits once more (bounded) for its MMAs in flight,
// frees its TMEM and returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include "gelu.cuh"
#include "wrach_internal.cuh"
#include "wrach_kernels.h"

namespace wrach {

namespace {

constexpr uint32_t kTcRows = 128;     // M: rows per tile
constexpr uint32_t kTcThreads = 256;  // two threads per row in the epilogues
constexpr uint32_t kTcCols = 128;     // TMEM columns: slot s's layers at 64 s .. 64 s + 63
constexpr uint32_t kTcPerSm = 4;      // CTAs per SM: 4 x 128 columns = the SM's 512
constexpr uint32_t kCoreRowBytes = 1024, kCoreKBytes = 128;

__host__ __device__ constexpr uint32_t cm_off(uint32_t r, uint32_t k) {
  return (r >> 3) * kCoreRowBytes + (k >> 3) * kCoreKBytes + (r & 7u) * 16u + (k & 7u) * 2u;
}

struct SmemTc {
  uint8_t a[2][kTcRows * kMlpIn * 2];   // per slot, its tile: features, then activations
  uint8_t w1[kMlpHidden * kMlpIn * 2];  // B operands, [out][in]
  uint8_t w2[kMlpHidden * kMlpHidden * 2];
  uint8_t w3[16 * kMlpHidden * 2];      // outputs 8..15 zero (N = 16)
  alignas(16) float b1[kMlpHidden];
  alignas(16) float b2[kMlpHidden];
  float b3[kMlpOutPad];
  uint64_t mbar[2];
  uint32_t tmem;
};
// a dynamic size that lets at most kTcPerSm CTAs share an SM (TMEM columns)
constexpr size_t kTcSmem = 56 * 1024;
static_assert(sizeof(SmemTc) <= kTcSmem, "the CTA's shared memory holds its operands");

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (no swizzle): start, leading (K-direction)
// and stride (row-direction) byte offsets, each stored >> 4, and the
// descriptor version 1 at bit 46.
__device__ __forceinline__ uint64_t smem_desc(const void* p) {
  const uint32_t a = smem_u32(p);
  return (uint64_t)((a & 0x3FFFFu) >> 4) | ((uint64_t)(kCoreKBytes >> 4) << 16) |
         ((uint64_t)(kCoreRowBytes >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bit 4), BF16 A and
// B (bits 7 and 10), both K-major, N / 8 at bit 17, M / 16 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t m, uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                    uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

// The layer: K = 64 as four K = 16 steps (two core matrices each), then the
// commit of the steps to the mbarrier.
__device__ __forceinline__ void mma_layer(uint32_t d_tmem, const uint8_t* a, const uint8_t* b,
                                          uint32_t idesc, uint64_t* mbar) {
#pragma unroll
  for (uint32_t kk = 0; kk < kMlpIn / 16; ++kk)
    mma(d_tmem, smem_desc(a + kk * 2 * kCoreKBytes), smem_desc(b + kk * 2 * kCoreKBytes), idesc,
        kk);
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t phase, uint64_t limit_ns) {
  const uint64_t t0 = global_ns();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(phase)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy writes to shared memory made visible to the tensor cores
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32 consecutive FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, float& v0, float& v1) {
  uint32_t r0, r1;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];"
               : "=r"(r0), "=r"(r1)
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  v0 = __uint_as_float(r0);
  v1 = __uint_as_float(r1);
}

// Bias, GELU and BF16 rounding of this thread's 32 accumulators (columns
// 32 h .. 32 h + 31 of the layer at TMEM address taddr), written into row
// `row` of the operand buffer.
__device__ __forceinline__ void hidden_epilogue(uint32_t taddr, const float* bias, uint8_t* a,
                                                uint32_t row, uint32_t h) {
  {
    float v[32];
    tmem_ld32(taddr + h * 32, v);
    const float4* b4 = reinterpret_cast<const float4*>(bias + h * 32);  // 16-byte aligned
#pragma unroll
    for (uint32_t c = 0; c < 4; ++c) {
      const float4 lo = b4[2 * c], hi = b4[2 * c + 1];
      const float b[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
      uint32_t w[4];
#pragma unroll
      for (uint32_t q = 0; q < 4; ++q) {
        const uint32_t k = c * 8 + 2 * q;
        w[q] = gelu2_bf16(v[k] + b[2 * q], v[k + 1] + b[2 * q + 1]);
      }
      *reinterpret_cast<uint4*>(a + cm_off(row, h * 32 + c * 8)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
}

// rows x 64 BF16 [n][k] from global memory into a core-matrix operand
__device__ __forceinline__ void load_operand(uint8_t* dst, const uint16_t* src, uint32_t rows,
                                             uint32_t zero_from) {
  for (uint32_t i = threadIdx.x; i < rows * 8; i += blockDim.x) {
    const uint32_t r = i >> 3, kc = i & 7u;
    const uint4 v = r < zero_from ? *reinterpret_cast<const uint4*>(src + r * kMlpIn + kc * 8)
                                  : make_uint4(0u, 0u, 0u, 0u);
    *reinterpret_cast<uint4*>(dst + cm_off(r, kc * 8)) = v;
  }
}

__global__ void __launch_bounds__(kTcThreads, kTcPerSm)
k_mlp_forward_tc(MlpDev m, const uint16_t* __restrict__ x, uint32_t n, float2* __restrict__ y,
                 uint32_t* __restrict__ flags) {
  extern __shared__ __align__(1024) uint8_t dyn[];
  SmemTc& s = *reinterpret_cast<SmemTc*>(dyn);
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  // epilogue rows and column half of this thread
  const uint32_t row_in_tile = (warp & 3u) * 32u + (tid & 31u), half = warp >> 2;
  load_operand(s.w1, m.w1t, kMlpHidden, kMlpHidden);
  load_operand(s.w2, m.w2t, kMlpHidden, kMlpHidden);
  load_operand(s.w3, m.w3t, 16, kMlpOutPad);
  for (uint32_t i = tid; i < kMlpHidden; i += blockDim.x) {
    s.b1[i] = m.b1[i];
    s.b2[i] = m.b2[i];
  }
  if (tid < kMlpOutPad) s.b3[tid] = m.b3[tid];
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&s.tmem)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (uint32_t q = 0; q < 2; ++q)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s.mbar[q])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_async_smem();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = s.tmem;
  const uint32_t lane_base = tmem + (((warp & 3u) * 32u) << 16);  // this warp's 32 TMEM lanes
  uint32_t phase[2] = {0u, 0u};
  bool pending[2] = {false, false};  // an MMA committed to the slot's mbarrier, not yet waited
  bool failed = false;               // a wait of this thread gave up
  // the layer of slot q: its operand buffer (written by every thread) made
  // visible to the tensor cores, the slot's earlier TMEM reads finished; the
  // barrier also tells every thread whether a wait gave up anywhere, in
  // which case nothing is issued and the caller stops
  auto issue = [&](uint32_t q, const uint8_t* w, uint32_t nout) {
    fence_async_smem();
    fence_before();
    if (__syncthreads_or(failed ? 1 : 0)) return false;
    if (tid == 0) {
      fence_after();
      mma_layer(tmem + 64u * q, s.a[q], w, idesc_bf16(kTcRows, nout), &s.mbar[q]);
    }
    pending[q] = true;
    return true;
  };
  // this thread's wait for slot q's MMA (no barrier: the next issue's
  // barrier reports a wait that gave up; one that gave up keeps the slot's
  // phase, so the last bounded wait before the TMEM is freed still waits
  // for that MMA)
  auto wait = [&](uint32_t q) {
    if (mbar_wait(&s.mbar[q], phase[q], kWaitLimitNs)) {
      phase[q] ^= 1u;
      pending[q] = false;
    } else {
      failed = true;
    }
    fence_after();
  };
  // a tile's features, 16-byte chunks with consecutive threads along a row,
  // into slot q's buffer by cp.async (rows past n are zero-filled)
  auto load = [&](uint32_t q, uint32_t tile) {
#pragma unroll
    for (uint32_t u = 0; u < kTcRows * 8 / kTcThreads; ++u) {
      const uint32_t i = tid + u * kTcThreads, grow = tile * kTcRows + (i >> 3);
      const bool in = grow < n;
      const uint16_t* src = x + (size_t)(in ? grow : 0u) * kMlpIn + (i & 7u) * 8;
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(
                       smem_u32(s.a[q] + cm_off(i >> 3, (i & 7u) * 8))),
                   "l"(src), "r"(in ? 16u : 0u)
                   : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  auto loaded = [&]() { asm volatile("cp.async.wait_all;" ::: "memory"); };
  auto output = [&](uint32_t q, uint32_t tile) {
    const uint32_t row = tile * kTcRows + row_in_tile;
    if (half == 0) {
      float y0, y1;
      tmem_ld2(lane_base + 64u * q, y0, y1);
      if (row < n) y[row] = make_float2(y0 + s.b3[0], y1 + s.b3[1]);
    }
  };
  const uint32_t step = 2u * gridDim.x;
  uint32_t t0 = blockIdx.x, t1 = blockIdx.x + gridDim.x;
  bool has0 = t0 * kTcRows < n, has1 = t1 * kTcRows < n;  // has1 implies has0
  bool ok = true;
  if (has0) load(0, t0);
  if (has1) load(1, t1);
  loaded();
  if (has0) ok = issue(0, s.w1, kMlpHidden);
  if (ok && has1) ok = issue(1, s.w1, kMlpHidden);
  while (ok && has0) {
    wait(0);
    hidden_epilogue(lane_base + 0u, s.b1, s.a[0], row_in_tile, half);
    if (!(ok = issue(0, s.w2, kMlpHidden))) break;
    if (has1) {
      wait(1);
      hidden_epilogue(lane_base + 64u, s.b1, s.a[1], row_in_tile, half);
      if (!(ok = issue(1, s.w2, kMlpHidden))) break;
    }
    wait(0);
    hidden_epilogue(lane_base + 0u, s.b2, s.a[0], row_in_tile, half);
    if (!(ok = issue(0, s.w3, 16))) break;
    if (has1) {
      wait(1);
      hidden_epilogue(lane_base + 64u, s.b2, s.a[1], row_in_tile, half);
      if (!(ok = issue(1, s.w3, 16))) break;
    }
    // the last layers read their buffers: once each is done, its next
    // tile's features are copied in while the outputs are written (a
    // buffer whose wait gave up is left alone)
    const uint32_t n0 = t0 + step, n1 = t1 + step;
    const bool next0 = n0 * kTcRows < n, next1 = n1 * kTcRows < n;
    wait(0);
    if (next0 && !failed) load(0, n0);
    output(0, t0);
    if (has1) {
      wait(1);
      if (next1 && !failed) load(1, n1);
      output(1, t1);
    }
    loaded();
    t0 = n0;
    t1 = n1;
    has0 = next0;
    has1 = next1;
    if (has0) ok = issue(0, s.w1, kMlpHidden);
    if (ok && has1) ok = issue(1, s.w1, kMlpHidden);
  }
  loaded();
  ok = __syncthreads_or(failed ? 1 : 0) == 0;
  if (!ok) {
    // a wait gave up: report it, give the MMAs in flight one more bounded
    // wait, then free the TMEM
    if (tid == 0) atomicOr(flags, kFlagTimeout);
    for (uint32_t q = 0; q < 2; ++q)
      if (pending[q]) mbar_wait(&s.mbar[q], phase[q], kWaitLimitNs);
  }
  fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols)
                 : "memory");
}

}  // namespace

cudaError_t launch_mlp_forward_tc(const MlpDev& m, const uint16_t* x, uint32_t n, float2* y,
                                  uint32_t* flags, int sms, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kTcSmem);
  if (e != cudaSuccess) return e;
  const uint32_t tiles = (n + kTcRows - 1) / kTcRows;
  const uint32_t wave = kTcPerSm * (uint32_t)(sms > 0 ? sms : 1);
  k_mlp_forward_tc<<<tiles < wave ? tiles : wave, kTcThreads, kTcSmem, st>>>(m, x, n, y, flags);
  return cudaGetLastError();
}

}  // namespace wrach
