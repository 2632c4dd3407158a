// The surrogate network's forward pass on the 5th-generation tensor cores
// (tcgen05): the same network as surrogate.cu's k_mlp_forward (64 -> 64 ->
// 64 -> 2, tanh-form GELU after the hidden layers on packed FP16 pairs,
// BF16 weights and activations, FP32 accumulation) with the operands in
// shared memory and the accumulators in tensor memory (TMEM) instead of
// registers.
//
// One CTA of 256 threads takes tiles of 128 rows (M = 128), persistent over
// the rows.  Per tile: the threads copy the tile's features into shared
// memory; one thread issues the layer's tcgen05.mma (K = 64 as four K = 16
// steps) and commits them to an mbarrier; the threads wait on it, read their
// part of the accumulator from TMEM (tcgen05.ld: warp w reads TMEM lanes
// 32 (w % 4) .. + 31, the tile's rows, and columns 32 (w / 4) .. + 31 of the
// layer), add the bias, apply the GELU, round to BF16 and write them back
// into the operand buffer for the next layer.  Several CTAs share an SM, so
// one CTA's MMAs overlap the others' epilogues.
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
constexpr uint32_t kTcCols = 128;     // TMEM columns: D1 at 0..63, D2 at 64..127, D3 at 0..15
constexpr uint32_t kTcPerSm = 4;      // CTAs per SM: 4 x 128 columns = the SM's 512
constexpr uint32_t kCoreRowBytes = 1024, kCoreKBytes = 128;

__host__ __device__ constexpr uint32_t cm_off(uint32_t r, uint32_t k) {
  return (r >> 3) * kCoreRowBytes + (k >> 3) * kCoreKBytes + (r & 7u) * 16u + (k & 7u) * 2u;
}

struct SmemTc {
  uint8_t a[kTcRows * kMlpIn * 2];      // the tile: features, then activations
  uint8_t w1[kMlpHidden * kMlpIn * 2];  // B operands, [out][in]
  uint8_t w2[kMlpHidden * kMlpHidden * 2];
  uint8_t w3[16 * kMlpHidden * 2];      // outputs 8..15 zero (N = 16)
  float b1[kMlpHidden], b2[kMlpHidden], b3[kMlpOutPad];
  uint64_t mbar;
  uint32_t tmem;
  uint32_t failed;
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
#pragma unroll
    for (uint32_t c = 0; c < 4; ++c) {
      uint32_t w[4];
#pragma unroll
      for (uint32_t q = 0; q < 4; ++q) {
        const uint32_t k = c * 8 + 2 * q;
        w[q] = gelu2_bf16(v[k] + bias[h * 32 + k], v[k + 1] + bias[h * 32 + k + 1]);
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
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s.mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s.failed = 0u;
  }
  fence_async_smem();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = s.tmem;
  const uint32_t lane_base = tmem + (((warp & 3u) * 32u) << 16);  // this warp's 32 TMEM lanes
  uint32_t phase = 0;
  bool ok = true;
  auto layer = [&](uint32_t d_col, const uint8_t* w, uint32_t nout) {
    fence_async_smem();
    fence_before();
    __syncthreads();
    if (tid == 0) {
      fence_after();
      mma_layer(tmem + d_col, s.a, w, idesc_bf16(kTcRows, nout), &s.mbar);
    }
    const bool done = mbar_wait(&s.mbar, phase, kWaitLimitNs);
    phase ^= 1u;
    fence_after();
    return __syncthreads_and(done ? 1 : 0) != 0;
  };
  // a tile's features, 16-byte chunks with consecutive threads along a row:
  // this thread's chunks are loaded into registers one tile ahead, so the
  // loads of the next tile are in flight while this one computes
  constexpr uint32_t kChunks = kTcRows * 8 / kTcThreads;
  uint4 next[kChunks];
  auto fetch = [&](uint32_t tile) {
#pragma unroll
    for (uint32_t u = 0; u < kChunks; ++u) {
      const uint32_t i = tid + u * kTcThreads, grow = tile * kTcRows + (i >> 3);
      next[u] = grow < n ? *reinterpret_cast<const uint4*>(x + (size_t)grow * kMlpIn + (i & 7u) * 8)
                         : make_uint4(0u, 0u, 0u, 0u);
    }
  };
  fetch(blockIdx.x);
  for (uint32_t tile = blockIdx.x; ok && tile * kTcRows < n; tile += gridDim.x) {
#pragma unroll
    for (uint32_t u = 0; u < kChunks; ++u) {
      const uint32_t i = tid + u * kTcThreads;
      *reinterpret_cast<uint4*>(s.a + cm_off(i >> 3, (i & 7u) * 8)) = next[u];
    }
    fetch(tile + gridDim.x);
    if (!(ok = layer(0, s.w1, kMlpHidden))) break;
    hidden_epilogue(lane_base + 0, s.b1, s.a, row_in_tile, half);
    if (!(ok = layer(kMlpHidden, s.w2, kMlpHidden))) break;
    hidden_epilogue(lane_base + kMlpHidden, s.b2, s.a, row_in_tile, half);
    if (!(ok = layer(0, s.w3, 16))) break;
    const uint32_t row = tile * kTcRows + row_in_tile;
    if (half == 0) {
      float y0, y1;
      tmem_ld2(lane_base + 0, y0, y1);
      if (row < n) y[row] = make_float2(y0 + s.b3[0], y1 + s.b3[1]);
    }
    fence_before();
    __syncthreads();  // the operand buffer and TMEM are free for the next tile
    fence_after();
  }
  if (!ok) {
    // a wait gave up: report it, give the MMAs in flight one more bounded
    // wait, then free the TMEM
    if (tid == 0) atomicOr(flags, kFlagTimeout);
    mbar_wait(&s.mbar, phase, kWaitLimitNs);
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
