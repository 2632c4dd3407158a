// The learned solver surrogate: a per-particle MLP that predicts the
// position correction of the first K-1 Jacobi iterations of the extended
// solve from the particle's k nearest neighbours.
//
//   features  knn_row: the 12 nearest taking-part particles within the 3x3
//             cells around the particle -- the candidates its Jacobi
//             iterations scan (squared distance, ties by index) -- each as
//             (dx, dy, dvx, dvy) relative to the particle, then the
//             particle's own velocity; 50 values padded to 64, BF16.
//   network   64 -> 64 -> 64 -> 2 (padded to 8), GELU (tanh form) after the
//             two hidden layers (inference evaluates it on packed FP16 pairs,
//             gelu.cuh); BF16 weights, FP32 accumulation, on the
//             tensor cores with mma.sync m16n8k16 (one warp per 16 rows; the
//             accumulator fragment of one layer is the A fragment of the
//             next, so the layers chain in registers).
//   training  k_mlp_backward recomputes the forward pass of its rows and
//             accumulates the gradients of 0.5 * mean squared error into
//             FP32 buffers; k_adam updates FP32 master weights and refreshes
//             their BF16 copies.
#include <cuda_bf16.h>
#include <stdint.h>

#include "gelu.cuh"
#include "wrach_internal.cuh"
#include "wrach_kernels.h"

namespace wrach {

namespace {

constexpr uint32_t kIn = kMlpIn, kHid = kMlpHidden, kOutPad = kMlpOutPad;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, "
      "{%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// GELU in its tanh form, 0.5 x (1 + tanh(c (x + a x^3))), c = sqrt(2/pi),
// a = 0.044715 (Hendrycks & Gimpel, 2016), with the hardware tanh
// (tanh.approx.f32, relative error about 2^-11, below the BF16 rounding the
// activations then get).
constexpr float kGeluC = 0.7978845608028654f, kGeluA = 0.044715f;

__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu(float x) {
  const float t = tanh_hw(kGeluC * x * (1.0f + kGeluA * x * x));
  return 0.5f * x * (1.0f + t);
}
// d/dx: 0.5 (1 + t) + 0.5 x (1 - t^2) c (1 + 3 a x^2)
__device__ __forceinline__ float gelu_grad(float x) {
  const float x2 = x * x;
  const float t = tanh_hw(kGeluC * x * (1.0f + kGeluA * x2));
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * kGeluC * (1.0f + 3.0f * kGeluA * x2);
}

// Shared-memory copy of the network for the forward pass: the weights as
// BF16 in the [out][in] layout (the B operand, k = in contiguous) and the
// biases in FP32.  Each row of 64 BF16 (32 words) is padded to kRow = 36
// words, so that the B-fragment loads of a warp (rows g = 0..7, words t =
// 0..3) fall in 32 distinct banks: (36 g + t) mod 32 = 4 g + t.
constexpr uint32_t kRow = kIn / 2 + 4;
static_assert(kIn == kHid, "one padded row length serves every layer");
struct SmemNet {
  uint32_t w1t[kHid * kRow], w2t[kHid * kRow], w3t[kOutPad * kRow];
  float b1[kHid], b2[kHid], b3[kOutPad];
};
// The [in][out] copies the backward pass multiplies the gradients by.
struct SmemNetT {
  uint32_t w1[kIn * kRow], w2[kHid * kRow], w3[kHid * kOutPad / 2];
};

// rows x 32 words from a packed global array into padded shared rows
__device__ __forceinline__ void load_rows(uint32_t* dst, const uint16_t* src, uint32_t rows) {
  const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
  for (uint32_t i = threadIdx.x; i < rows * (kIn / 2); i += blockDim.x)
    dst[(i / (kIn / 2)) * kRow + i % (kIn / 2)] = s[i];
}

__device__ void load_net(const MlpDev& m, SmemNet& s, SmemNetT* st) {
  load_rows(s.w1t, m.w1t, kHid);
  load_rows(s.w2t, m.w2t, kHid);
  load_rows(s.w3t, m.w3t, kOutPad);
  if (st) {
    load_rows(st->w1, m.w1, kIn);
    load_rows(st->w2, m.w2, kHid);
    for (uint32_t i = threadIdx.x; i < kHid * kOutPad / 2; i += blockDim.x)
      st->w3[i] = reinterpret_cast<const uint32_t*>(m.w3)[i];
  }
  for (uint32_t i = threadIdx.x; i < kHid; i += blockDim.x) {
    s.b1[i] = m.b1[i];
    s.b2[i] = m.b2[i];
  }
  for (uint32_t i = threadIdx.x; i < kOutPad; i += blockDim.x) s.b3[i] = m.b3[i];
  __syncthreads();
}

// B fragment of a weight matrix stored [n][k] in padded rows: k-tile kk,
// n-tile nt.
__device__ __forceinline__ void bfrag(const uint32_t* wt, uint32_t kk, uint32_t nt,
                                      uint32_t lane, uint32_t& b0, uint32_t& b1) {
  const uint32_t g = lane >> 2, t = lane & 3;
  const uint32_t row = (nt * 8 + g) * kRow;
  b0 = wt[row + kk * 8 + t];
  b1 = wt[row + kk * 8 + 4 + t];
}

// Forward pass of one 16-row tile held by a warp.  `ax` is the A fragment of
// the input (4 k-tiles).  Writes the pre-activations z1, z2 (C layout, 8
// n-tiles), the A fragments h1, h2 of the activations and the output y
// (one n-tile).
__device__ __forceinline__ void mlp_tile_forward(const SmemNet& s, uint32_t lane,
                                                 const uint32_t (&ax)[4][4],
                                                 float (&z1)[8][4], uint32_t (&h1)[4][4],
                                                 float (&z2)[8][4], uint32_t (&h2)[4][4],
                                                 float (&y)[4]) {
  const uint32_t t = lane & 3;
#pragma unroll
  for (uint32_t nt = 0; nt < 8; ++nt) {
    const float bl = s.b1[nt * 8 + 2 * t], bh = s.b1[nt * 8 + 2 * t + 1];
    z1[nt][0] = bl; z1[nt][1] = bh; z1[nt][2] = bl; z1[nt][3] = bh;
#pragma unroll
    for (uint32_t kk = 0; kk < 4; ++kk) {
      uint32_t b0, b1;
      bfrag(s.w1t, kk, nt, lane, b0, b1);
      mma_bf16(z1[nt], ax[kk], b0, b1);
    }
  }
#pragma unroll
  for (uint32_t kk = 0; kk < 4; ++kk) {
    h1[kk][0] = pack_bf16(gelu(z1[2 * kk][0]), gelu(z1[2 * kk][1]));
    h1[kk][1] = pack_bf16(gelu(z1[2 * kk][2]), gelu(z1[2 * kk][3]));
    h1[kk][2] = pack_bf16(gelu(z1[2 * kk + 1][0]), gelu(z1[2 * kk + 1][1]));
    h1[kk][3] = pack_bf16(gelu(z1[2 * kk + 1][2]), gelu(z1[2 * kk + 1][3]));
  }
#pragma unroll
  for (uint32_t nt = 0; nt < 8; ++nt) {
    const float bl = s.b2[nt * 8 + 2 * t], bh = s.b2[nt * 8 + 2 * t + 1];
    z2[nt][0] = bl; z2[nt][1] = bh; z2[nt][2] = bl; z2[nt][3] = bh;
#pragma unroll
    for (uint32_t kk = 0; kk < 4; ++kk) {
      uint32_t b0, b1;
      bfrag(s.w2t, kk, nt, lane, b0, b1);
      mma_bf16(z2[nt], h1[kk], b0, b1);
    }
  }
#pragma unroll
  for (uint32_t kk = 0; kk < 4; ++kk) {
    h2[kk][0] = pack_bf16(gelu(z2[2 * kk][0]), gelu(z2[2 * kk][1]));
    h2[kk][1] = pack_bf16(gelu(z2[2 * kk][2]), gelu(z2[2 * kk][3]));
    h2[kk][2] = pack_bf16(gelu(z2[2 * kk + 1][0]), gelu(z2[2 * kk + 1][1]));
    h2[kk][3] = pack_bf16(gelu(z2[2 * kk + 1][2]), gelu(z2[2 * kk + 1][3]));
  }
  {
    const float bl = s.b3[2 * t], bh = s.b3[2 * t + 1];
    y[0] = bl; y[1] = bh; y[2] = bl; y[3] = bh;
#pragma unroll
    for (uint32_t kk = 0; kk < 4; ++kk) {
      uint32_t b0, b1;
      bfrag(s.w3t, kk, 0, lane, b0, b1);
      mma_bf16(y, h2[kk], b0, b1);
    }
  }
}

// A shared-memory word read that the compiler keeps in place (it would
// otherwise hoist the loop-invariant weight fragments of a persistent loop
// into registers and lose occupancy).
__device__ __forceinline__ uint32_t lds_keep(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.shared.b32 %0, [%1];"
               : "=r"(v)
               : "r"((uint32_t)__cvta_generic_to_shared(p)));
  return v;
}

// The forward pass of a 16-row tile for inference only: the same products in
// the same order as mlp_tile_forward, computed two n-tiles at a time so that
// no pre-activation array stays live, with the GELU on packed FP16 pairs
// (gelu2_bf16; the training pass keeps the FP32 GELU and its derivative).
__device__ __forceinline__ void mlp_tile_infer(const SmemNet& s, uint32_t lane,
                                               const uint32_t (&ax)[4][4], float (&y)[4]) {
  const uint32_t g = lane >> 2, t = lane & 3;
  uint32_t h1[4][4], h2[4][4];
#pragma unroll
  for (uint32_t kq = 0; kq < 4; ++kq) {
    float z[2][4];
#pragma unroll
    for (uint32_t u = 0; u < 2; ++u) {
      const uint32_t nt = 2 * kq + u;
      const float bl = s.b1[nt * 8 + 2 * t], bh = s.b1[nt * 8 + 2 * t + 1];
      z[u][0] = bl; z[u][1] = bh; z[u][2] = bl; z[u][3] = bh;
      const uint32_t* row = s.w1t + (nt * 8 + g) * kRow + t;
#pragma unroll
      for (uint32_t kk = 0; kk < 4; ++kk)
        mma_bf16(z[u], ax[kk], lds_keep(row + kk * 8), lds_keep(row + kk * 8 + 4));
    }
    h1[kq][0] = gelu2_bf16(z[0][0], z[0][1]);
    h1[kq][1] = gelu2_bf16(z[0][2], z[0][3]);
    h1[kq][2] = gelu2_bf16(z[1][0], z[1][1]);
    h1[kq][3] = gelu2_bf16(z[1][2], z[1][3]);
  }
#pragma unroll
  for (uint32_t kq = 0; kq < 4; ++kq) {
    float z[2][4];
#pragma unroll
    for (uint32_t u = 0; u < 2; ++u) {
      const uint32_t nt = 2 * kq + u;
      const float bl = s.b2[nt * 8 + 2 * t], bh = s.b2[nt * 8 + 2 * t + 1];
      z[u][0] = bl; z[u][1] = bh; z[u][2] = bl; z[u][3] = bh;
      const uint32_t* row = s.w2t + (nt * 8 + g) * kRow + t;
#pragma unroll
      for (uint32_t kk = 0; kk < 4; ++kk)
        mma_bf16(z[u], h1[kk], lds_keep(row + kk * 8), lds_keep(row + kk * 8 + 4));
    }
    h2[kq][0] = gelu2_bf16(z[0][0], z[0][1]);
    h2[kq][1] = gelu2_bf16(z[0][2], z[0][3]);
    h2[kq][2] = gelu2_bf16(z[1][0], z[1][1]);
    h2[kq][3] = gelu2_bf16(z[1][2], z[1][3]);
  }
  const float bl = s.b3[2 * t], bh = s.b3[2 * t + 1];
  y[0] = bl; y[1] = bh; y[2] = bl; y[3] = bh;
  const uint32_t* row = s.w3t + g * kRow + t;
#pragma unroll
  for (uint32_t kk = 0; kk < 4; ++kk)
    mma_bf16(y, h2[kk], lds_keep(row + kk * 8), lds_keep(row + kk * 8 + 4));
}

// A fragment (4 k-tiles) of 16 rows of X (BF16 [rows][64]); rows past n read
// as zero.
__device__ __forceinline__ void load_x_tile(const uint16_t* x, uint32_t row0, uint32_t n,
                                            uint32_t lane, uint32_t (&ax)[4][4]) {
  const uint32_t g = lane >> 2, t = lane & 3;
  const uint32_t r0 = row0 + g, r1 = row0 + g + 8;
  const uint32_t* p0 = reinterpret_cast<const uint32_t*>(x + (size_t)r0 * kIn);
  const uint32_t* p1 = reinterpret_cast<const uint32_t*>(x + (size_t)r1 * kIn);
#pragma unroll
  for (uint32_t kk = 0; kk < 4; ++kk) {
    ax[kk][0] = r0 < n ? p0[kk * 8 + t] : 0u;
    ax[kk][1] = r1 < n ? p1[kk * 8 + t] : 0u;
    ax[kk][2] = r0 < n ? p0[kk * 8 + 4 + t] : 0u;
    ax[kk][3] = r1 < n ? p1[kk * 8 + 4 + t] : 0u;
  }
}

__global__ void __launch_bounds__(128) k_mlp_forward(MlpDev m, const uint16_t* __restrict__ x,
                                                     uint32_t n, float2* __restrict__ y) {
  __shared__ SmemNet s;
  load_net(m, s, nullptr);
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t g = lane >> 2, t = lane & 3;
  const uint32_t tiles = (n + 15) / 16;
  for (uint32_t tile = blockIdx.x * 4 + warp; tile < tiles; tile += gridDim.x * 4) {
    uint32_t ax[4][4];
    float out[4];
    load_x_tile(x, tile * 16, n, lane, ax);
    mlp_tile_infer(s, lane, ax, out);
    if (t == 0) {
      const uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
      if (r0 < n) y[r0] = make_float2(out[0], out[1]);
      if (r1 < n) y[r1] = make_float2(out[2], out[3]);
    }
  }
}

// Per-warp scratch of the backward pass: activations and gradients of one
// tile stored transposed ([feature][row], rows contiguous) as BF16 pairs, the
// A operand layout of the weight-gradient products X^T dZ1, H1^T dZ2, H2^T dY.
struct SmemBack {
  uint16_t xt[kIn][16], h1t[kHid][16], h2t[kHid][16];
  uint16_t dz1t[kHid][16], dz2t[kHid][16], dyt[kOutPad][16];
};

// Accumulators of the block: FP32 gradients, in the parameter order.
struct SmemGrad {
  float w1[kIn * kHid], b1[kHid], w2[kHid * kHid], b2[kHid], w3[kHid * kOutPad], b3[kOutPad];
};
static_assert(sizeof(SmemGrad) == kMlpParams * sizeof(float), "gradient order = parameters");

__device__ __forceinline__ uint16_t bf16_bits(float v) {
  __nv_bfloat16 b = __float2bfloat16_rn(v);
  return *reinterpret_cast<uint16_t*>(&b);
}

// Scatter a C-layout tile (8 n-tiles of 16x8) into a transposed BF16 array.
__device__ __forceinline__ void store_ct(uint16_t (*dst)[16], const float (&c)[8][4],
                                         uint32_t lane) {
  const uint32_t g = lane >> 2, t = lane & 3;
#pragma unroll
  for (uint32_t nt = 0; nt < 8; ++nt) {
    const uint32_t col = nt * 8 + 2 * t;
    dst[col][g] = bf16_bits(c[nt][0]);
    dst[col + 1][g] = bf16_bits(c[nt][1]);
    dst[col][g + 8] = bf16_bits(c[nt][2]);
    dst[col + 1][g + 8] = bf16_bits(c[nt][3]);
  }
}

// Scatter an A-layout BF16 tile (4 k-tiles) into a transposed array.
__device__ __forceinline__ void store_at(uint16_t (*dst)[16], const uint32_t (&a)[4][4],
                                         uint32_t lane) {
  const uint32_t g = lane >> 2, t = lane & 3;
#pragma unroll
  for (uint32_t kk = 0; kk < 4; ++kk) {
    const uint32_t c0 = kk * 16 + 2 * t, c1 = c0 + 8;
    dst[c0][g] = (uint16_t)(a[kk][0] & 0xFFFF);
    dst[c0 + 1][g] = (uint16_t)(a[kk][0] >> 16);
    dst[c0][g + 8] = (uint16_t)(a[kk][1] & 0xFFFF);
    dst[c0 + 1][g + 8] = (uint16_t)(a[kk][1] >> 16);
    dst[c1][g] = (uint16_t)(a[kk][2] & 0xFFFF);
    dst[c1 + 1][g] = (uint16_t)(a[kk][2] >> 16);
    dst[c1][g + 8] = (uint16_t)(a[kk][3] & 0xFFFF);
    dst[c1 + 1][g + 8] = (uint16_t)(a[kk][3] >> 16);
  }
}

// dW[m][n] += sum over the 16 rows of AT[m][row] * BT[n][row] for m in
// [0, mdim), n in [0, ndim): the tile's weight-gradient product on the
// tensor cores (K = 16 rows), added into the block's FP32 accumulator.
__device__ __forceinline__ void grad_product(const uint16_t (*at)[16], uint32_t mdim,
                                             const uint16_t (*bt)[16], uint32_t ndim,
                                             float* acc, uint32_t lane) {
  const uint32_t g = lane >> 2, t = lane & 3;
  for (uint32_t mt = 0; mt < mdim / 16; ++mt) {
    uint32_t a[4];
    a[0] = *reinterpret_cast<const uint32_t*>(&at[mt * 16 + g][2 * t]);
    a[1] = *reinterpret_cast<const uint32_t*>(&at[mt * 16 + g + 8][2 * t]);
    a[2] = *reinterpret_cast<const uint32_t*>(&at[mt * 16 + g][2 * t + 8]);
    a[3] = *reinterpret_cast<const uint32_t*>(&at[mt * 16 + g + 8][2 * t + 8]);
    for (uint32_t nt = 0; nt < ndim / 8; ++nt) {
      const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&bt[nt * 8 + g][2 * t]);
      const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&bt[nt * 8 + g][2 * t + 8]);
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      mma_bf16(d, a, b0, b1);
      const uint32_t m0 = mt * 16 + g, n0 = nt * 8 + 2 * t;
      atomicAdd(&acc[m0 * ndim + n0], d[0]);
      atomicAdd(&acc[m0 * ndim + n0 + 1], d[1]);
      atomicAdd(&acc[(m0 + 8) * ndim + n0], d[2]);
      atomicAdd(&acc[(m0 + 8) * ndim + n0 + 1], d[3]);
    }
  }
}

// Gradients of L = 0.5 * sum over rows and the 2 outputs of (y - target)^2 /
// `scale_rows` with respect to every parameter, added into `grad` (FP32,
// the MlpDev parameter order: w1 [in][out], b1, w2, b2, w3 [in][8], b3).
// Also adds the loss into *loss.
__global__ void __launch_bounds__(128) k_mlp_backward(MlpDev m, const uint16_t* __restrict__ x,
                                                      const float2* __restrict__ target,
                                                      uint32_t n, float inv_rows,
                                                      float* __restrict__ grad,
                                                      float* __restrict__ loss) {
  extern __shared__ __align__(16) uint8_t dyn[];
  SmemNet& s = *reinterpret_cast<SmemNet*>(dyn);
  SmemNetT& st = *reinterpret_cast<SmemNetT*>(dyn + sizeof(SmemNet));
  SmemGrad& acc = *reinterpret_cast<SmemGrad*>(dyn + sizeof(SmemNet) + sizeof(SmemNetT));
  SmemBack* back =
      reinterpret_cast<SmemBack*>(dyn + sizeof(SmemNet) + sizeof(SmemNetT) + sizeof(SmemGrad));
  load_net(m, s, &st);
  float* accf = reinterpret_cast<float*>(&acc);
  for (uint32_t i = threadIdx.x; i < sizeof(SmemGrad) / 4; i += blockDim.x) accf[i] = 0.f;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t g = lane >> 2, t = lane & 3;
  SmemBack& sb = back[warp];
  float lsum = 0.f;
  const uint32_t tiles = (n + 15) / 16;
  for (uint32_t tile = blockIdx.x * 4 + warp; tile < tiles; tile += gridDim.x * 4) {
    uint32_t ax[4][4], h1[4][4], h2[4][4];
    float z1[8][4], z2[8][4], y[4];
    load_x_tile(x, tile * 16, n, lane, ax);
    mlp_tile_forward(s, lane, ax, z1, h1, z2, h2, y);
    // dY (C layout, one n-tile; only columns 0 and 1 are real outputs)
    const uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
    float dy[4] = {0.f, 0.f, 0.f, 0.f};
    if (t == 0) {
      if (r0 < n) {
        const float2 tg = target[r0];
        const float e0 = y[0] - tg.x, e1 = y[1] - tg.y;
        lsum += 0.5f * (e0 * e0 + e1 * e1);
        dy[0] = e0 * inv_rows;
        dy[1] = e1 * inv_rows;
      }
      if (r1 < n) {
        const float2 tg = target[r1];
        const float e0 = y[2] - tg.x, e1 = y[3] - tg.y;
        lsum += 0.5f * (e0 * e0 + e1 * e1);
        dy[2] = e0 * inv_rows;
        dy[3] = e1 * inv_rows;
      }
    }
    // dH2 = dY W3^T  (K = 8 outputs padded to 16 with zeros)
    uint32_t ady[4];
    ady[0] = pack_bf16(dy[0], dy[1]);
    ady[1] = pack_bf16(dy[2], dy[3]);
    ady[2] = 0u;
    ady[3] = 0u;
    float dz2[8][4];
#pragma unroll
    for (uint32_t nt = 0; nt < 8; ++nt) {
      dz2[nt][0] = dz2[nt][1] = dz2[nt][2] = dz2[nt][3] = 0.f;
      // B(k = out, n = in) = W3[in][out]; W3 stored [in][8]
      const uint32_t b0 = st.w3[(nt * 8 + g) * (kOutPad / 2) + t];
      mma_bf16(dz2[nt], ady, b0, 0u);
    }
#pragma unroll
    for (uint32_t nt = 0; nt < 8; ++nt)
#pragma unroll
      for (uint32_t q = 0; q < 4; ++q) dz2[nt][q] *= gelu_grad(z2[nt][q]);
    // dH1 = dZ2 W2^T
    uint32_t adz2[4][4];
#pragma unroll
    for (uint32_t kk = 0; kk < 4; ++kk) {
      adz2[kk][0] = pack_bf16(dz2[2 * kk][0], dz2[2 * kk][1]);
      adz2[kk][1] = pack_bf16(dz2[2 * kk][2], dz2[2 * kk][3]);
      adz2[kk][2] = pack_bf16(dz2[2 * kk + 1][0], dz2[2 * kk + 1][1]);
      adz2[kk][3] = pack_bf16(dz2[2 * kk + 1][2], dz2[2 * kk + 1][3]);
    }
    float dz1[8][4];
#pragma unroll
    for (uint32_t nt = 0; nt < 8; ++nt) {
      dz1[nt][0] = dz1[nt][1] = dz1[nt][2] = dz1[nt][3] = 0.f;
#pragma unroll
      for (uint32_t kk = 0; kk < 4; ++kk) {
        uint32_t b0, b1;
        bfrag(st.w2, kk, nt, lane, b0, b1);  // W2 [in][out]: B(k=out, n=in)
        mma_bf16(dz1[nt], adz2[kk], b0, b1);
      }
    }
#pragma unroll
    for (uint32_t nt = 0; nt < 8; ++nt)
#pragma unroll
      for (uint32_t q = 0; q < 4; ++q) dz1[nt][q] *= gelu_grad(z1[nt][q]);

    // bias gradients: column sums over the tile's rows
#pragma unroll
    for (uint32_t nt = 0; nt < 8; ++nt) {
      float s2a = dz2[nt][0] + dz2[nt][2], s2b = dz2[nt][1] + dz2[nt][3];
      float s1a = dz1[nt][0] + dz1[nt][2], s1b = dz1[nt][1] + dz1[nt][3];
#pragma unroll
      for (uint32_t o = 4; o < 32; o <<= 1) {
        s2a += __shfl_xor_sync(0xffffffffu, s2a, o);
        s2b += __shfl_xor_sync(0xffffffffu, s2b, o);
        s1a += __shfl_xor_sync(0xffffffffu, s1a, o);
        s1b += __shfl_xor_sync(0xffffffffu, s1b, o);
      }
      if (g == 0) {
        atomicAdd(&acc.b2[nt * 8 + 2 * t], s2a);
        atomicAdd(&acc.b2[nt * 8 + 2 * t + 1], s2b);
        atomicAdd(&acc.b1[nt * 8 + 2 * t], s1a);
        atomicAdd(&acc.b1[nt * 8 + 2 * t + 1], s1b);
      }
    }
    {
      float a0 = dy[0] + dy[2], a1 = dy[1] + dy[3];
#pragma unroll
      for (uint32_t o = 4; o < 32; o <<= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      }
      if (g == 0 && t == 0) {
        atomicAdd(&acc.b3[0], a0);
        atomicAdd(&acc.b3[1], a1);
      }
    }
    // weight gradients: X^T dZ1, H1^T dZ2, H2^T dY (K = the tile's 16 rows)
    store_at(sb.xt, ax, lane);
    store_at(sb.h1t, h1, lane);
    store_at(sb.h2t, h2, lane);
    store_ct(sb.dz1t, dz1, lane);
    store_ct(sb.dz2t, dz2, lane);
    {
      // dY transposed: 8 output columns x 16 rows
      for (uint32_t c = 0; c < kOutPad; ++c) {
        sb.dyt[c][g] = 0;
        sb.dyt[c][g + 8] = 0;
      }
      __syncwarp();
      if (t == 0) {
        sb.dyt[0][g] = bf16_bits(dy[0]);
        sb.dyt[1][g] = bf16_bits(dy[1]);
        sb.dyt[0][g + 8] = bf16_bits(dy[2]);
        sb.dyt[1][g + 8] = bf16_bits(dy[3]);
      }
    }
    __syncwarp();
    grad_product(sb.xt, kIn, sb.dz1t, kHid, acc.w1, lane);
    grad_product(sb.h1t, kHid, sb.dz2t, kHid, acc.w2, lane);
    grad_product(sb.h2t, kHid, sb.dyt, kOutPad, acc.w3, lane);
    __syncwarp();
  }
  // the tile losses of the warp, then the block's gradients into global
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0 && lsum != 0.f) atomicAdd(loss, lsum * inv_rows);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < sizeof(SmemGrad) / 4; i += blockDim.x)
    if (accf[i] != 0.f) atomicAdd(&grad[i], accf[i]);
}

size_t backward_smem() {
  return sizeof(SmemNet) + sizeof(SmemNetT) + sizeof(SmemGrad) + 4 * sizeof(SmemBack);
}

// Adam on the FP32 master parameters (the SmemGrad order), then the BF16
// copies in both layouts.
__global__ void k_adam(MlpDev m, const float* __restrict__ grad, float* __restrict__ mom1,
                       float* __restrict__ mom2, float lr, float b1, float b2, float eps,
                       float bc1, float bc2, uint32_t nparams) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nparams) return;
  const float gr = grad[i];
  const float a = b1 * mom1[i] + (1.f - b1) * gr;
  const float b = b2 * mom2[i] + (1.f - b2) * gr * gr;
  mom1[i] = a;
  mom2[i] = b;
  const float step = lr * (a / bc1) / (sqrtf(b / bc2) + eps);
  float* p = m.params;
  const float v = p[i] - step;
  p[i] = v;
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  // parameter order: w1 [in][hid], b1, w2 [hid][hid], b2, w3 [hid][8], b3
  const uint32_t o_b1 = kIn * kHid, o_w2 = o_b1 + kHid, o_b2 = o_w2 + kHid * kHid;
  const uint32_t o_w3 = o_b2 + kHid, o_b3 = o_w3 + kHid * kOutPad;
  __nv_bfloat16* w1 = reinterpret_cast<__nv_bfloat16*>(m.w1);
  __nv_bfloat16* w1t = reinterpret_cast<__nv_bfloat16*>(m.w1t);
  __nv_bfloat16* w2 = reinterpret_cast<__nv_bfloat16*>(m.w2);
  __nv_bfloat16* w2t = reinterpret_cast<__nv_bfloat16*>(m.w2t);
  __nv_bfloat16* w3 = reinterpret_cast<__nv_bfloat16*>(m.w3);
  __nv_bfloat16* w3t = reinterpret_cast<__nv_bfloat16*>(m.w3t);
  if (i < o_b1) {
    const uint32_t r = i / kHid, c = i % kHid;  // in, out
    w1[i] = h;
    w1t[c * kIn + r] = h;
  } else if (i < o_w2) {
    m.b1[i - o_b1] = v;
  } else if (i < o_b2) {
    const uint32_t j = i - o_w2, r = j / kHid, c = j % kHid;
    w2[j] = h;
    w2t[c * kHid + r] = h;
  } else if (i < o_w3) {
    m.b2[i - o_b2] = v;
  } else if (i < o_b3) {
    const uint32_t j = i - o_w3, r = j / kOutPad, c = j % kOutPad;
    w3[j] = h;
    w3t[c * kHid + r] = h;
  } else {
    m.b3[i - o_b3] = v;
  }
}

// ---------------------------------------------------------------------------
// Features
// ---------------------------------------------------------------------------

constexpr uint32_t kK = kKnn;

// Features of the taking-part particle of compacted index t (cell c) into
// `row` (32 words, global or shared memory): the 12 nearest taking-part
// particles in the 3x3 cells around its cell -- the candidates of its Jacobi
// iterations, one contiguous compacted range per neighbour row -- by binary32
// squared distance (each product and sum rounded on its own), ties by index;
// each as (dx, dy, dvx, dvy) relative to the particle; then the own
// velocity; zero padding to 64.  Positions and velocities are the frame's
// binned state, compacted (tpp, tpv).
__device__ __forceinline__ void knn_row(const WorldDev& w, const uint32_t* __restrict__ ct,
                                        const float2* __restrict__ tpp,
                                        const float2* __restrict__ tpv, uint32_t c, uint32_t t,
                                        uint32_t* row) {
  uint32_t cx, cy;
  cell_xy(w, c - w.cell_off, cx, cy);
  const uint32_t x0 = cx > 0 ? cx - 1 : 0;
  const uint32_t x1 = cx + 1 < w.gx ? cx + 1 : w.gx - 1;
  uint32_t rs[3], re[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const int ny = (int)cy - 1 + r;
    const bool ok = ny >= 0 && ny < (int)w.gy;
    const uint32_t rb = w.cell_off + (uint32_t)(ok ? ny : 0) * w.gx;
    rs[r] = ok ? ct[rb + x0] : 0u;
    re[r] = ok ? ct[rb + x1 + 1] : 0u;
  }
  const float2 pi = tpp[t], vi = tpv[t];
  float bd[kK];
  uint32_t bj[kK];
#pragma unroll
  for (uint32_t k = 0; k < kK; ++k) {
    bd[k] = INFINITY;
    bj[k] = 0xFFFFFFFFu;
  }
  // the candidates come in ascending index order (rows bottom-up, compacted
  // order inside a row), so a tie in distance keeps the one already listed;
  // each is inserted into the ascending list: every comparison against the
  // old list first, then the shift
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    for (uint32_t j = rs[r]; j < re[r]; ++j) {
      if (j == t) continue;
      const float2 pj = tpp[j];
      const float dx = __fsub_rn(pj.x, pi.x), dy = __fsub_rn(pj.y, pi.y);
      const float d = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
      if (!(d < bd[kK - 1])) continue;
      bool lt[kK];
#pragma unroll
      for (uint32_t k = 0; k < kK; ++k) lt[k] = d < bd[k];
#pragma unroll
      for (uint32_t k = kK - 1; k > 0; --k) {
        bd[k] = lt[k - 1] ? bd[k - 1] : (lt[k] ? d : bd[k]);
        bj[k] = lt[k - 1] ? bj[k - 1] : (lt[k] ? j : bj[k]);
      }
      bd[0] = lt[0] ? d : bd[0];
      bj[0] = lt[0] ? j : bj[0];
    }
  }
#pragma unroll
  for (uint32_t k = 0; k < kK; ++k) {
    if (bj[k] != 0xFFFFFFFFu) {
      const float2 pj = tpp[bj[k]], vj = tpv[bj[k]];
      row[2 * k] = pack_bf16(__fsub_rn(pj.x, pi.x), __fsub_rn(pj.y, pi.y));
      row[2 * k + 1] = pack_bf16(__fsub_rn(vj.x, vi.x), __fsub_rn(vj.y, vi.y));
    } else {
      row[2 * k] = 0u;
      row[2 * k + 1] = 0u;
    }
  }
  row[2 * kK] = pack_bf16(vi.x, vi.y);
#pragma unroll
  for (uint32_t k = 2 * kK + 1; k < kIn / 2; ++k) row[k] = 0u;
}

__device__ __forceinline__ void zero_row(uint32_t* row) {
#pragma unroll
  for (uint32_t k = 0; k < kIn / 2; ++k) row[k] = 0u;
}

// Features of the binned frame into x (BF16 [n][64]), one thread per frame
// particle; a particle that does not take part (past the capacity of its
// cell) gets all zeros.
__global__ void __launch_bounds__(256)
k_knn_features(const WorldDev* __restrict__ worlds, int nworlds, PhysDev ph, uint32_t n,
               const uint32_t* __restrict__ cell_start, const uint32_t* __restrict__ ct,
               const uint32_t* __restrict__ cell_of, const float2* __restrict__ tpp,
               const float2* __restrict__ tpv, uint16_t* __restrict__ x) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t* row = reinterpret_cast<uint32_t*>(x + (size_t)i * kIn);
  const uint32_t c = cell_of[i];
  const uint32_t t = tp_index(cell_start, ct, c, i, ph.cap);
  if (t == 0xFFFFFFFFu) {
    zero_row(row);
    return;
  }
  knn_row(worlds[world_of_cell(worlds, nworlds, c)], ct, tpp, tpv, c, t, row);
}

// Training samples of the binned frame: the features of the taking-part
// particles t = phase + k * stride, k = 0, 1, ..., into rows k of x (at most
// `rows`), and their targets q_t - p_t from the compacted iterate q (the
// plain solver's first iterations) into target.
__global__ void __launch_bounds__(256)
k_samples(const WorldDev* __restrict__ worlds, int nworlds, uint32_t ncells,
          const uint32_t* __restrict__ ct, const uint32_t* __restrict__ tp_cell,
          const float2* __restrict__ tpp, const float2* __restrict__ tpv,
          const float2* __restrict__ q, uint32_t stride, uint32_t phase, uint32_t rows,
          uint16_t* __restrict__ x, float2* __restrict__ target) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t t = phase + k * stride;
  if (k >= rows || t >= __ldg(ct + ncells)) return;
  const uint32_t c = tp_cell[t];
  knn_row(worlds[world_of_cell(worlds, nworlds, c)], ct, tpp, tpv, c, t,
          reinterpret_cast<uint32_t*>(x + (size_t)k * kIn));
  const float2 p = tpp[t], v = q[t];
  target[k] = make_float2(v.x - p.x, v.y - p.y);
}

// The surrogate correction of a frame in one pass over its taking-part
// particles (compacted): per tile of 256 of them, the features go to shared
// memory (padded rows, so the A-fragment loads are conflict-free like the
// weights'), each warp runs the network on 32 of the rows, and the
// correction is applied on the spot: the compacted iterate q_t = p_t +
// correction.  `corr` (optional) receives the correction at the frame index
// of each taking-part particle.  Persistent: the network is loaded once per
// block.
constexpr uint32_t kFuseThreads = 256;

__global__ void __launch_bounds__(kFuseThreads, 3)
k_surrogate_correct(MlpDev m, const WorldDev* __restrict__ worlds, int nworlds,
                    uint32_t ncells, const uint32_t* __restrict__ cell_start,
                    const uint32_t* __restrict__ ct, const uint32_t* __restrict__ tp_cell,
                    const float2* __restrict__ tpp, const float2* __restrict__ tpv,
                    float2* __restrict__ q, float2* __restrict__ corr) {
  extern __shared__ __align__(16) uint8_t dyn[];
  SmemNet& s = *reinterpret_cast<SmemNet*>(dyn);
  uint32_t* sx = reinterpret_cast<uint32_t*>(dyn + sizeof(SmemNet));  // [256][kRow]
  load_net(m, s, nullptr);
  const uint32_t ntp = __ldg(ct + ncells);
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t g = lane >> 2, t4 = lane & 3;
  for (uint32_t base = blockIdx.x * kFuseThreads; base < ntp; base += gridDim.x * kFuseThreads) {
    const uint32_t t = base + threadIdx.x;
    uint32_t* row = sx + threadIdx.x * kRow;
    if (t < ntp) {
      const uint32_t c = tp_cell[t];
      knn_row(worlds[world_of_cell(worlds, nworlds, c)], ct, tpp, tpv, c, t, row);
    } else {
      zero_row(row);
    }
    __syncthreads();
#pragma unroll 1
    for (uint32_t rt = 0; rt < 2; ++rt) {
      const uint32_t r0 = warp * 32 + rt * 16;
      uint32_t ax[4][4];
      float out[4];
      const uint32_t* p0 = sx + (r0 + g) * kRow;
      const uint32_t* p1 = sx + (r0 + g + 8) * kRow;
#pragma unroll
      for (uint32_t kk = 0; kk < 4; ++kk) {
        ax[kk][0] = p0[kk * 8 + t4];
        ax[kk][1] = p1[kk * 8 + t4];
        ax[kk][2] = p0[kk * 8 + 4 + t4];
        ax[kk][3] = p1[kk * 8 + 4 + t4];
      }
      mlp_tile_infer(s, lane, ax, out);
      if (t4 == 0) {
#pragma unroll
        for (uint32_t h = 0; h < 2; ++h) {
          const uint32_t idx = base + r0 + g + 8 * h;
          if (idx < ntp) {
            const float cxv = out[2 * h], cyv = out[2 * h + 1];
            const float2 p = tpp[idx];
            q[idx] = make_float2(__fadd_rn(p.x, cxv), __fadd_rn(p.y, cyv));
            if (corr) {
              const uint32_t c = tp_cell[idx];
              corr[cell_start[c] + (idx - ct[c])] = make_float2(cxv, cyv);
            }
          }
        }
      }
    }
    __syncthreads();
  }
}

size_t correct_smem() { return sizeof(SmemNet) + (size_t)kFuseThreads * kRow * 4; }

// target = q - p, the first K-1 iterations' correction of frame particle i
// (q compacted: zero for a particle that takes no part)
__global__ void k_target(uint32_t n, PhysDev ph, const uint32_t* __restrict__ cell_start,
                         const uint32_t* __restrict__ ct, const uint32_t* __restrict__ cell_of,
                         const float2* __restrict__ pos, const float2* __restrict__ q,
                         float2* __restrict__ target) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t t = tp_index(cell_start, ct, cell_of[i], i, ph.cap);
  if (t == 0xFFFFFFFFu) {
    target[i] = make_float2(0.f, 0.f);
    return;
  }
  const float2 p = pos[i], v = q[t];
  target[i] = make_float2(v.x - p.x, v.y - p.y);
}

// Sums of a block: 5 values per thread (sum, max, sum, sum, sum order in
// `v`), reduced over the block and written to part[blockIdx.x * 8 + k].
__device__ __forceinline__ void block_partials(float (&v)[5], float* __restrict__ part) {
  __shared__ float red[32][5];
#pragma unroll
  for (uint32_t o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const float u = __shfl_xor_sync(0xffffffffu, v[k], o);
      v[k] = k == 1 ? fmaxf(v[k], u) : v[k] + u;
    }
  }
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 5; ++k) red[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x < 5) {
    float acc = red[0][threadIdx.x];
    for (uint32_t w = 1; w < nw; ++w)
      acc = threadIdx.x == 1 ? fmaxf(acc, red[w][threadIdx.x]) : acc + red[w][threadIdx.x];
    part[blockIdx.x * 8 + threadIdx.x] = acc;
  }
}

// Frame metrics (report only): per taking-part particle the deepest overlap
// with a taking-part neighbour of the 3x3 cells, max(0, max_j (min_d -
// |p_j - p_i|)); per block: [0] sum of overlaps, [1] max overlap, [2] number
// of taking-part particles, [3] kinetic energy, [4] 0.
__global__ void __launch_bounds__(256)
k_penetration(const WorldDev* __restrict__ worlds, int nworlds, PhysDev ph, uint32_t n,
              const uint32_t* __restrict__ cell_start, const uint32_t* __restrict__ cell_of,
              const float2* __restrict__ pos, const float2* __restrict__ vel,
              float* __restrict__ part) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float pen = 0.f, ke = 0.f, cnt = 0.f;
  if (i < n) {
    const float2 v = vel[i];
    ke = __fmul_rn(0.5f, __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y)));
    const uint32_t c = cell_of[i];
    if (i - cell_start[c] < ph.cap) {
      cnt = 1.f;
      const WorldDev w = worlds[world_of_cell(worlds, nworlds, c)];
      uint32_t cx, cy;
      cell_xy(w, c - w.cell_off, cx, cy);
      const float2 pi = pos[i];
      const int y0 = max((int)cy - 1, 0), y1 = min((int)cy + 1, (int)w.gy - 1);
      const int x0 = max((int)cx - 1, 0), x1 = min((int)cx + 1, (int)w.gx - 1);
      for (int ny = y0; ny <= y1; ++ny) {
        const uint32_t rb = w.cell_off + (uint32_t)ny * w.gx;
        for (int nx = x0; nx <= x1; ++nx) {
          const uint32_t js = cell_start[rb + nx];
          const uint32_t je = min(cell_start[rb + nx + 1], js + ph.cap);
          for (uint32_t j = js; j < je; ++j) {
            if (j == i) continue;
            const float2 pj = pos[j];
            const float dx = __fsub_rn(pj.x, pi.x), dy = __fsub_rn(pj.y, pi.y);
            const float s2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
            if (s2 >= ph.skip_d2) continue;  // no overlap
            pen = fmaxf(pen, __fsub_rn(ph.min_d, __fsqrt_rn(s2)));
          }
        }
      }
    }
  }
  float v[5] = {pen, pen, cnt, ke, 0.f};
  block_partials(v, part);
}

// Deterministic sum of per-block partials: out[k] for k in 0..4 (out[1] the
// max), one block of 256 threads.
__global__ void __launch_bounds__(256)
k_reduce_partials(const float* __restrict__ part, uint32_t nparts, float* __restrict__ out) {
  float v[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  // unrolled, so that the loads of several partials are in flight at once
#pragma unroll 4
  for (uint32_t b = threadIdx.x; b < nparts; b += blockDim.x) {
#pragma unroll
    for (int k = 0; k < 5; ++k) v[k] = k == 1 ? fmaxf(v[k], part[b * 8 + k]) : v[k] + part[b * 8 + k];
  }
  block_partials(v, out - blockIdx.x * 8);
}

// The fallback gate of a surrogate frame, one block.  The partials come from
// the final Jacobi iteration ([0] sum and [1] max of the deepest overlap
// before that iteration, [2] taking-part count, [3] kinetic energy of the
// output, [4] kinetic energy the plain frame has); `mode`:
//   0  after the surrogate correction and the last plain iteration: the frame
//      falls back when its mean overlap exceeds the latest plain frame's by
//      more than `tol`, or its kinetic energy deviates from the plain value
//      by more than `max_drift` (relative); NaN falls back too;
//   1  after the (gated) fallback solve: when the frame fell back, its plain
//      metrics become the reference;
//   2  after a plain calibration frame: its metrics become the reference.
__global__ void __launch_bounds__(1024)
k_gate(const float* __restrict__ part, uint32_t nparts, GateState* __restrict__ gs, int mode) {
  if (mode == 1 && gs->fallback == 0u) return;
  float v[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  // unrolled, so that the loads of several partials are in flight at once
#pragma unroll 4
  for (uint32_t b = threadIdx.x; b < nparts; b += blockDim.x) {
#pragma unroll
    for (int k = 0; k < 5; ++k) v[k] = k == 1 ? fmaxf(v[k], part[b * 8 + k]) : v[k] + part[b * 8 + k];
  }
  __shared__ float tot[8];
  block_partials(v, tot - blockIdx.x * 8);
  __syncthreads();
  if (threadIdx.x != 0) return;
  const float mean = tot[2] > 0.f ? tot[0] / tot[2] : 0.f;
  const float drift = tot[4] > 0.f ? fabsf(tot[3] - tot[4]) / tot[4] : 0.f;
  if (mode == 0) {
    const bool ok = mean <= gs->pen_ref + gs->tol && drift <= gs->max_drift;
    gs->fallback = ok ? 0u : 1u;
    gs->frames += 1;
    gs->drift_max = fmaxf(gs->drift_max, drift);
    if (ok) {
      gs->pen_sum += mean;
      gs->pen_max = fmaxf(gs->pen_max, tot[1]);
    } else {
      gs->fallbacks += 1;
    }
  } else {
    gs->pen_ref = mean;
    gs->pen_sum += mean;
    gs->pen_max = fmaxf(gs->pen_max, tot[1]);
    if (mode == 2) {
      gs->frames += 1;
      gs->calibrations += 1;
    }
  }
}

// Squared errors of the correction against the target, and of zero against
// the target, over taking-part particles: out[0] += |corr - t|^2,
// out[1] += |t|^2, out[2] += count.
__global__ void k_errors(PhysDev ph, uint32_t n, const uint32_t* __restrict__ cell_start,
                         const uint32_t* __restrict__ cell_of, const float2* __restrict__ corr,
                         const float2* __restrict__ target, float* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float e = 0.f, z = 0.f, c = 0.f;
  if (i < n && i - cell_start[cell_of[i]] < ph.cap) {
    const float2 a = corr[i], t = target[i];
    e = (a.x - t.x) * (a.x - t.x) + (a.y - t.y) * (a.y - t.y);
    z = t.x * t.x + t.y * t.y;
    c = 1.f;
  }
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) {
    e += __shfl_xor_sync(0xffffffffu, e, o);
    z += __shfl_xor_sync(0xffffffffu, z, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&out[0], e);
    atomicAdd(&out[1], z);
    atomicAdd(&out[2], c);
  }
}

}  // namespace

cudaError_t launch_errors(const SolveArgs& a, const float2* corr, const float2* target, float* out,
                          cudaStream_t st) {
  if (a.n == 0) return cudaSuccess;
  k_errors<<<(a.n + 255) / 256, 256, 0, st>>>(a.ph, a.n, a.cell_start, a.cell_of, corr, target,
                                              out);
  return cudaGetLastError();
}

cudaError_t launch_knn_features(const SolveArgs& a, uint16_t* x, cudaStream_t st) {
  if (a.n == 0) return cudaSuccess;
  k_knn_features<<<(a.n + 255) / 256, 256, 0, st>>>(a.worlds, a.nworlds, a.ph, a.n, a.cell_start,
                                                    a.ct, a.cell_of, a.tp_pos, a.tp_vel, x);
  return cudaGetLastError();
}

cudaError_t launch_samples(const SolveArgs& a, const float2* q, uint32_t stride, uint32_t phase,
                           uint32_t rows, uint16_t* x, float2* target, cudaStream_t st) {
  if (rows == 0) return cudaSuccess;
  k_samples<<<(rows + 255) / 256, 256, 0, st>>>(a.worlds, a.nworlds, a.ncells, a.ct, a.tp_cell,
                                                a.tp_pos, a.tp_vel, q, stride, phase, rows, x,
                                                target);
  return cudaGetLastError();
}

int surrogate_correct_blocks(int device) {
  const size_t smem = correct_smem();
  if (cudaFuncSetAttribute(k_surrogate_correct, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return 0;
  // persistent: one wave of co-resident blocks
  int sms = 0, per_sm = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_surrogate_correct, kFuseThreads,
                                                    smem) != cudaSuccess)
    return 0;
  return sms * (per_sm > 0 ? per_sm : 1);
}

cudaError_t launch_surrogate_correct(const MlpDev& m, const SolveArgs& a, float2* q, float2* corr,
                                     int blocks, cudaStream_t st) {
  if (a.n == 0) return cudaSuccess;
  const int need = (int)((a.n + kFuseThreads - 1) / kFuseThreads);
  k_surrogate_correct<<<need < blocks ? need : blocks, kFuseThreads, correct_smem(), st>>>(
      m, a.worlds, a.nworlds, a.ncells, a.cell_start, a.ct, a.tp_cell, a.tp_pos, a.tp_vel, q,
      corr);
  return cudaGetLastError();
}

cudaError_t launch_gate(const float* part, uint32_t nparts, GateState* gs, int mode,
                        cudaStream_t st) {
  k_gate<<<1, 1024, 0, st>>>(part, nparts, gs, mode);
  return cudaGetLastError();
}

cudaError_t launch_mlp_forward(const MlpDev& m, const uint16_t* x, uint32_t n, float2* y,
                               int blocks, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int need = (int)((n + 63) / 64);
  k_mlp_forward<<<need < blocks ? need : blocks, 128, 0, st>>>(m, x, n, y);
  return cudaGetLastError();
}

cudaError_t launch_mlp_backward(const MlpDev& m, const uint16_t* x, const float2* target,
                                uint32_t n, float inv_rows, float* grad, float* loss, int blocks,
                                cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const size_t smem = backward_smem();
  cudaError_t e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  const int need = (int)((n + 63) / 64);
  k_mlp_backward<<<need < blocks ? need : blocks, 128, smem, st>>>(m, x, target, n, inv_rows,
                                                                   grad, loss);
  return cudaGetLastError();
}

cudaError_t launch_adam(const MlpDev& m, const float* grad, float* mom1, float* mom2, float lr,
                        uint32_t step, cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  k_adam<<<(kMlpParams + 255) / 256, 256, 0, st>>>(m, grad, mom1, mom2, lr, b1, b2, eps, bc1,
                                                    bc2, kMlpParams);
  return cudaGetLastError();
}

cudaError_t launch_target(const SolveArgs& a, uint32_t n, const float2* q, float2* target,
                          cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_target<<<(n + 255) / 256, 256, 0, st>>>(n, a.ph, a.cell_start, a.ct, a.cell_of, a.pos, q,
                                            target);
  return cudaGetLastError();
}

cudaError_t launch_penetration(const SolveArgs& a, const float2* pos, const float2* vel,
                               float* part, float* out, cudaStream_t st) {
  const uint32_t blocks = (a.n + 255) / 256;
  if (blocks) {
    k_penetration<<<blocks, 256, 0, st>>>(a.worlds, a.nworlds, a.ph, a.n, a.cell_start, a.cell_of,
                                          pos, vel, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  k_reduce_partials<<<1, 256, 0, st>>>(part, blocks, out);
  return cudaGetLastError();
}

}  // namespace wrach
