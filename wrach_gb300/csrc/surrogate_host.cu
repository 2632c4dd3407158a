// The C ABI of the learned surrogate (include/wrach.h: wrach_surrogate_*
// and wrach_frame_metrics): parameters, training on collected frames, and the
// gated surrogate frame.  Host orchestration of the kernels in surrogate.cu.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "context_internal.h"

using namespace wrach::host;

namespace {

uint16_t to_bf16(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u && (u & 0x007FFFFFu)) return (uint16_t)((u >> 16) | 0x40);
  u += 0x7FFFu + ((u >> 16) & 1u);  // round to nearest even
  return (uint16_t)(u >> 16);
}

// BF16 copies of the FP32 parameters in both layouts, uploaded.
int upload_params(WrachContext* ctx, const float* p) {
  using namespace wrach;
  const uint32_t o_b1 = kMlpIn * kMlpHidden, o_w2 = o_b1 + kMlpHidden;
  const uint32_t o_b2 = o_w2 + kMlpHidden * kMlpHidden, o_w3 = o_b2 + kMlpHidden;
  std::vector<uint16_t> h((size_t)2 * (2 * kMlpIn * kMlpHidden + kMlpHidden * kMlpOutPad));
  uint16_t* w1 = h.data();
  uint16_t* w1t = w1 + kMlpIn * kMlpHidden;
  uint16_t* w2 = w1t + kMlpIn * kMlpHidden;
  uint16_t* w2t = w2 + kMlpHidden * kMlpHidden;
  uint16_t* w3 = w2t + kMlpHidden * kMlpHidden;
  uint16_t* w3t = w3 + kMlpHidden * kMlpOutPad;
  for (uint32_t r = 0; r < kMlpIn; ++r)
    for (uint32_t c = 0; c < kMlpHidden; ++c) {
      w1[r * kMlpHidden + c] = w1t[c * kMlpIn + r] = to_bf16(p[r * kMlpHidden + c]);
      w2[r * kMlpHidden + c] = w2t[c * kMlpHidden + r] = to_bf16(p[o_w2 + r * kMlpHidden + c]);
    }
  for (uint32_t r = 0; r < kMlpHidden; ++r)
    for (uint32_t c = 0; c < kMlpOutPad; ++c)
      w3[r * kMlpOutPad + c] = w3t[c * kMlpHidden + r] = to_bf16(p[o_w3 + r * kMlpOutPad + c]);
  CK(cudaMemcpyAsync(ctx->sur.params, p, kMlpParams * 4, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->sur.bf16, h.data(), h.size() * 2, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  (void)o_b2;
  return WRACH_OK;
}

int surrogate_ready(WrachContext* ctx) {
  if (!ctx) return WRACH_ERR_INVALID_ARGUMENT;
  if (!ctx->sur.ready) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "call wrach_surrogate_init first");
  return WRACH_OK;
}

// The metric buffers: 8 floats of sums, per-block partials for a solve
// launch of up to total_cap / 32 blocks, and the gate state.
int ensure_metrics(WrachContext* ctx) {
  auto& S = ctx->sur;
  if (!S.metrics) CK(dalloc(&S.metrics, 8));
  if (!S.part) CK(dalloc(&S.part, ((size_t)ctx->total_cap / 32 + 2) * 8));
  if (!S.gate) CK(dalloc(&S.gate, 1));
  return WRACH_OK;
}

// The rebin of a frame whose solve output is in pos_o / vel_o / keys.
int enqueue_rebin(WrachContext* ctx) {
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
  CK(wrach::launch_count_sort(r, ctx->big_blocks, ctx->stream));
  ctx->launches += wrach::count_sort_launches(r.n, ctx->ncells);
  ctx->cur ^= 1;
  return WRACH_OK;
}

// The plain extended solve of the binned frame into pos_o / vel_o / keys;
// the final pass writes the gate metrics when `a.part` is set.
int enqueue_plain_solve(WrachContext* ctx, const wrach::SolveArgs& a) {
  wrach::SolveArgs inner = a;
  inner.part = nullptr;
  const float2* q = nullptr;
  CK(enqueue_iterations(ctx, inner, ctx->ph.iterations - 1, ctx->stream, &q, []() {}));
  CK(wrach::launch_jacobi_final(a, q, 1, ctx->stream));
  ctx->launches += ctx->n ? ctx->ph.iterations : 0u;
  return WRACH_OK;
}

// every kCalibrationPeriod-th surrogate frame, the first included, is a
// plain frame whose metrics become the gate's reference
constexpr uint32_t kCalibrationPeriod = 32;

// One surrogate frame, or a plain calibration frame, with no host
// synchronisation: the gate decides on the device.
int enqueue_surrogate_frame(WrachContext* ctx, int calibration) {
  auto& S = ctx->sur;
  wrach::SolveArgs a = solve_args(ctx);
  a.part = S.part;
  int rc;
  if (calibration) {
    // a plain frame: its metrics are the reference of the next frames
    if ((rc = enqueue_plain_solve(ctx, a))) return rc;
    CK(wrach::launch_gate(S.part, wrach::solve_blocks(a), S.gate, 2, ctx->stream));
    ctx->launches += 1;
  } else {
    // the surrogate correction, the last plain iteration, the gate
    CK(wrach::launch_surrogate_correct(S.m, a, ctx->q1, nullptr, S.correct_blocks, ctx->stream));
    CK(wrach::launch_jacobi_final(a, ctx->q1, 1, ctx->stream));
    CK(wrach::launch_gate(S.part, wrach::solve_blocks(a), S.gate, 0, ctx->stream));
    // the plain solve of the same frame, run only when the gate failed it
    // (its launches stride over the frame with few blocks, so skipping them
    // is cheap), and the gate again on its metrics
    a.run_if = &S.gate->fallback;
    if ((rc = enqueue_plain_solve(ctx, a))) return rc;
    CK(wrach::launch_gate(S.part, wrach::solve_blocks(a), S.gate, 1, ctx->stream));
    ctx->launches += (ctx->n ? 2 : 0) + 2;
  }
  return enqueue_rebin(ctx);
}

}  // namespace

extern "C" {

uint32_t wrach_surrogate_param_count(void) { return wrach::kMlpParams; }

int wrach_surrogate_init(WrachContext* ctx, uint32_t seed, uint32_t max_samples) {
  using namespace wrach;
  if (!ctx) return WRACH_ERR_INVALID_ARGUMENT;
  if (ctx->ph.mode != WRACH_MODE_EXTENDED || ctx->ph.iterations < 2)
    return fail(ctx, WRACH_ERR_UNSUPPORTED,
                "the surrogate replaces iterations of the extended solve: mode EXTENDED, iterations >= 2");
  DeviceGuard guard(ctx->device);
  auto& S = ctx->sur;
  if (!S.ready) {
    const size_t nbf = (size_t)2 * (2 * kMlpIn * kMlpHidden + kMlpHidden * kMlpOutPad);
    CK(dalloc(&S.params, kMlpParams));
    CK(dalloc(&S.grad, kMlpParams));
    CK(dalloc(&S.mom1, kMlpParams));
    CK(dalloc(&S.mom2, kMlpParams));
    CK(dalloc(&S.loss, 1));
    CK(dalloc(&S.metrics, 8));
    CK(dalloc(&S.bf16, nbf));
    CK(dalloc(&S.x, (size_t)ctx->total_cap * kMlpIn));
    CK(dalloc(&S.corr, ctx->total_cap));
    S.m.params = S.params;
    S.m.b1 = S.params + kMlpIn * kMlpHidden;
    S.m.b2 = S.m.b1 + kMlpHidden + kMlpHidden * kMlpHidden;
    S.m.b3 = S.m.b2 + kMlpHidden + kMlpHidden * kMlpOutPad;
    S.m.w1 = S.bf16;
    S.m.w1t = S.m.w1 + kMlpIn * kMlpHidden;
    S.m.w2 = S.m.w1t + kMlpIn * kMlpHidden;
    S.m.w2t = S.m.w2 + kMlpHidden * kMlpHidden;
    S.m.w3 = S.m.w2t + kMlpHidden * kMlpHidden;
    S.m.w3t = S.m.w3 + kMlpHidden * kMlpOutPad;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    S.blocks = sms > 0 ? 4 * sms : 64;
    S.correct_blocks = wrach::surrogate_correct_blocks(ctx->device);
    if (S.correct_blocks <= 0) return fail(ctx, WRACH_ERR_CUDA, "surrogate kernel set-up failed");
  }
  if (max_samples > S.max_samples) {
    dfree(S.tx);
    dfree(S.tt);
    S.tx = nullptr;
    S.tt = nullptr;
    CK(dalloc(&S.tx, (size_t)max_samples * kMlpIn));
    CK(dalloc(&S.tt, max_samples));
    S.max_samples = max_samples;
  }
  S.nsamples = 0;
  S.step = 0;
  S.collects = 0;
  // Glorot-uniform weights from a fixed-seed generator, zero biases, a
  // small last layer so that the initial correction is near zero
  std::vector<float> p(kMlpParams, 0.0f);
  uint64_t st = 0x9E3779B97F4A7C15ull ^ ((uint64_t)seed * 0xBF58476D1CE4E5B9ull);
  auto uni = [&]() {
    st ^= st >> 12; st ^= st << 25; st ^= st >> 27;
    return ((st * 0x2545F4914F6CDD1Dull) >> 40) * (1.0 / 16777216.0) * 2.0 - 1.0;
  };
  const uint32_t o_w2 = kMlpIn * kMlpHidden + kMlpHidden;
  const uint32_t o_w3 = o_w2 + kMlpHidden * kMlpHidden + kMlpHidden;
  const float a1 = std::sqrt(6.0f / (kMlpIn + kMlpHidden)), a2 = std::sqrt(6.0f / (2 * kMlpHidden));
  const float a3 = 0.1f * std::sqrt(6.0f / (kMlpHidden + 2));
  for (uint32_t i = 0; i < kMlpIn * kMlpHidden; ++i) p[i] = (float)(a1 * uni());
  for (uint32_t i = 0; i < kMlpHidden * kMlpHidden; ++i) p[o_w2 + i] = (float)(a2 * uni());
  for (uint32_t r = 0; r < kMlpHidden; ++r)
    for (uint32_t c = 0; c < 2; ++c) p[o_w3 + r * kMlpOutPad + c] = (float)(a3 * uni());
  CK(cudaMemsetAsync(S.mom1, 0, kMlpParams * 4, ctx->stream));
  CK(cudaMemsetAsync(S.mom2, 0, kMlpParams * 4, ctx->stream));
  int rc = upload_params(ctx, p.data());
  if (rc) return rc;
  S.ready = true;
  return WRACH_OK;
}

int wrach_surrogate_set_params(WrachContext* ctx, const float* params, uint32_t count) {
  int rc = surrogate_ready(ctx);
  if (rc) return rc;
  if (!params || count != wrach::kMlpParams) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "need all parameters");
  DeviceGuard guard(ctx->device);
  return upload_params(ctx, params);
}

int wrach_surrogate_get_params(WrachContext* ctx, float* params, uint32_t count) {
  int rc = surrogate_ready(ctx);
  if (rc) return rc;
  if (!params || count < wrach::kMlpParams) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "buffer too small");
  DeviceGuard guard(ctx->device);
  CK(cudaMemcpyAsync(params, ctx->sur.params, wrach::kMlpParams * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return WRACH_OK;
}

int wrach_surrogate_features(WrachContext* ctx, uint16_t* d_x, uint32_t rows) {
  int rc = surrogate_ready(ctx);
  if (rc) return rc;
  if (!d_x || rows < ctx->n) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "feature buffer too small");
  DeviceGuard guard(ctx->device);
  CK(wrach::launch_knn_features(solve_args(ctx), d_x, ctx->stream));
  ctx->launches += ctx->n ? 1 : 0;
  return WRACH_OK;
}

int wrach_surrogate_forward(WrachContext* ctx, const uint16_t* d_x, uint32_t n, float* d_y) {
  int rc = surrogate_ready(ctx);
  if (rc) return rc;
  if (n && (!d_x || !d_y)) return WRACH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(ctx->device);
  CK(wrach::launch_mlp_forward_tc(ctx->sur.m, d_x, n, reinterpret_cast<float2*>(d_y),
                                  &ctx->ctrl->flags, ctx->sms, ctx->stream));
  ctx->launches += n ? 1 : 0;
  return WRACH_OK;
}

int wrach_surrogate_forward_mma(WrachContext* ctx, const uint16_t* d_x, uint32_t n, float* d_y) {
  int rc = surrogate_ready(ctx);
  if (rc) return rc;
  if (n && (!d_x || !d_y)) return WRACH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(ctx->device);
  CK(wrach::launch_mlp_forward(ctx->sur.m, d_x, n, reinterpret_cast<float2*>(d_y), ctx->sur.blocks,
                               ctx->stream));
  ctx->launches += n ? 1 : 0;
  return WRACH_OK;
}

int wrach_surrogate_gradients(WrachContext* ctx, const uint16_t* d_x, const float* d_t, uint32_t n,
                              float* grad, float* loss) {
  int rc = surrogate_ready(ctx);
  if (rc) return rc;
  if (!n || !d_x || !d_t || !grad || !loss) return WRACH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(ctx->device);
  auto& S = ctx->sur;
  CK(cudaMemsetAsync(S.grad, 0, wrach::kMlpParams * 4, ctx->stream));
  CK(cudaMemsetAsync(S.loss, 0, 4, ctx->stream));
  CK(wrach::launch_mlp_backward(S.m, d_x, reinterpret_cast<const float2*>(d_t), n, 1.0f / n, S.grad,
                                S.loss, S.blocks, ctx->stream));
  ctx->launches += 1;
  CK(cudaMemcpyAsync(grad, S.grad, wrach::kMlpParams * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(loss, S.loss, 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return WRACH_OK;
}

int wrach_surrogate_collect(WrachContext* ctx, uint32_t stride, uint32_t* total) {
  int rc = surrogate_ready(ctx);
  if (rc) return rc;
  DeviceGuard guard(ctx->device);
  auto& S = ctx->sur;
  if (stride == 0) stride = 1;
  wrach::SolveArgs a = solve_args(ctx);
  // the frame's taking-part particles: every stride-th of them, from an
  // offset that turns with each call, so that consecutive frames give others
  uint32_t ntp = 0;
  if (ctx->n) {
    CK(cudaMemcpyAsync(&ntp, a.ct + ctx->ncells, 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  const uint32_t phase = S.collects++ % stride;
  const uint32_t rows = ntp > phase ? (ntp - phase + stride - 1) / stride : 0u;
  const uint32_t take = std::min(rows, S.max_samples - S.nsamples);
  if (take) {
    // the features, then the correction of the frame's first K-1 iterations
    const float2* q = nullptr;
    CK(enqueue_iterations(ctx, a, ctx->ph.iterations - 1, ctx->stream, &q, []() {}));
    CK(wrach::launch_samples(a, q, stride, phase, take, S.tx + (size_t)S.nsamples * wrach::kMlpIn,
                             S.tt + S.nsamples, ctx->stream));
    ctx->launches += ctx->ph.iterations;
    S.nsamples += take;
  }
  if (total) *total = S.nsamples;
  return WRACH_OK;
}

int wrach_surrogate_evaluate(WrachContext* ctx, float* mse_network, float* mse_zero) {
  int rc = surrogate_ready(ctx);
  if (rc) return rc;
  if (!mse_network || !mse_zero) return WRACH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(ctx->device);
  auto& S = ctx->sur;
  wrach::SolveArgs a = solve_args(ctx);
  CK(wrach::launch_knn_features(a, S.x, ctx->stream));
  CK(wrach::launch_mlp_forward(S.m, S.x, ctx->n, S.corr, S.blocks, ctx->stream));
  const float2* q = nullptr;
  CK(enqueue_iterations(ctx, a, ctx->ph.iterations - 1, ctx->stream, &q, []() {}));
  // the target lands in pos_o (scratch between frames)
  CK(wrach::launch_target(a, ctx->n, q, ctx->pos_o, ctx->stream));
  CK(cudaMemsetAsync(S.metrics, 0, 8 * 4, ctx->stream));
  CK(wrach::launch_errors(a, S.corr, ctx->pos_o, S.metrics, ctx->stream));
  float h[8];
  CK(cudaMemcpyAsync(h, S.metrics, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->launches += ctx->ph.iterations + 3;
  *mse_network = h[2] > 0.f ? h[0] / h[2] : 0.f;
  *mse_zero = h[2] > 0.f ? h[1] / h[2] : 0.f;
  return WRACH_OK;
}

int wrach_frame_metrics(WrachContext* ctx, float* mean_penetration, float* max_penetration,
                        float* kinetic_energy) {
  if (!ctx || !mean_penetration || !max_penetration || !kinetic_energy)
    return WRACH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(ctx->device);
  int rc = ensure_metrics(ctx);
  if (rc) return rc;
  wrach::SolveArgs a = solve_args(ctx);
  CK(wrach::launch_penetration(a, ctx->pos, ctx->vel, ctx->sur.part, ctx->sur.metrics, ctx->stream));
  float h[8];
  CK(cudaMemcpyAsync(h, ctx->sur.metrics, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->launches += ctx->n ? 2 : 1;
  *mean_penetration = h[2] > 0.f ? h[0] / h[2] : 0.f;
  *max_penetration = h[1];
  *kinetic_energy = h[3];
  return WRACH_OK;
}

int wrach_surrogate_correction(WrachContext* ctx, float* d_corr) {
  int rc = surrogate_ready(ctx);
  if (rc) return rc;
  if (!d_corr && ctx->n) return WRACH_ERR_INVALID_ARGUMENT;
  DeviceGuard guard(ctx->device);
  wrach::SolveArgs a = solve_args(ctx);
  // the particles that take no part get a zero correction
  if (ctx->n) CK(cudaMemsetAsync(d_corr, 0, (size_t)ctx->n * sizeof(float2), ctx->stream));
  CK(wrach::launch_surrogate_correct(ctx->sur.m, a, ctx->q1, reinterpret_cast<float2*>(d_corr),
                                     ctx->sur.correct_blocks, ctx->stream));
  ctx->launches += ctx->n ? 1 : 0;
  return WRACH_OK;
}

int wrach_surrogate_train(WrachContext* ctx, uint32_t steps, uint32_t batch, float lr, float* loss) {
  int rc = surrogate_ready(ctx);
  if (rc) return rc;
  auto& S = ctx->sur;
  if (!batch || S.nsamples == 0) return fail(ctx, WRACH_ERR_INVALID_ARGUMENT, "no samples collected");
  DeviceGuard guard(ctx->device);
  const uint32_t b = std::min(batch, S.nsamples);
  for (uint32_t s = 0; s < steps; ++s) {
    // a window of the sample buffer, spread over it by a multiplicative hash
    const uint32_t span = S.nsamples - b + 1;
    const uint32_t off = (uint32_t)(((uint64_t)(S.step + 1) * 2654435761ull) % span);
    CK(cudaMemsetAsync(S.grad, 0, wrach::kMlpParams * 4, ctx->stream));
    CK(cudaMemsetAsync(S.loss, 0, 4, ctx->stream));
    CK(wrach::launch_mlp_backward(S.m, S.tx + (size_t)off * wrach::kMlpIn, S.tt + off, b, 1.0f / b,
                                  S.grad, S.loss, S.blocks, ctx->stream));
    ++S.step;
    CK(wrach::launch_adam(S.m, S.grad, S.mom1, S.mom2, lr, S.step, ctx->stream));
    ctx->launches += 2;
  }
  if (loss) {
    CK(cudaMemcpyAsync(loss, S.loss, 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return WRACH_OK;
}

int wrach_surrogate_step(WrachContext* ctx, uint32_t nsteps, float max_penetration,
                         float max_energy_drift, WrachSurrogateStats* stats) {
  int rc = surrogate_ready(ctx);
  if (rc) return rc;
  DeviceGuard guard(ctx->device);
  if ((rc = ensure_metrics(ctx))) return rc;
  auto& S = ctx->sur;
  wrach::GateState g0{};
  g0.tol = max_penetration;
  g0.max_drift = max_energy_drift;
  CK(cudaMemcpyAsync(S.gate, &g0, sizeof(g0), cudaMemcpyHostToDevice, ctx->stream));
  for (uint32_t f = 0; f < nsteps; ++f) {
    const int calibration = f % kCalibrationPeriod == 0 ? 1 : 0;
    const int parity = ctx->cur;
    cudaGraphExec_t& g = S.graph[parity][calibration];
    // a graph holds the particle count (grid sizes) it was captured with
    if (g && S.graph_n[parity][calibration] != ctx->n) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
    if (!g && ctx->graph_ok) {
      const uint64_t launches = ctx->launches;
      cudaGraph_t graph = nullptr;
      bool ok = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      if (ok) {
        rc = enqueue_surrogate_frame(ctx, calibration);
        ok = cudaStreamEndCapture(ctx->stream, &graph) == cudaSuccess && rc == WRACH_OK && graph;
        ctx->cur = parity;
        S.graph_launches[parity][calibration] = (uint32_t)(ctx->launches - launches);
        ctx->launches = launches;
        if (ok) ok = cudaGraphInstantiate(&g, graph, 0) == cudaSuccess;
        if (graph) cudaGraphDestroy(graph);
      }
      if (!ok) {
        // capture unavailable: this and later frames run eagerly
        cudaGetLastError();
        g = nullptr;
        ctx->graph_ok = false;
        ctx->err.clear();
      } else {
        S.graph_n[parity][calibration] = ctx->n;
      }
    }
    if (g) {
      CK(cudaGraphLaunch(g, ctx->stream));
      ctx->launches += S.graph_launches[parity][calibration];
      ctx->cur ^= 1;
    } else if ((rc = enqueue_surrogate_frame(ctx, calibration))) {
      return rc;
    }
  }
  wrach::GateState g{};
  CK(cudaMemcpyAsync(&g, S.gate, sizeof(g), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  WrachSurrogateStats st{};
  st.frames = g.frames;
  st.fallbacks = g.fallbacks;
  st.calibrations = g.calibrations;
  st.mean_penetration = g.frames ? g.pen_sum / (float)g.frames : 0.f;
  st.max_penetration = g.pen_max;
  st.max_energy_drift = g.drift_max;
  st.reference_penetration = g.pen_ref;
  if (stats) *stats = st;
  return WRACH_OK;
}

}  // extern "C"
