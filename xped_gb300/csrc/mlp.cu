// Rank-predictor MLP: kFeatures -> 64 -> 64 -> 64 -> 2, ReLU hidden layers,
// FP32.  Forward, backward (mean-squared-error loss) and Adam are this
// file's kernels; a CTA works on tiles of kTile samples with the weights in
// shared memory (rows padded to an odd stride so that both the row-wise and
// the column-wise sweeps are bank-conflict free).  Gradients are reduced
// per CTA into a private slot and summed in a fixed order by the Adam
// kernel, so training is deterministic.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "kernels.hpp"

namespace xgb {
namespace {

constexpr int F = kMlpIn, H = kMlpHidden, O = kMlpOut;
constexpr int kTile = 32;
constexpr int kThreads = 256;
// padded shared-memory strides
constexpr int L1 = F + 1, LH = H + 1;
// offsets of the packed parameter vector (row-major W[out][in], then b)
constexpr int oW1 = 0, oB1 = oW1 + H * F, oW2 = oB1 + H, oB2 = oW2 + H * H, oW3 = oB2 + H, oB3 = oW3 + H * H,
              oW4 = oB3 + H, oB4 = oW4 + O * H, kP = oB4 + O;
static_assert(kP == kMlpParams, "parameter count");
// shared layout (floats)
constexpr int sW1 = 0, sW2 = sW1 + H * L1, sW3 = sW2 + H * LH, sW4 = sW3 + H * LH, sB = sW4 + O * LH,
              sWend = sB + 3 * H + O;

struct Smem {
  float* w;               // padded weights + biases
  float* g;               // padded gradient accumulators (same layout)
  float* x;               // kTile x F
  float* h[3];            // kTile x H activations (post ReLU)
  float* y;               // kTile x O
  float* d[2];            // kTile x H deltas
};

__device__ void load_params(const float* __restrict__ p, float* w) {
  for (int e = threadIdx.x; e < H * F; e += kThreads) w[sW1 + (e / F) * L1 + e % F] = p[oW1 + e];
  for (int e = threadIdx.x; e < H * H; e += kThreads) {
    w[sW2 + (e / H) * LH + e % H] = p[oW2 + e];
    w[sW3 + (e / H) * LH + e % H] = p[oW3 + e];
  }
  for (int e = threadIdx.x; e < O * H; e += kThreads) w[sW4 + (e / H) * LH + e % H] = p[oW4 + e];
  for (int e = threadIdx.x; e < H; e += kThreads) {
    w[sB + e] = p[oB1 + e];
    w[sB + H + e] = p[oB2 + e];
    w[sB + 2 * H + e] = p[oB3 + e];
  }
  for (int e = threadIdx.x; e < O; e += kThreads) w[sB + 3 * H + e] = p[oB4 + e];
}

// out[s][j] = act(sum_k in[s][k] W[j][k] + b[j]) for s < S, j < J
__device__ void fwd(const float* in, int ldin, int K, const float* W, int ldw, const float* b, float* out, int J, int S,
                    bool relu) {
  for (int e = threadIdx.x; e < S * J; e += kThreads) {
    const int s = e / J, j = e % J;
    float acc = b[j];
    for (int k = 0; k < K; ++k) acc = fmaf(in[s * ldin + k], W[j * ldw + k], acc);
    out[s * J + j] = relu ? fmaxf(acc, 0.0f) : acc;
  }
  __syncthreads();
}

// dW[j][k] += sum_s dout[s][j] in[s][k];  db[j] += sum_s dout[s][j]
__device__ void grad_w(const float* dout, int J, const float* in, int ldin, int K, float* dW, int ldw, float* db, int S) {
  for (int e = threadIdx.x; e < J * K; e += kThreads) {
    const int j = e / K, k = e % K;
    float acc = 0;
    for (int s = 0; s < S; ++s) acc = fmaf(dout[s * J + j], in[s * ldin + k], acc);
    dW[j * ldw + k] += acc;
  }
  for (int j = threadIdx.x; j < J; j += kThreads) {
    float acc = 0;
    for (int s = 0; s < S; ++s) acc += dout[s * J + j];
    db[j] += acc;
  }
}

// din[s][k] = (sum_j dout[s][j] W[j][k]) * [act[s][k] > 0]
__device__ void back(const float* dout, int J, const float* W, int ldw, const float* act, float* din, int K, int S) {
  for (int e = threadIdx.x; e < S * K; e += kThreads) {
    const int s = e / K, k = e % K;
    float acc = 0;
    for (int j = 0; j < J; ++j) acc = fmaf(dout[s * J + j], W[j * ldw + k], acc);
    din[s * K + k] = act[s * K + k] > 0.0f ? acc : 0.0f;
  }
}

__device__ void carve(Smem& m, float* base) {
  m.w = base;
  m.g = m.w + sWend;
  m.x = m.g + sWend;
  m.h[0] = m.x + kTile * F;
  m.h[1] = m.h[0] + kTile * H;
  m.h[2] = m.h[1] + kTile * H;
  m.y = m.h[2] + kTile * H;
  m.d[0] = m.y + kTile * O;
  m.d[1] = m.d[0] + kTile * H;
}

constexpr int kSmemFloats = 2 * sWend + kTile * F + 3 * kTile * H + kTile * O + 2 * kTile * H;

__device__ int forward_tile(const Smem& m, const float* __restrict__ X, int64_t n, int64_t t0) {
  const int S = int(n - t0 < kTile ? n - t0 : kTile);
  for (int e = threadIdx.x; e < S * F; e += kThreads) m.x[e] = X[t0 * F + e];
  __syncthreads();
  fwd(m.x, F, F, m.w + sW1, L1, m.w + sB, m.h[0], H, S, true);
  fwd(m.h[0], H, H, m.w + sW2, LH, m.w + sB + H, m.h[1], H, S, true);
  fwd(m.h[1], H, H, m.w + sW3, LH, m.w + sB + 2 * H, m.h[2], H, S, true);
  fwd(m.h[2], H, H, m.w + sW4, LH, m.w + sB + 3 * H, m.y, O, S, false);
  return S;
}

__global__ void __launch_bounds__(kThreads) mlp_forward_kernel(const float* __restrict__ p, const float* __restrict__ X,
                                                               int64_t n, float* __restrict__ Y) {
  extern __shared__ float smem[];
  Smem m;
  carve(m, smem);
  load_params(p, m.w);
  __syncthreads();
  for (int64_t t0 = int64_t(blockIdx.x) * kTile; t0 < n; t0 += int64_t(gridDim.x) * kTile) {
    const int S = forward_tile(m, X, n, t0);
    for (int e = threadIdx.x; e < S * O; e += kThreads) Y[t0 * O + e] = m.y[e];
    __syncthreads();
  }
}

// loss = (1/n) sum_s sum_o (y - t)^2 / 2 ; per-CTA gradient slot g (kP floats) and loss slot
__global__ void __launch_bounds__(kThreads) mlp_grad_kernel(const float* __restrict__ p, const float* __restrict__ X,
                                                            const float* __restrict__ T, int64_t n,
                                                            float* __restrict__ gpart, float* __restrict__ lpart) {
  extern __shared__ float smem[];
  __shared__ float lsum[kThreads];
  Smem m;
  carve(m, smem);
  load_params(p, m.w);
  for (int e = threadIdx.x; e < sWend; e += kThreads) m.g[e] = 0.0f;
  float myloss = 0.0f;
  const float inv_n = 1.0f / float(n);
  __syncthreads();
  for (int64_t t0 = int64_t(blockIdx.x) * kTile; t0 < n; t0 += int64_t(gridDim.x) * kTile) {
    const int S = forward_tile(m, X, n, t0);
    // dy = (y - t) / n into d[1] (kTile x O)
    for (int e = threadIdx.x; e < S * O; e += kThreads) {
      const float r = m.y[e] - T[t0 * O + e];
      myloss = fmaf(r, r, myloss);
      m.d[1][e] = r * inv_n;
    }
    __syncthreads();
    grad_w(m.d[1], O, m.h[2], H, H, m.g + sW4, LH, m.g + sB + 3 * H, S);
    back(m.d[1], O, m.w + sW4, LH, m.h[2], m.d[0], H, S);
    __syncthreads();
    grad_w(m.d[0], H, m.h[1], H, H, m.g + sW3, LH, m.g + sB + 2 * H, S);
    back(m.d[0], H, m.w + sW3, LH, m.h[1], m.d[1], H, S);
    __syncthreads();
    grad_w(m.d[1], H, m.h[0], H, H, m.g + sW2, LH, m.g + sB + H, S);
    back(m.d[1], H, m.w + sW2, LH, m.h[0], m.d[0], H, S);
    __syncthreads();
    grad_w(m.d[0], H, m.x, F, F, m.g + sW1, L1, m.g + sB, S);
    __syncthreads();
  }
  float* gp = gpart + int64_t(blockIdx.x) * kP;
  for (int e = threadIdx.x; e < H * F; e += kThreads) gp[oW1 + e] = m.g[sW1 + (e / F) * L1 + e % F];
  for (int e = threadIdx.x; e < H * H; e += kThreads) {
    gp[oW2 + e] = m.g[sW2 + (e / H) * LH + e % H];
    gp[oW3 + e] = m.g[sW3 + (e / H) * LH + e % H];
  }
  for (int e = threadIdx.x; e < O * H; e += kThreads) gp[oW4 + e] = m.g[sW4 + (e / H) * LH + e % H];
  for (int e = threadIdx.x; e < H; e += kThreads) {
    gp[oB1 + e] = m.g[sB + e];
    gp[oB2 + e] = m.g[sB + H + e];
    gp[oB3 + e] = m.g[sB + 2 * H + e];
  }
  for (int e = threadIdx.x; e < O; e += kThreads) gp[oB4 + e] = m.g[sB + 3 * H + e];
  lsum[threadIdx.x] = myloss;
  __syncthreads();
  if (threadIdx.x == 0) {
    float acc = 0;
    for (int i = 0; i < kThreads; ++i) acc += lsum[i];
    lpart[blockIdx.x] = 0.5f * acc * inv_n;
  }
}

// grad = sum of the per-CTA slots in CTA order; optional Adam step
__global__ void mlp_reduce_adam_kernel(float* __restrict__ p, float* __restrict__ mom, float* __restrict__ vel,
                                       const float* __restrict__ gpart, int slots, float* __restrict__ grad_out,
                                       int adam, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kP) return;
  float g = 0;
  for (int s = 0; s < slots; ++s) g += gpart[int64_t(s) * kP + i];
  if (grad_out) grad_out[i] = g;
  if (!adam) return;
  const float m1 = b1 * mom[i] + (1.0f - b1) * g;
  const float v1 = b2 * vel[i] + (1.0f - b2) * g * g;
  mom[i] = m1;
  vel[i] = v1;
  p[i] -= lr * (m1 / c1) / (sqrtf(v1 / c2) + eps);
}

std::once_flag g_attr_set;

void set_attrs() {
  std::call_once(g_attr_set, [] {
    const int bytes = kSmemFloats * int(sizeof(float));
    cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  });
}

int grid_for(int64_t n) {
  const int64_t tiles = (n + kTile - 1) / kTile;
  const int64_t cap = int64_t(num_sms());
  return int(tiles < cap ? (tiles < 1 ? 1 : tiles) : cap);
}

}  // namespace

int mlp_grad_slots(int64_t n) { return grid_for(n); }

void launch_mlp_forward(const float* params, const float* X, int64_t n, float* Y, cudaStream_t s) {
  if (n <= 0) return;
  set_attrs();
  mlp_forward_kernel<<<grid_for(n), kThreads, kSmemFloats * sizeof(float), s>>>(params, X, n, Y);
  count_launch();
}

void launch_mlp_grad(const float* params, const float* X, const float* T, int64_t n, float* gpart, float* lpart,
                     cudaStream_t s) {
  if (n <= 0) return;
  set_attrs();
  mlp_grad_kernel<<<grid_for(n), kThreads, kSmemFloats * sizeof(float), s>>>(params, X, T, n, gpart, lpart);
  count_launch();
}

void launch_mlp_reduce_adam(float* params, float* mom, float* vel, const float* gpart, int slots, float* grad_out,
                            int adam, float lr, float b1, float b2, float eps, int step, cudaStream_t s) {
  const float c1 = 1.0f - powf(b1, float(step)), c2 = 1.0f - powf(b2, float(step));
  mlp_reduce_adam_kernel<<<(kP + 255) / 256, 256, 0, s>>>(params, mom, vel, gpart, slots, grad_out, adam, lr, b1, b2,
                                                          eps, adam ? c1 : 1.0f, adam ? c2 : 1.0f);
  count_launch();
}

}  // namespace xgb
