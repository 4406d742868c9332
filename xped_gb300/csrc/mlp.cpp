// Host side of the rank-predictor MLP (device parameters, Adam state, the
// width policy of the randomized projector SVD).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "rank_model.hpp"

namespace xgb {
namespace {

void ok(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

double normal(uint64_t& s) {  // Box-Muller
  const double u1 = (double(splitmix(s) >> 11) + 1.0) * 0x1.0p-53, u2 = double(splitmix(s) >> 11) * 0x1.0p-53;
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

template <class T>
T* dalloc(size_t n) { return static_cast<T*>(dev_alloc(sizeof(T) * std::max<size_t>(n, 1))); }

}  // namespace

RankModel::RankModel(uint64_t seed) {
  std::vector<float> p(kMlpParams, 0.0f);
  const int dims[5] = {kMlpIn, kMlpHidden, kMlpHidden, kMlpHidden, kMlpOut};
  uint64_t s = seed;
  size_t o = 0;
  for (int l = 0; l < 4; ++l) {
    const double sd = std::sqrt(2.0 / dims[l]);
    for (int e = 0; e < dims[l + 1] * dims[l]; ++e) p[o++] = float(sd * normal(s));
    o += size_t(dims[l + 1]);  // biases stay zero
  }
  params_ = dalloc<float>(kMlpParams);
  mom_ = dalloc<float>(kMlpParams);
  vel_ = dalloc<float>(kMlpParams);
  set_params(p.data());
}

RankModel::~RankModel() {
  dev_free(params_);
  dev_free(mom_);
  dev_free(vel_);
}

void RankModel::set_params(const float* host) {
  cudaStream_t st = stream();
  ok(cudaMemcpyAsync(params_, host, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, st), "h2d params");
  ok(cudaMemsetAsync(mom_, 0, sizeof(float) * kMlpParams, st), "memset");
  ok(cudaMemsetAsync(vel_, 0, sizeof(float) * kMlpParams, st), "memset");
  ok(cudaStreamSynchronize(st), "sync");
  step_ = 0;
}

void RankModel::get_params(float* host) const {
  cudaStream_t st = stream();
  ok(cudaMemcpyAsync(host, params_, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, st), "d2h params");
  ok(cudaStreamSynchronize(st), "sync");
}

void RankModel::predict(const float* X, int64_t n, float* Y) {
  if (n <= 0) return;
  cudaStream_t st = stream();
  float* dX = dalloc<float>(size_t(n) * kMlpIn);
  float* dY = dalloc<float>(size_t(n) * kMlpOut);
  ok(cudaMemcpyAsync(dX, X, sizeof(float) * size_t(n) * kMlpIn, cudaMemcpyHostToDevice, st), "h2d");
  prof_begin(K_MLP, st);
  launch_mlp_forward(params_, dX, n, dY, st);
  prof_end(K_MLP, st, 2.0 * double(n) * double(kMlpParams));
  ok(cudaMemcpyAsync(Y, dY, sizeof(float) * size_t(n) * kMlpOut, cudaMemcpyDeviceToHost, st), "d2h");
  ok(cudaStreamSynchronize(st), "sync");
  dev_free(dX);
  dev_free(dY);
}

double RankModel::gradient(const float* X, const float* T, int64_t n, float* grad) {
  if (n <= 0) throw std::runtime_error("rank model: no samples");
  cudaStream_t st = stream();
  const int slots = mlp_grad_slots(n);
  float* dX = dalloc<float>(size_t(n) * kMlpIn);
  float* dT = dalloc<float>(size_t(n) * kMlpOut);
  float* gp = dalloc<float>(size_t(slots) * kMlpParams);
  float* lp = dalloc<float>(size_t(slots));
  float* dg = dalloc<float>(kMlpParams);
  ok(cudaMemcpyAsync(dX, X, sizeof(float) * size_t(n) * kMlpIn, cudaMemcpyHostToDevice, st), "h2d");
  ok(cudaMemcpyAsync(dT, T, sizeof(float) * size_t(n) * kMlpOut, cudaMemcpyHostToDevice, st), "h2d");
  prof_begin(K_MLP, st);
  launch_mlp_grad(params_, dX, dT, n, gp, lp, st);
  launch_mlp_reduce_adam(params_, mom_, vel_, gp, slots, dg, 0, 0, 0, 0, 0, 1, st);
  prof_end(K_MLP, st, 6.0 * double(n) * double(kMlpParams));
  std::vector<float> lh(static_cast<size_t>(slots));
  ok(cudaMemcpyAsync(grad, dg, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, st), "d2h");
  ok(cudaMemcpyAsync(lh.data(), lp, sizeof(float) * size_t(slots), cudaMemcpyDeviceToHost, st), "d2h");
  ok(cudaStreamSynchronize(st), "sync");
  for (void* p : {static_cast<void*>(dX), static_cast<void*>(dT), static_cast<void*>(gp), static_cast<void*>(lp),
                  static_cast<void*>(dg)})
    dev_free(p);
  double loss = 0;
  for (float v : lh) loss += v;
  return loss;
}

double RankModel::train(const float* X, const float* T, int64_t n, int steps, float lr) {
  if (n <= 0 || steps <= 0) throw std::runtime_error("rank model: no samples or steps");
  cudaStream_t st = stream();
  const int slots = mlp_grad_slots(n);
  float* dX = dalloc<float>(size_t(n) * kMlpIn);
  float* dT = dalloc<float>(size_t(n) * kMlpOut);
  float* gp = dalloc<float>(size_t(slots) * kMlpParams);
  float* lp = dalloc<float>(size_t(slots));
  ok(cudaMemcpyAsync(dX, X, sizeof(float) * size_t(n) * kMlpIn, cudaMemcpyHostToDevice, st), "h2d");
  ok(cudaMemcpyAsync(dT, T, sizeof(float) * size_t(n) * kMlpOut, cudaMemcpyHostToDevice, st), "h2d");
  prof_begin(K_MLP, st);
  for (int it = 0; it < steps; ++it) {
    launch_mlp_grad(params_, dX, dT, n, gp, lp, st);
    ++step_;
    launch_mlp_reduce_adam(params_, mom_, vel_, gp, slots, nullptr, 1, lr, 0.9f, 0.999f, 1e-8f, int(step_), st);
  }
  prof_end(K_MLP, st, 6.0 * double(n) * double(kMlpParams) * steps);
  std::vector<float> lh(static_cast<size_t>(slots));
  ok(cudaMemcpyAsync(lh.data(), lp, sizeof(float) * size_t(slots), cudaMemcpyDeviceToHost, st), "d2h");
  ok(cudaStreamSynchronize(st), "sync");
  for (void* p : {static_cast<void*>(dX), static_cast<void*>(dT), static_cast<void*>(gp), static_cast<void*>(lp)})
    dev_free(p);
  double loss = 0;
  for (float v : lh) loss += v;
  return loss;
}

std::vector<int64_t> MlpPolicy::widths(const TensorMeta& m, const History& last, int64_t chi) {
  if (!model) throw std::runtime_error("MlpPolicy without a model");
  const size_t n = m.sectors.size();
  std::vector<float> X, Y(n * kMlpOut);
  sector_features(m, last, chi, X);
  model->predict(X.data(), int64_t(n), Y.data());
  std::vector<int64_t> w(n, 0);
  for (size_t i = 0; i < n; ++i) {
    if (last.find(m.sectors[i]) == last.end()) continue;  // never seen: exact
    const double k = std::max(0.0, std::exp2(double(Y[i * kMlpOut])) - 1.0);
    const double p = std::max(0.0, std::exp2(double(Y[i * kMlpOut + 1])) - 1.0);
    w[i] = int64_t(std::ceil(k * (1.0 + margin))) + std::max<int64_t>(min_oversample, int64_t(std::ceil(p)));
  }
  return w;
}

}  // namespace xgb
