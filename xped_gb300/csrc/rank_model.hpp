// Learned sketch widths for the randomized projector SVD: a small MLP
// (features of one sector -> predicted kept count and oversampling), trained
// and evaluated on the device by the kernels of mlp.cu.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "tensor.hpp"

namespace xgb {

static_assert(kFeatures == kMlpIn, "feature count of the rank predictor");

class RankModel {
 public:
  explicit RankModel(uint64_t seed);  // He-normal weights, zero biases
  ~RankModel();
  RankModel(const RankModel&) = delete;
  RankModel& operator=(const RankModel&) = delete;

  void set_params(const float* host);
  void get_params(float* host) const;
  // Y (n x kMlpOut) = net(X (n x kMlpIn)); host arrays
  void predict(const float* X, int64_t n, float* Y);
  // mean-squared-error loss and its gradient w.r.t. the packed parameters
  double gradient(const float* X, const float* T, int64_t n, float* grad);
  // `steps` full-batch Adam steps on (X, T); returns the loss before the last step
  double train(const float* X, const float* T, int64_t n, int steps, float lr);
  int64_t adam_steps() const { return step_; }

 private:
  float *params_ = nullptr, *mom_ = nullptr, *vel_ = nullptr;
  int64_t step_ = 0;
};

// Widths = ceil(2^y0 - 1) * (1 + margin) + ceil(2^y1 - 1) with (y0, y1) the
// model's prediction of log2(1 + kept) and log2(1 + oversampling); sectors
// without history are decomposed exactly.
struct MlpPolicy : WidthPolicy {
  std::shared_ptr<RankModel> model;
  double margin = 0.0;
  int64_t min_oversample = 2;
  std::vector<int64_t> widths(const TensorMeta& m, const History& last, int64_t chi) override;
};

}  // namespace xgb
