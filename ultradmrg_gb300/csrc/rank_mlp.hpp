// Learned per-sector rank predictor for the randomized truncated SVD.
//
// A two-layer perceptron y = w2 . relu(W1 x + b1) + b2 (FP32) maps the
// spectrum a bond sector had at the previous visit of its bond to the number
// of states the truncation keeps now, as y = log2(1 + kept).  Features
// (kRankIn = 70): log10 of the leading 64 singular values of the sector
// (floored at 1e-20, divided by 10), the two components of the sector QN
// relative to the bond's dominant sector (divided by 4), log10 of the
// truncation target (/10), log2(1 + previous kept count) (/10), log10 of the
// smallest singular value kept on the whole bond at the previous visit (/10)
// and log2(Dmax / previous bond dimension) (the room the bond has to grow).
// Training and inference run on the device with this library's kernels
// (forward, backward of the mean squared error, Adam).
#pragma once

#include "btensor.hpp"

namespace udmrg {

constexpr int kRankIn = 70;
constexpr int kRankHidden = 128;
constexpr int kRankSv = 64;
constexpr int kRankParams = kRankHidden * kRankIn + kRankHidden + kRankHidden + 1;

struct RankModel {
  Ctx *ctx = nullptr;
  float *params = nullptr;  // W1 (H x In, row-major) | b1 (H) | w2 (H) | b2 (1)
  float *grad = nullptr;
  float *m = nullptr, *v = nullptr;  // Adam moments
  int64_t step = 0;
  explicit RankModel(Ctx &c, uint64_t seed);
  ~RankModel();
  // y[i] for n samples (x: device, n x kRankIn)
  void predict(const float *x, int64_t n, float *y);
  // loss and gradient (into grad) of mean((y - t)^2) over n samples (device)
  float loss_grad(const float *x, const float *t, int64_t n);
  void adam(float lr, float b1 = 0.9f, float b2 = 0.999f, float eps = 1e-8f);
};

// Host-side feature vector of one sector.
void rank_features(const std::vector<double> &prev_svals, const QN &qn, const QN &top_qn,
                   double trunc_err, int64_t prev_kept, double prev_cut, double growth,
                   float *out);

}  // namespace udmrg
