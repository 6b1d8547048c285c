// Rank-predictor MLP: forward, backward (MSE) and Adam kernels, FP32.
// Reductions over the batch are done by one thread per parameter walking the
// samples in order, so gradients are deterministic.
#include <cmath>

#include "rank_mlp.hpp"

namespace udmrg {

namespace {

constexpr int H = kRankHidden, IN = kRankIn;

__device__ __forceinline__ float hidden(const float *__restrict__ p, const float *__restrict__ x,
                                        int j) {
  const float *w = p + j * IN;
  float s = p[H * IN + j];
  for (int k = 0; k < IN; ++k) s = fmaf(w[k], x[k], s);
  return s;
}

// y[i] = w2 . relu(W1 x_i + b1) + b2; optionally stores the pre-activations
__global__ void mlp_forward_kernel(const float *__restrict__ p, const float *__restrict__ x,
                                   int64_t n, float *__restrict__ y, float *__restrict__ pre) {
  __shared__ float red[H];
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
    const int j = threadIdx.x;  // blockDim.x == H
    const float a = hidden(p, x + i * IN, j);
    if (pre) pre[i * H + j] = a;
    red[j] = fmaxf(a, 0.f) * p[H * IN + H + j];
    __syncthreads();
    for (int s = H / 2; s > 0; s >>= 1) {
      if (j < s) red[j] += red[j + s];
      __syncthreads();
    }
    if (j == 0) y[i] = red[0] + p[H * IN + 2 * H];
    __syncthreads();
  }
}

// dy[i] = 2 (y_i - t_i) / n, per-sample squared error in err[i]
__global__ void mlp_dy_kernel(const float *__restrict__ y, const float *__restrict__ t, int64_t n,
                              float *__restrict__ dy, float *__restrict__ err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float d = y[i] - t[i];
    dy[i] = 2.f * d / (float)n;
    err[i] = d * d;
  }
}

// gradient of every parameter; thread g owns parameter g
__global__ void mlp_grad_kernel(const float *__restrict__ p, const float *__restrict__ x,
                                const float *__restrict__ pre, const float *__restrict__ dy,
                                int64_t n, float *__restrict__ grad) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= kRankParams) return;
  double acc = 0.0;
  if (g < H * IN) {  // W1[j][k]
    const int j = g / IN, k = g % IN;
    const float w2j = p[H * IN + H + j];
    for (int64_t i = 0; i < n; ++i)
      if (pre[i * H + j] > 0.f) acc += (double)dy[i] * w2j * x[i * IN + k];
  } else if (g < H * IN + H) {  // b1[j]
    const int j = g - H * IN;
    const float w2j = p[H * IN + H + j];
    for (int64_t i = 0; i < n; ++i)
      if (pre[i * H + j] > 0.f) acc += (double)dy[i] * w2j;
  } else if (g < H * IN + 2 * H) {  // w2[j]
    const int j = g - H * IN - H;
    for (int64_t i = 0; i < n; ++i) acc += (double)dy[i] * fmaxf(pre[i * H + j], 0.f);
  } else {  // b2
    for (int64_t i = 0; i < n; ++i) acc += dy[i];
  }
  grad[g] = (float)acc;
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g,
                            float *__restrict__ m, float *__restrict__ v, int n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  m[i] = b1 * m[i] + (1.f - b1) * g[i];
  v[i] = b2 * v[i] + (1.f - b2) * g[i] * g[i];
  const float mh = m[i] / c1, vh = v[i] / c2;
  p[i] -= lr * mh / (sqrtf(vh) + eps);
}

// deterministic initialisation: uniform(-a, a) per layer (He-style scale)
__global__ void mlp_init_kernel(float *__restrict__ p, uint64_t seed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kRankParams) return;
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  const float u = (float)((z >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f;
  if (i < H * IN)
    p[i] = u * sqrtf(6.f / IN);
  else if (i < H * IN + H)
    p[i] = 0.f;
  else if (i < H * IN + 2 * H)
    p[i] = u * sqrtf(6.f / H);
  else
    p[i] = 0.f;
}

}  // namespace

RankModel::RankModel(Ctx &c, uint64_t seed) : ctx(&c) {
  params = (float *)c.alloc(kRankParams * sizeof(float));
  grad = (float *)c.alloc(kRankParams * sizeof(float));
  m = (float *)c.alloc(kRankParams * sizeof(float));
  v = (float *)c.alloc(kRankParams * sizeof(float));
  UDMRG_CHECK_CUDA(cudaMemsetAsync(m, 0, kRankParams * sizeof(float), c.stream));
  UDMRG_CHECK_CUDA(cudaMemsetAsync(v, 0, kRankParams * sizeof(float), c.stream));
  mlp_init_kernel<<<(kRankParams + 255) / 256, 256, 0, c.stream>>>(params, seed);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  c.launches++;
}

RankModel::~RankModel() {
  for (float *p : {params, grad, m, v}) ctx->free(p);
}

void RankModel::predict(const float *x, int64_t n, float *y) {
  if (n == 0) return;
  const int grid = (int)std::min<int64_t>(n, 8 * ctx->num_sms);
  mlp_forward_kernel<<<grid, H, 0, ctx->stream>>>(params, x, n, y, nullptr);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx->launches++;
}

float RankModel::loss_grad(const float *x, const float *t, int64_t n) {
  UDMRG_REQUIRE(n > 0, "rank model: empty batch");
  DeviceScratch s(*ctx);
  float *y = s.get<float>(n), *pre = s.get<float>(n * H), *dy = s.get<float>(n),
        *err = s.get<float>(n);
  const int grid = (int)std::min<int64_t>(n, 8 * ctx->num_sms);
  mlp_forward_kernel<<<grid, H, 0, ctx->stream>>>(params, x, n, y, pre);
  mlp_dy_kernel<<<(int)std::min<int64_t>((n + 255) / 256, 1024), 256, 0, ctx->stream>>>(y, t, n,
                                                                                      dy, err);
  mlp_grad_kernel<<<(kRankParams + 127) / 128, 128, 0, ctx->stream>>>(params, x, pre, dy, n, grad);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx->launches += 3;
  std::vector<float> h(n);
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(h.data(), err, n * sizeof(float), cudaMemcpyDeviceToHost,
                                   ctx->stream));
  ctx->sync();
  double l = 0;
  for (float e : h) l += e;
  return (float)(l / n);
}

void RankModel::adam(float lr, float b1, float b2, float eps) {
  ++step;
  const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
  adam_kernel<<<(kRankParams + 255) / 256, 256, 0, ctx->stream>>>(params, grad, m, v, kRankParams,
                                                                 lr, b1, b2, eps, c1, c2);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx->launches++;
}

void rank_features(const std::vector<double> &sv, const QN &qn, const QN &top, double trunc_err,
                   int64_t prev_kept, double prev_cut, double growth, float *out) {
  for (int i = 0; i < kRankSv; ++i) {
    const double s = i < (int)sv.size() ? sv[i] : 0.0;
    out[i] = (float)(std::log10(std::max(s, 1e-20)) / 10.0);
  }
  out[kRankSv] = (float)((qn.v[0] - top.v[0]) / 4.0);
  out[kRankSv + 1] = (float)((qn.v[1] - top.v[1]) / 4.0);
  out[kRankSv + 2] = (float)(std::log10(std::max(trunc_err, 1e-30)) / 10.0);
  out[kRankSv + 3] = (float)(std::log2(1.0 + (double)prev_kept) / 10.0);
  out[kRankSv + 4] = (float)(std::log10(std::max(prev_cut, 1e-20)) / 10.0);
  out[kRankSv + 5] = (float)growth;
}

}  // namespace udmrg
