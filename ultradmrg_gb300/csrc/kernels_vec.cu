// Krylov vector kernels (HBM-bound): dot products, the fused three-term
// Lanczos update with its norm, scaling, multi-vector combinations, conjugation.
// Reductions are two-stage with a fixed grid, so results are deterministic.
#include "vecops.hpp"

namespace udmrg {

namespace {

constexpr int kRedThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Sum of `nv` per-thread values across the block; result in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *out) {
  __shared__ double sh[NV][kRedThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double s = warp_sum(v[i]);
    if (lane == 0) sh[i][w] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      double s = 0;
      for (int j = 0; j < kRedThreads / 32; ++j) s += sh[i][j];
      out[i] = s;
    }
  }
}

// partial[b] = sum over this block's slice of conj(x) * y (re, im)
__global__ void dot_partial_kernel(const double *__restrict__ x, const double *__restrict__ y,
                                   int64_t n, int cplx, double *__restrict__ partial) {
  double v[2] = {0.0, 0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (!cplx) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
      v[0] = fma(x[i], y[i], v[0]);
  } else {
    const double2 *x2 = (const double2 *)x, *y2 = (const double2 *)y;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
      double2 a = x2[i], b = y2[i];
      v[0] = fma(a.x, b.x, fma(a.y, b.y, v[0]));
      v[1] = fma(a.x, b.y, fma(-a.y, b.x, v[1]));
    }
  }
  double out[2];
  block_sum<2>(v, out);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = out[0];
    partial[2 * blockIdx.x + 1] = out[1];
  }
}

// Sums `nb` partial pairs into res[0..1] in a fixed order.
__global__ void finish_sum_kernel(const double *__restrict__ partial, int nb, int width,
                                  double *__restrict__ res) {
  double v[2] = {0.0, 0.0};
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    v[0] += partial[width * i];
    if (width > 1) v[1] += partial[width * i + 1];
  }
  double out[2];
  block_sum<2>(v, out);
  if (threadIdx.x == 0) {
    res[0] = out[0];
    res[1] = out[1];
  }
}

// g = g - c1 * v1 - c2 * v2 (real coefficients), partial[b] = |g|^2 slice
__global__ void lanczos_update_kernel(double *__restrict__ g, const double *__restrict__ v1,
                                      const double *__restrict__ v2, double c1, double c2,
                                      int64_t n, double *__restrict__ partial) {
  double v[1] = {0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    double x = g[i];
    x = fma(-c1, v1[i], x);
    if (v2) x = fma(-c2, v2[i], x);
    g[i] = x;
    v[0] = fma(x, x, v[0]);
  }
  double out[1];
  block_sum<1>(v, out);
  if (threadIdx.x == 0) partial[blockIdx.x] = out[0];
}

__global__ void scale_kernel(double *__restrict__ x, int64_t n, double s) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) x[i] *= s;
}

// out[i] = sum_j coef[j] * vec[j][i]; complex when cplx (coef interleaved)
__global__ void lincomb_kernel(double *__restrict__ out, const double *const *__restrict__ vecs,
                               const double *__restrict__ coef, int m, int64_t n, int cplx) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (!cplx) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
      double s = 0.0;
      for (int j = 0; j < m; ++j) s = fma(coef[j], vecs[j][i], s);
      out[i] = s;
    }
  } else {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
      double sr = 0.0, si = 0.0;
      for (int j = 0; j < m; ++j) {
        const double2 v = ((const double2 *)vecs[j])[i];
        const double cr = coef[2 * j], ci = coef[2 * j + 1];
        sr = fma(cr, v.x, fma(-ci, v.y, sr));
        si = fma(cr, v.y, fma(ci, v.x, si));
      }
      ((double2 *)out)[i] = make_double2(sr, si);
    }
  }
}

__global__ void conj_kernel(double2 *__restrict__ x, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    x[i].y = -x[i].y;
}

__global__ void real_to_complex_kernel(const double *__restrict__ x, double2 *__restrict__ y,
                                       int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = make_double2(x[i], 0.0);
}

int red_grid(const Ctx &ctx, int64_t n) {
  int64_t g = (n + kRedThreads - 1) / kRedThreads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 4 * ctx.num_sms));
}

int ew_grid(const Ctx &ctx, int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 8 * ctx.num_sms));
}

}  // namespace

VecWork::VecWork(Ctx &c) : ctx(c) {
  partial = (double *)ctx.alloc(sizeof(double) * 2 * 8 * 1024);
  result = (double *)ctx.alloc(sizeof(double) * 2 * kMaxVecs);
  ptrs = (const double **)ctx.alloc(sizeof(double *) * kMaxVecs);
  coefs = (double *)ctx.alloc(sizeof(double) * 2 * kMaxVecs);
}

VecWork::~VecWork() {
  ctx.free(partial);
  ctx.free(result);
  ctx.free((void *)ptrs);
  ctx.free(coefs);
}

void dot_async(VecWork &w, const double *x, const double *y, int64_t n, bool cplx, double *dres) {
  Ctx &ctx = w.ctx;
  const int g = red_grid(ctx, n);
  dot_partial_kernel<<<g, kRedThreads, 0, ctx.stream>>>(x, y, n, cplx ? 1 : 0, w.partial);
  finish_sum_kernel<<<1, kRedThreads, 0, ctx.stream>>>(w.partial, g, 2, dres);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches += 2;
}

std::complex<double> dot(VecWork &w, const double *x, const double *y, int64_t n, bool cplx) {
  dot_async(w, x, y, n, cplx, w.result);
  double *h = w.ctx.host_scratch(2);
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(h, w.result, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                   w.ctx.stream));
  w.ctx.sync();
  return {h[0], h[1]};
}

void lanczos_update_async(VecWork &w, double *g, const double *v1, const double *v2, double c1,
                          double c2, int64_t n_doubles, double *dnorm2) {
  Ctx &ctx = w.ctx;
  const int gr = red_grid(ctx, n_doubles);
  lanczos_update_kernel<<<gr, kRedThreads, 0, ctx.stream>>>(g, v1, v2, c1, c2, n_doubles,
                                                             w.partial);
  finish_sum_kernel<<<1, kRedThreads, 0, ctx.stream>>>(w.partial, gr, 1, dnorm2);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches += 2;
}

double norm2(VecWork &w, const double *x, int64_t n_doubles) {
  return dot(w, x, x, n_doubles, false).real();
}

void scale(Ctx &ctx, double *x, int64_t n_doubles, double s) {
  if (n_doubles == 0) return;
  scale_kernel<<<ew_grid(ctx, n_doubles), 256, 0, ctx.stream>>>(x, n_doubles, s);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

void lincomb(VecWork &w, double *out, const std::vector<const double *> &vecs,
             const std::vector<double> &coef_interleaved, int64_t n, bool cplx) {
  Ctx &ctx = w.ctx;
  const int m = (int)vecs.size();
  UDMRG_REQUIRE(m <= kMaxVecs, "lincomb: too many vectors");
  if (n == 0) return;
  double *h = ctx.host_scratch(2 * kMaxVecs + kMaxVecs);
  // stage coefficients and pointers through pinned memory (one copy each)
  std::memcpy(h, coef_interleaved.data(), sizeof(double) * coef_interleaved.size());
  std::memcpy(h + 2 * kMaxVecs, vecs.data(), sizeof(double *) * m);
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(w.coefs, h, sizeof(double) * coef_interleaved.size(),
                                   cudaMemcpyHostToDevice, ctx.stream));
  UDMRG_CHECK_CUDA(cudaMemcpyAsync((void *)w.ptrs, h + 2 * kMaxVecs, sizeof(double *) * m,
                                   cudaMemcpyHostToDevice, ctx.stream));
  lincomb_kernel<<<ew_grid(ctx, n), 256, 0, ctx.stream>>>(out, w.ptrs, w.coefs, m, n,
                                                          cplx ? 1 : 0);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
  ctx.sync();  // pinned staging buffer is reused by the next call
}

void conj_inplace(Ctx &ctx, double *x, int64_t n_cplx) {
  if (n_cplx == 0) return;
  conj_kernel<<<ew_grid(ctx, n_cplx), 256, 0, ctx.stream>>>((double2 *)x, n_cplx);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

void real_to_complex(Ctx &ctx, const double *x, double *y, int64_t n) {
  if (n == 0) return;
  real_to_complex_kernel<<<ew_grid(ctx, n), 256, 0, ctx.stream>>>(x, (double2 *)y, n);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

}  // namespace udmrg
