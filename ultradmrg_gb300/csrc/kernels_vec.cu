// Krylov vector kernels (HBM-bound): dot products, the fused three-term
// Lanczos update with its norm, scaling, multi-vector combinations, conjugation.
// Reductions are two-stage with a fixed grid, so results are deterministic.
#include <type_traits>

#include "vecops.hpp"

#include <algorithm>
#include <cmath>
#include <vector>

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

// ---- device-resident Krylov step ----

constexpr int kMdThreads = 256;
constexpr int kMdWarps = kMdThreads / 32;
constexpr int kMdPer = 4;  // elements of g per lane and chunk, held in registers

// Second Gram-Schmidt pass only where the first one removed a large part of
// the vector: |g|^2 after the pass < 1/2 |g|^2 before it (the classical
// "twice is enough" test, eta = 1/sqrt(2)).  gate == nullptr: always run.
__device__ __forceinline__ bool gate_open(const double *gate) {
  return gate == nullptr || gate[1] < 0.5 * gate[0];
}

// partial[(j * gridDim.x + b) * 2 + {0,1}] = block b's share of <v_j | g>,
// j < m = step + 1.  For each group of G vectors a lane streams its grid-strided
// elements of g and of the group's vectors, keeping G running sums in
// registers (no reduction inside the stream); at the end of the group the
// sums are reduced over the warp and over the block's warps (shared memory,
// 2 * m * kMdWarps doubles).  g is read once per group.
template <bool CPLX>
__global__ void __launch_bounds__(kMdThreads)
    multidot_kernel(const double *const *__restrict__ vecs, const int *__restrict__ step,
                    const double *__restrict__ g, int64_t n, double *__restrict__ partial,
                    const double *__restrict__ gate) {
  if (!gate_open(gate)) return;
  const int m = *step + 1;
  constexpr int G = CPLX ? 4 : 8;  // vectors per group
  constexpr int U = 2;             // elements per lane per step (independent loads)
  using E = typename std::conditional<CPLX, double2, double>::type;
  extern __shared__ double md_sm[];  // [m][kMdWarps][2]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const E *ge = (const E *)g;
  const int64_t stride = (int64_t)gridDim.x * kMdThreads;
  const int64_t i0 = (int64_t)blockIdx.x * kMdThreads + threadIdx.x;
  for (int j0 = 0; j0 < m; j0 += G) {
    const E *v[G];
#pragma unroll
    for (int q = 0; q < G; ++q) v[q] = (const E *)vecs[j0 + q < m ? j0 + q : j0];
    double sr[G], si[G];
#pragma unroll
    for (int q = 0; q < G; ++q) sr[q] = si[q] = 0.0;
    for (int64_t i = i0; i < n; i += U * stride) {
      E gv[U], vv[U][G];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t ii = i + u * stride;
        const bool ok = ii < n;
        if constexpr (CPLX)
          gv[u] = ok ? ge[ii] : make_double2(0.0, 0.0);
        else
          gv[u] = ok ? ge[ii] : 0.0;
#pragma unroll
        for (int q = 0; q < G; ++q) {
          if constexpr (CPLX)
            vv[u][q] = ok ? v[q][ii] : make_double2(0.0, 0.0);
          else
            vv[u][q] = ok ? v[q][ii] : 0.0;
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int q = 0; q < G; ++q) {
          if constexpr (CPLX) {  // conj(v) g
            sr[q] = fma(vv[u][q].x, gv[u].x, fma(vv[u][q].y, gv[u].y, sr[q]));
            si[q] = fma(vv[u][q].x, gv[u].y, fma(-vv[u][q].y, gv[u].x, si[q]));
          } else {
            sr[q] = fma(vv[u][q], gv[u], sr[q]);
          }
        }
    }
#pragma unroll
    for (int q = 0; q < G; ++q) {
      const double a = warp_sum(sr[q]);
      const double b = CPLX ? warp_sum(si[q]) : 0.0;
      if (lane == 0 && j0 + q < m) {
        md_sm[(2 * (j0 + q)) * kMdWarps + 2 * warp] = a;
        md_sm[(2 * (j0 + q)) * kMdWarps + 2 * warp + 1] = b;
      }
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < m; j += kMdThreads) {
    double sr = 0.0, si = 0.0;
    for (int w = 0; w < kMdWarps; ++w) {
      sr += md_sm[(2 * j) * kMdWarps + 2 * w];
      si += md_sm[(2 * j) * kMdWarps + 2 * w + 1];
    }
    partial[((int64_t)j * gridDim.x + blockIdx.x) * 2] = sr;
    partial[((int64_t)j * gridDim.x + blockIdx.x) * 2 + 1] = si;
  }
}

// res[2 j .. 2 j + 1] = sum over the nb partial pairs of row j (block j, fixed
// order) for j <= step; the grid covers the largest step, later blocks return
__global__ void multidot_finish_kernel(const double *__restrict__ partial, int nb,
                                       double *__restrict__ res, const int *__restrict__ step,
                                       const double *__restrict__ gate) {
  if (!gate_open(gate) || (int)blockIdx.x > *step) return;
  const double *p = partial + (int64_t)blockIdx.x * nb * 2;
  double v[2] = {0.0, 0.0};
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    v[0] += p[2 * i];
    v[1] += p[2 * i + 1];
  }
  double out[2];
  block_sum<2>(v, out);
  if (threadIdx.x == 0) {
    res[2 * blockIdx.x] = out[0];
    res[2 * blockIdx.x + 1] = out[1];
  }
}

// g -= sum_{j <= step} c_j v_j (complex c_j when CPLX), partial[b] = |g|^2
// slice.  The vector loop is unrolled by 8 with two accumulators, so eight loads are in
// flight per element.
template <bool CPLX>
__global__ void project_kernel(double *__restrict__ g, const double *const *__restrict__ vecs,
                               const double *__restrict__ c, const int *__restrict__ step,
                               int64_t n, double *__restrict__ partial,
                               const double *__restrict__ gate) {
  if (!gate_open(gate)) return;
  const int m = *step + 1;
  __shared__ double cs[2 * kMaxVecs];
  __shared__ const double *vs[kMaxVecs];
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    cs[2 * j] = c[2 * j];
    cs[2 * j + 1] = c[2 * j + 1];
    vs[j] = vecs[j];
  }
  __syncthreads();
  double v[1] = {0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    if constexpr (CPLX) {
      double2 x = ((double2 *)g)[i], y = make_double2(0.0, 0.0);
#pragma unroll 8
      for (int j = 0; j < m; ++j) {
        const double2 a = ((const double2 *)vs[j])[i];
        const double cr = cs[2 * j], ci = cs[2 * j + 1];
        if (j & 1) {
          y.x = fma(cr, a.x, fma(-ci, a.y, y.x));
          y.y = fma(cr, a.y, fma(ci, a.x, y.y));
        } else {
          x.x = fma(-cr, a.x, fma(ci, a.y, x.x));
          x.y = fma(-cr, a.y, fma(-ci, a.x, x.y));
        }
      }
      x.x -= y.x;
      x.y -= y.y;
      ((double2 *)g)[i] = x;
      v[0] = fma(x.x, x.x, fma(x.y, x.y, v[0]));
    } else {
      double x = g[i], y = 0.0;
#pragma unroll 8
      for (int j = 0; j < m; ++j) {
        if (j & 1)
          y = fma(cs[2 * j], vs[j][i], y);
        else
          x = fma(-cs[2 * j], vs[j][i], x);
      }
      x -= y;
      g[i] = x;
      v[0] = fma(x, x, v[0]);
    }
  }
  double out[1];
  block_sum<1>(v, out);
  if (threadIdx.x == 0) partial[blockIdx.x] = out[0];
}

// nrm2[step + 1] = sum of the nb partials (fixed order); with keep, keep[0] =
// its previous value (|g|^2 before a Gram-Schmidt pass) and keep[1] = the sum
__global__ void norm_finish_kernel(const double *__restrict__ partial, int nb,
                                   double *__restrict__ nrm2, const int *__restrict__ step,
                                   double *__restrict__ keep, const double *__restrict__ gate) {
  if (!gate_open(gate)) return;
  double *res = nrm2 + *step + 1;
  double v[1] = {0.0};
  for (int i = threadIdx.x; i < nb; i += blockDim.x) v[0] += partial[i];
  double out[1];
  block_sum<1>(v, out);
  if (threadIdx.x == 0) {
    if (keep) {
      keep[0] = res[0];
      keep[1] = out[0];
    }
    res[0] = out[0];
  }
}

// s = step: g = g - Re(alpha[s]) v1 - sqrt(nrm2[s]) v_{s-1} (the second term
// when s > 0), partial = |g|^2 slices
__global__ void krylov_update_kernel(double *__restrict__ g, const double *__restrict__ v1,
                                     const double *const *__restrict__ vecs,
                                     const int *__restrict__ step,
                                     const double *__restrict__ alpha,
                                     const double *__restrict__ nrm2, int64_t n,
                                     double *__restrict__ partial) {
  const int s = *step;
  const double *v2 = s > 0 ? vecs[s - 1] : nullptr;
  const double c1 = alpha[2 * s], c2 = v2 ? sqrt(nrm2[s]) : 0.0;
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

// s = step: v_s = y / sqrt(nrm2[s]) (y unchanged when the norm is zero),
// written to the registered basis vector s and to x
__global__ void krylov_normalise_kernel(const double *__restrict__ y, double *__restrict__ x,
                                        const double *const *__restrict__ vecs,
                                        const int *__restrict__ step,
                                        const double *__restrict__ nrm2, int64_t n) {
  const int s = *step;
  const double nr = sqrt(nrm2[s]);
  const double sc = nr == 0.0 ? 1.0 : 1.0 / nr;
  double *v = const_cast<double *>(vecs[s]);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const double t = nr == 0.0 ? y[i] : y[i] * sc;
    x[i] = t;
    v[i] = t;
  }
}

// res[stride * step + offset + {0, 1}] = the sum of nb partials of `width`
// values (the second only when width > 1), fixed order
__global__ void finish_step_kernel(const double *__restrict__ partial, int nb, int width,
                                   double *__restrict__ res, const int *__restrict__ step,
                                   int stride, int offset) {
  double v[2] = {0.0, 0.0};
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    v[0] += partial[width * i];
    if (width > 1) v[1] += partial[width * i + 1];
  }
  double out[2];
  block_sum<2>(v, out);
  if (threadIdx.x == 0) {
    double *r = res + (int64_t)stride * *step + offset;
    r[0] = out[0];
    if (width > 1) r[1] = out[1];
  }
}

// host-visible results of step s, then the step counter moves on
__global__ void krylov_publish_kernel(const double *__restrict__ alpha,
                                      const double *__restrict__ nrm2, int *__restrict__ step,
                                      double *__restrict__ hres) {
  const int s = *step;
  hres[0] = alpha[2 * s];
  hres[1] = nrm2[s + 1];
  hres[2] = nrm2[s];
  *step = s + 1;
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

KrylovWork::KrylovWork(Ctx &c, int64_t n_elems, bool complex_data, int64_t max_steps)
    : ctx(c), n(n_elems), cplx(complex_data) {
  mcap = (int)std::max<int64_t>(1, std::min<int64_t>(max_steps + 1, kMaxVecs));
  const int64_t blocks = (n + kMdThreads * kMdPer - 1) / (kMdThreads * kMdPer);
  nb = (int)std::max<int64_t>(1, std::min<int64_t>(blocks, 2 * ctx.num_sms));
  partial = (double *)ctx.alloc(sizeof(double) * 2 * (size_t)mcap * nb);
  gate = (double *)ctx.alloc(sizeof(double) * 2);
  const int msm = (int)(sizeof(double) * 2 * kMaxVecs * kMdWarps);
  UDMRG_CHECK_CUDA(cudaFuncSetAttribute(multidot_kernel<true>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, msm));
  UDMRG_CHECK_CUDA(cudaFuncSetAttribute(multidot_kernel<false>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, msm));
  red = (double *)ctx.alloc(sizeof(double) * 8 * 1024);
  coef = (double *)ctx.alloc(sizeof(double) * 2 * kMaxVecs);
  alpha = (double *)ctx.alloc(sizeof(double) * 2 * kMaxVecs);
  nrm2 = (double *)ctx.alloc(sizeof(double) * (kMaxVecs + 2));
  ptrs = (const double **)ctx.alloc(sizeof(double *) * kMaxVecs);
  step = (int *)ctx.alloc(sizeof(int));
  const size_t vbytes = sizeof(double) * std::max<int64_t>(1, n * (cplx ? 2 : 1));
  X = (double *)ctx.alloc(vbytes);
  Y = (double *)ctx.alloc(vbytes);
  UDMRG_CHECK_CUDA(cudaMallocHost((void **)&hptrs, sizeof(double *) * kMaxVecs));
  UDMRG_CHECK_CUDA(cudaHostAlloc((void **)&hres, sizeof(double) * 4, cudaHostAllocMapped));
  UDMRG_CHECK_CUDA(cudaHostGetDevicePointer((void **)&dres, hres, 0));
}

KrylovWork::~KrylovWork() {
  cudaStreamSynchronize(ctx.stream);  // pinned sources of queued copies
  cudaFreeHost((void *)hptrs);
  cudaFreeHost(hres);
  ctx.free(partial);
  ctx.free(gate);
  ctx.free(red);
  ctx.free(coef);
  ctx.free(alpha);
  ctx.free(nrm2);
  ctx.free((void *)ptrs);
  ctx.free(step);
  ctx.free(X);
  ctx.free(Y);
}

void KrylovWork::push(int j, const double *v) {
  UDMRG_REQUIRE(j < mcap, "Krylov basis: more vectors than the solve's step limit");
  hptrs[j] = v;
  UDMRG_CHECK_CUDA(cudaMemcpyAsync((void *)(ptrs + j), (const void *)(hptrs + j),
                                   sizeof(double *), cudaMemcpyHostToDevice, ctx.stream));
}

void krylov_begin(KrylovWork &k, const double *v0) {
  Ctx &ctx = k.ctx;
  const int64_t nd = k.n * (k.cplx ? 2 : 1);
  if (nd > 0)
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(k.Y, v0, nd * sizeof(double), cudaMemcpyDeviceToDevice,
                                     ctx.stream));
  UDMRG_CHECK_CUDA(cudaMemsetAsync(k.step, 0, sizeof(int), ctx.stream));
  const int g = red_grid(ctx, nd);
  dot_partial_kernel<<<g, kRedThreads, 0, ctx.stream>>>(k.Y, k.Y, nd, 0, k.red);
  // the partials are (re, im) pairs: nrm2[0] = |v0|^2, nrm2[1] = 0 (step 0 overwrites it)
  finish_step_kernel<<<1, kRedThreads, 0, ctx.stream>>>(k.red, g, 2, k.nrm2, k.step, 1, 0);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches += 2;
}

void krylov_normalise(KrylovWork &k) {
  Ctx &ctx = k.ctx;
  const int64_t nd = k.n * (k.cplx ? 2 : 1);
  krylov_normalise_kernel<<<ew_grid(ctx, nd), 256, 0, ctx.stream>>>(k.Y, k.X, k.ptrs, k.step,
                                                                     k.nrm2, nd);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

void krylov_alpha(KrylovWork &k) {
  Ctx &ctx = k.ctx;
  const int g = red_grid(ctx, k.n);
  dot_partial_kernel<<<g, kRedThreads, 0, ctx.stream>>>(k.X, k.Y, k.n, k.cplx ? 1 : 0, k.red);
  finish_step_kernel<<<1, kRedThreads, 0, ctx.stream>>>(k.red, g, 2, k.alpha, k.step, 2, 0);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches += 2;
}

void krylov_update(KrylovWork &k) {
  Ctx &ctx = k.ctx;
  const int64_t nd = k.n * (k.cplx ? 2 : 1);
  const int gr = red_grid(ctx, nd);
  krylov_update_kernel<<<gr, kRedThreads, 0, ctx.stream>>>(k.Y, k.X, k.ptrs, k.step, k.alpha,
                                                           k.nrm2, nd, k.red);
  finish_step_kernel<<<1, kRedThreads, 0, ctx.stream>>>(k.red, gr, 1, k.nrm2, k.step, 1, 1);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches += 2;
}

void krylov_project(KrylovWork &k, bool second) {
  Ctx &ctx = k.ctx;
  // gate[0] = |g|^2 before the first pass, gate[1] = after it (k.gate has
  // the two slots for the current step)
  const double *gate = second ? k.gate : nullptr;
  // shared memory for the largest basis of the solve (the step is read on the device)
  const size_t msm = sizeof(double) * 2 * (size_t)k.mcap * kMdWarps;
  if (k.cplx)
    multidot_kernel<true><<<k.nb, kMdThreads, msm, ctx.stream>>>(k.ptrs, k.step, k.Y, k.n,
                                                                 k.partial, gate);
  else
    multidot_kernel<false><<<k.nb, kMdThreads, msm, ctx.stream>>>(k.ptrs, k.step, k.Y, k.n,
                                                                  k.partial, gate);
  multidot_finish_kernel<<<k.mcap, kRedThreads, 0, ctx.stream>>>(k.partial, k.nb, k.coef,
                                                                  k.step, gate);
  const int gr = red_grid(ctx, k.n);
  if (k.cplx)
    project_kernel<true><<<gr, kRedThreads, 0, ctx.stream>>>(k.Y, k.ptrs, k.coef, k.step, k.n,
                                                             k.red, gate);
  else
    project_kernel<false><<<gr, kRedThreads, 0, ctx.stream>>>(k.Y, k.ptrs, k.coef, k.step, k.n,
                                                              k.red, gate);
  // both passes end in nrm2[s+1]; the first also sets gate = {before, after}
  norm_finish_kernel<<<1, kRedThreads, 0, ctx.stream>>>(k.red, gr, k.nrm2, k.step,
                                                        second ? nullptr : k.gate, gate);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches += 4;
}

namespace {
// uniform deviates in [-w, w] from a counter hash (probe data only)
__global__ void probe_fill_kernel(double *__restrict__ x, int64_t n, uint64_t seed, double w) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    uint64_t h = seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(i + 1));
    h = (h ^ (h >> 30)) * 0xBF58476D1CE4E5B9ull;
    h = (h ^ (h >> 27)) * 0x94D049BB133111EBull;
    h ^= h >> 31;
    x[i] = w * (2.0 * ((double)(h >> 11) * (1.0 / 9007199254740992.0)) - 1.0);
  }
}
}  // namespace

void krylov_step_probe(Ctx &ctx, int64_t n, int s, double ms[5], double bytes[5],
                       int *second_ran) {
  UDMRG_REQUIRE(n > 0 && s >= 1 && s + 2 <= kMaxVecs, "Krylov probe: 1 <= step <= 509, n > 0");
  KrylovWork kw(ctx, n, false, s + 1);
  // basis vectors 0 .. s + 1 with unit norm on average (random vectors of this
  // length are nearly orthogonal), Y likewise; every nrm2 entry 1
  std::vector<double *> basis(s + 2);
  const double w = std::sqrt(3.0 / (double)n);
  const int g = ew_grid(ctx, n);
  for (int j = 0; j < s + 2; ++j) {
    basis[j] = (double *)ctx.alloc(sizeof(double) * n);
    probe_fill_kernel<<<g, 256, 0, ctx.stream>>>(basis[j], n, 1000003ull * (j + 1), w);
    kw.push(j, basis[j]);
  }
  std::vector<double> ones(kMaxVecs + 2, 1.0);
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(kw.nrm2, ones.data(), ones.size() * sizeof(double),
                                   cudaMemcpyHostToDevice, ctx.stream));
  cudaEvent_t ev[6];
  for (auto &e : ev) UDMRG_CHECK_CUDA(cudaEventCreate(&e));
  double best[5];
  for (int rep = 0; rep < 4; ++rep) {
    probe_fill_kernel<<<g, 256, 0, ctx.stream>>>(kw.Y, n, 7ull + rep, w);
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(kw.step, &s, sizeof(int), cudaMemcpyHostToDevice, ctx.stream));
    cudaEventRecord(ev[0], ctx.stream);
    krylov_normalise(kw);
    cudaEventRecord(ev[1], ctx.stream);
    krylov_alpha(kw);
    cudaEventRecord(ev[2], ctx.stream);
    krylov_update(kw);
    cudaEventRecord(ev[3], ctx.stream);
    krylov_project(kw, false);
    cudaEventRecord(ev[4], ctx.stream);
    krylov_project(kw, true);
    cudaEventRecord(ev[5], ctx.stream);
    UDMRG_CHECK_CUDA(cudaEventSynchronize(ev[5]));
    for (int i = 0; i < 5; ++i) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
      best[i] = rep == 0 ? t : std::min(best[i], (double)t);
    }
  }
  double gate[2];
  UDMRG_CHECK_CUDA(cudaMemcpy(gate, kw.gate, sizeof(gate), cudaMemcpyDeviceToHost));
  for (auto &e : ev) cudaEventDestroy(e);
  for (double *b : basis) ctx.free(b);
  ctx.launches += (s + 2) + 4;  // the fills (the step's kernels count themselves)
  const double v = 8.0 * (double)n;  // bytes of one vector
  // normalise: Y read, X and v_s written; alpha: X, Y read; update: Y, X,
  // v_{s-1} read, Y written; a projection pass: the multi-dot reads v_0..v_s
  // and Y, the projection reads them again and writes Y
  const double b[5] = {3 * v, 2 * v, 4 * v, (2.0 * (s + 1) + 3) * v, (2.0 * (s + 1) + 3) * v};
  *second_ran = gate[1] < 0.5 * gate[0] ? 1 : 0;
  for (int i = 0; i < 5; ++i) {
    ms[i] = best[i];
    bytes[i] = (i == 4 && !*second_ran) ? 0.0 : b[i];
  }
}

void krylov_publish(KrylovWork &k) {
  Ctx &ctx = k.ctx;
  krylov_publish_kernel<<<1, 1, 0, ctx.stream>>>(k.alpha, k.nrm2, k.step, k.dres);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
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
