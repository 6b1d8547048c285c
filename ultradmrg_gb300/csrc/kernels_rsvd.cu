// Kernels of the sector-wise randomized SVD: Gaussian sketch matrices from a
// counter-based generator, and the inverse Cholesky factor of small
// symmetric positive semi-definite Gram matrices (one CTA per sector) used by
// Cholesky-QR orthonormalisation.
#include "svd.hpp"

namespace udmrg {

namespace {

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Standard normal deviates by the Box-Muller transform of two uniforms.
__global__ void fill_normal_kernel(double *__restrict__ x, int64_t n, uint64_t seed) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t a = splitmix64(seed ^ (uint64_t)(2 * i)), b = splitmix64(seed + (uint64_t)(2 * i + 1));
    const double u1 = ((double)(a >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);
    x[i] = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
  }
}

// S (n x n, symmetric PSD, row-major) -> R^{-T} (R^{-1} transposed, into
// work) where S = R^T R,
// R upper triangular (kept in S's upper triangle).  Pivots below
// rel_tol * max diag drop their direction (row/column of R^{-1} set to zero),
// which handles rank-deficient sketches.  One CTA per job; the matrix stays in
// global memory (L1/L2 resident).  The trailing update runs one warp per row
// over the upper triangle; R^{-1} is built row by row from the bottom, all
// columns of a row in parallel.
__global__ void chol_inv_kernel(const EigJob *__restrict__ jobs, double *__restrict__ S_all,
                                double *__restrict__ work_all, double rel_tol) {
  const EigJob job = jobs[blockIdx.x];
  const int n = job.n;
  if (n == 0) return;
  double *S = S_all + job.g_off;
  double *Ri = work_all + job.g_off;  // R^{-1}
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  __shared__ double dmax;
  __shared__ double piv;
  if (tid == 0) {
    double m = 0;
    for (int i = 0; i < n; ++i) m = fmax(m, S[(int64_t)i * n + i]);
    dmax = m;
  }
  __syncthreads();
  // Cholesky, upper factor R stored in the upper triangle of S (row k of R)
  for (int k = 0; k < n; ++k) {
    if (tid == 0) {
      const double d = S[(int64_t)k * n + k];
      piv = (d > rel_tol * dmax && d > 0) ? sqrt(d) : 0.0;
      S[(int64_t)k * n + k] = piv;
    }
    __syncthreads();
    const double p = piv;
    const double ip = p > 0 ? 1.0 / p : 0.0;
    for (int j = k + 1 + tid; j < n; j += nt) S[(int64_t)k * n + j] *= ip;
    __syncthreads();
    // trailing update S[i][j] -= R[k][i] R[k][j] for k < i <= j
    if (p > 0)
      for (int i = k + 1 + warp; i < n; i += nwarp) {
        const double rki = S[(int64_t)k * n + i];
        double *si = S + (int64_t)i * n;
        const double *rk = S + (int64_t)k * n;
        for (int j = i + lane; j < n; j += 32) si[j] -= rki * rk[j];
      }
    __syncthreads();
  }
  // R^{-1}, stored transposed (RiT[j][k] = R^{-1}[k][j]): row i from the rows
  // below, R^{-1}[i][j] = -(sum_{i<k<=j} R[i][k] R^{-1}[k][j]) / R[i][i];
  // one warp per column j, lanes over k (contiguous in both R and RiT)
  double *RiT = Ri;
  for (int64_t e = tid; e < (int64_t)n * n; e += nt) RiT[e] = 0.0;
  __syncthreads();
  for (int i = n - 1; i >= 0; --i) {
    const double dii = S[(int64_t)i * n + i];
    if (dii != 0.0) {
      const double inv = 1.0 / dii;
      const double *ri = S + (int64_t)i * n;
      if (tid == 0) RiT[(int64_t)i * n + i] = inv;
      for (int j = i + 1 + warp; j < n; j += nwarp) {
        const double *xj = RiT + (int64_t)j * n;
        double acc = 0.0;
        for (int k = i + 1 + lane; k <= j; k += 32) acc += ri[k] * xj[k];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) RiT[(int64_t)j * n + i] = -acc * inv;
      }
    }
    __syncthreads();
  }
}

// Sum of squares of every column of row-major rows x cols matrices (one CTA
// per matrix, consecutive threads on consecutive columns).
__global__ void col_sumsq_kernel(const ScaleJob *__restrict__ jobs, const double *__restrict__ X,
                                 double *__restrict__ out) {
  const ScaleJob jb = jobs[blockIdx.x];
  for (int j = threadIdx.x; j < jb.cols; j += blockDim.x) {
    double acc = 0.0;
    const double *x = X + jb.x_off + j;
    for (int i = 0; i < jb.rows; ++i) {
      const double v = x[(int64_t)i * jb.cols];
      acc = fma(v, v, acc);
    }
    out[jb.f_off + j] = acc;
  }
}

}  // namespace

void run_col_sumsq(Ctx &ctx, const std::vector<ScaleJob> &jobs, const double *X, double *out) {
  if (jobs.empty()) return;
  ScaleJob *d = (ScaleJob *)ctx.alloc(jobs.size() * sizeof(ScaleJob));
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(d, jobs.data(), jobs.size() * sizeof(ScaleJob),
                                   cudaMemcpyHostToDevice, ctx.stream));
  col_sumsq_kernel<<<(int)jobs.size(), 128, 0, ctx.stream>>>(d, X, out);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
  ctx.sync();
  ctx.free(d);
}

void fill_normal(Ctx &ctx, double *x, int64_t n, uint64_t seed) {
  if (n == 0) return;
  const int grid = (int)std::min<int64_t>((n + 255) / 256, 8 * ctx.num_sms);
  fill_normal_kernel<<<grid, 256, 0, ctx.stream>>>(x, n, seed);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

void run_chol_inv(Ctx &ctx, const std::vector<EigJob> &jobs, double *S, double *Rinv,
                  double rel_tol) {
  if (jobs.empty()) return;
  EigJob *d = (EigJob *)ctx.alloc(jobs.size() * sizeof(EigJob));
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(d, jobs.data(), jobs.size() * sizeof(EigJob),
                                   cudaMemcpyHostToDevice, ctx.stream));
  chol_inv_kernel<<<(int)jobs.size(), 256, 0, ctx.stream>>>(d, S, Rinv, rel_tol);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
  ctx.sync();
  ctx.free(d);
}

}  // namespace udmrg
