// Truncated block SVD kernels: strided 2-D copies (gather / scatter between
// block tensors and dense sector matrices) and row/column scaling.  The
// eigensolver is in kernels_eig.cu.
#include "svd.hpp"

namespace udmrg {

namespace {

// dst[dst_off + i*dst_ld + j*dst_cs] = src[src_off + i*src_ld + j*src_cs]
__global__ void copy2d_kernel(const Copy2D *__restrict__ ops, int nops,
                              const double *__restrict__ src, double *__restrict__ dst,
                              int cplx) {
  for (int o = blockIdx.x; o < nops; o += gridDim.x) {
    const Copy2D c = ops[o];
    const int64_t tot = (int64_t)c.rows * c.cols;
    for (int64_t e = threadIdx.x; e < tot; e += blockDim.x) {
      const int64_t i = e / c.cols, j = e - i * c.cols;
      const int64_t s = c.src_off + i * c.src_ld + j * c.src_cs;
      const int64_t d = c.dst_off + i * c.dst_ld + j * c.dst_cs;
      if (cplx) {
        ((double2 *)dst)[d] = ((const double2 *)src)[s];
      } else {
        dst[d] = src[s];
      }
    }
  }
}

// X[row r, col j] *= f[j] (column scaling) or f[r] (row scaling) for dense
// sector matrices listed in `jobs`.
__global__ void scale_cols_kernel(const ScaleJob *__restrict__ jobs, int njobs,
                                  double *__restrict__ X, const double *__restrict__ f,
                                  int cplx) {
  for (int o = blockIdx.x; o < njobs; o += gridDim.x) {
    const ScaleJob jb = jobs[o];
    const int64_t tot = (int64_t)jb.rows * jb.cols;
    for (int64_t e = threadIdx.x; e < tot; e += blockDim.x) {
      const int64_t i = e / jb.cols, j = e - i * jb.cols;
      const double s = f[jb.f_off + (jb.by_row ? i : j)];
      const int64_t x = jb.x_off + i * jb.cols + j;
      if (cplx) {
        double2 v = ((double2 *)X)[x];
        ((double2 *)X)[x] = make_double2(v.x * s, v.y * s);
      } else {
        X[x] *= s;
      }
    }
  }
}

}  // namespace

void run_copy2d(Ctx &ctx, const std::vector<Copy2D> &ops, const double *src, double *dst,
                bool cplx) {
  if (ops.empty()) return;
  Copy2D *d = (Copy2D *)ctx.alloc(ops.size() * sizeof(Copy2D));
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(d, ops.data(), ops.size() * sizeof(Copy2D),
                                   cudaMemcpyHostToDevice, ctx.stream));
  const int grid = (int)std::min<size_t>(ops.size(), 8 * (size_t)ctx.num_sms);
  copy2d_kernel<<<grid, 256, 0, ctx.stream>>>(d, (int)ops.size(), src, dst, cplx ? 1 : 0);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
  ctx.free(d);
  ctx.sync();  // host vector `ops` must outlive the upload
}

void run_scale(Ctx &ctx, const std::vector<ScaleJob> &jobs, double *X, const double *f,
               bool cplx) {
  if (jobs.empty()) return;
  ScaleJob *d = (ScaleJob *)ctx.alloc(jobs.size() * sizeof(ScaleJob));
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(d, jobs.data(), jobs.size() * sizeof(ScaleJob),
                                   cudaMemcpyHostToDevice, ctx.stream));
  const int grid = (int)std::min<size_t>(jobs.size(), 8 * (size_t)ctx.num_sms);
  scale_cols_kernel<<<grid, 256, 0, ctx.stream>>>(d, (int)jobs.size(), X, f, cplx ? 1 : 0);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
  ctx.sync();
  ctx.free(d);
}

}  // namespace udmrg
