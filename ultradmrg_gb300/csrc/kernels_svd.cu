// Truncated block SVD kernels: strided 2-D copies (gather / scatter between
// block tensors and dense sector matrices), a batched cyclic Jacobi
// eigensolver for the symmetric Gram matrix of every bond sector (one CTA per
// sector), and row/column scaling.
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

// One CTA per sector: eigen-decomposition of the symmetric (Hermitian for
// complex data is handled by the real 2n x 2n embedding on the host side) n x n
// matrix G by the cyclic Jacobi method with a round-robin ordering, so every
// round rotates n/2 disjoint (p, q) pairs in parallel.  Rotation angles follow
// Rutishauser's formulation (t = sgn(tau)/(|tau| + sqrt(1 + tau^2))).
// Outputs: eigenvalues in descending order and the matching eigenvectors as
// the columns of V (row-major n x n).
__global__ void jacobi_eig_kernel(const EigJob *__restrict__ jobs, double *__restrict__ G_all,
                                  double *__restrict__ V_all, double *__restrict__ lam_all,
                                  double *__restrict__ W_all, int max_sweeps, double tol,
                                  int *__restrict__ status) {
  extern __shared__ double sm[];
  const EigJob job = jobs[blockIdx.x];
  const int n = job.n;
  if (n == 0) return;
  double *G = job.smem ? sm : G_all + job.g_off;
  double *V = job.smem ? sm + (int64_t)n * n : W_all + job.g_off;
  const int tid = threadIdx.x, nt = blockDim.x;
  __shared__ double cs_c[512], cs_s[512];
  __shared__ int pp[512], qq[512];
  __shared__ double red[32];
  __shared__ int done;

  if (job.smem)
    for (int64_t e = tid; e < (int64_t)n * n; e += nt) G[e] = G_all[job.g_off + e];
  for (int64_t e = tid; e < (int64_t)n * n; e += nt) V[e] = (e / n == e % n) ? 1.0 : 0.0;
  // scale to unit max-abs, so the stopping test below cannot underflow for a
  // sector of tiny weight; non-finite input is reported, not iterated on
  __shared__ double gscale;
  __shared__ int nonfinite;
  {
    double mx = 0.0;
    int bad = 0;
    for (int64_t e = tid; e < (int64_t)n * n; e += nt) {
      const double g = G[e];
      bad |= !isfinite(g);
      mx = fmax(mx, fabs(g));
    }
    for (int o = 16; o > 0; o >>= 1) {
      mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
      bad |= __shfl_down_sync(0xffffffffu, bad, o);
    }
    if (tid == 0) nonfinite = 0;
    __syncthreads();
    if ((tid & 31) == 0) {
      red[tid >> 5] = mx;
      if (bad) atomicOr(&nonfinite, 1);
    }
    __syncthreads();
    if (tid == 0) {
      double m = 0.0;
      for (int w = 0; w < (nt + 31) / 32; ++w) m = fmax(m, red[w]);
      gscale = m;
    }
    __syncthreads();
  }
  if (nonfinite) {
    if (tid == 0) atomicExch(status, 2);
    return;
  }
  const double gs = gscale;
  if (gs > 0.0 && gs != 1.0) {
    const double inv = 1.0 / gs;
    for (int64_t e = tid; e < (int64_t)n * n; e += nt) G[e] *= inv;
  }
  __syncthreads();

  const int npad = n + (n & 1);
  const int npairs = npad / 2;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    // re-symmetrise: the input Gram matrix and the parallel rotations are
    // symmetric only up to rounding, and rotations preserve the norm of an
    // antisymmetric part, which would otherwise floor the off-diagonal norm
    for (int64_t e = tid; e < (int64_t)n * n; e += nt) {
      const int i = (int)(e / n), j = (int)(e % n);
      if (i < j) {
        const double v = 0.5 * (G[(int64_t)i * n + j] + G[(int64_t)j * n + i]);
        G[(int64_t)i * n + j] = v;
        G[(int64_t)j * n + i] = v;
      }
    }
    __syncthreads();
    // convergence: off-diagonal norm vs diagonal norm
    double off = 0.0, dia = 0.0;
    for (int64_t e = tid; e < (int64_t)n * n; e += nt) {
      const int i = (int)(e / n), j = (int)(e % n);
      const double g = G[e];
      if (i == j)
        dia += g * g;
      else
        off += g * g;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_down_sync(0xffffffffu, off, o);
      dia += __shfl_down_sync(0xffffffffu, dia, o);
    }
    if ((tid & 31) == 0) red[tid >> 5] = off;
    __syncthreads();
    if (tid == 0) {
      double s = 0;
      for (int w = 0; w < (nt + 31) / 32; ++w) s += red[w];
      red[31] = s;
    }
    __syncthreads();
    const double off_tot = red[31];
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = dia;
    __syncthreads();
    if (tid == 0) {
      double s = 0;
      for (int w = 0; w < (nt + 31) / 32; ++w) s += red[w];
      // rounding keeps the off-diagonal norm near n * eps * |G|: scale the target with n
      const double t = tol * (double)n;
      done = (off_tot <= t * t * s) ? 1 : 0;
    }
    __syncthreads();
    if (done) break;
    for (int r = 0; r < npad - 1; ++r) {
      // round-robin pairing: position 0 fixed, the others rotate
      for (int i = tid; i < npairs; i += nt) {
        const int pa = i, pb = npad - 1 - i;
        const int a = pa == 0 ? 0 : 1 + (pa - 1 + r) % (npad - 1);
        const int b = pb == 0 ? 0 : 1 + (pb - 1 + r) % (npad - 1);
        int p = min(a, b), q = max(a, b);
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double gpq = G[(int64_t)p * n + q];
          const double gpp = G[(int64_t)p * n + p], gqq = G[(int64_t)q * n + q];
          if (fabs(gpq) > 1e-300 && fabs(gpq) > 1e-18 * sqrt(fabs(gpp * gqq))) {
            const double tau = (gqq - gpp) / (2.0 * gpq);
            const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        } else {
          q = -1;
        }
        cs_c[i] = c;
        cs_s[i] = s;
        pp[i] = p;
        qq[i] = q;
      }
      __syncthreads();
      // rows p, q
      for (int64_t e = tid; e < (int64_t)npairs * n; e += nt) {
        const int i = (int)(e / n), j = (int)(e % n);
        const int q = qq[i];
        if (q < 0 || cs_s[i] == 0.0) continue;
        const int p = pp[i];
        const double c = cs_c[i], s = cs_s[i];
        const double gp = G[(int64_t)p * n + j], gq = G[(int64_t)q * n + j];
        G[(int64_t)p * n + j] = c * gp - s * gq;
        G[(int64_t)q * n + j] = s * gp + c * gq;
      }
      __syncthreads();
      // columns p, q of G and V
      for (int64_t e = tid; e < (int64_t)npairs * n; e += nt) {
        const int i = (int)(e / n), k = (int)(e % n);
        const int q = qq[i];
        if (q < 0 || cs_s[i] == 0.0) continue;
        const int p = pp[i];
        const double c = cs_c[i], s = cs_s[i];
        const double gp = G[(int64_t)k * n + p], gq = G[(int64_t)k * n + q];
        G[(int64_t)k * n + p] = c * gp - s * gq;
        G[(int64_t)k * n + q] = s * gp + c * gq;
        const double vp = V[(int64_t)k * n + p], vq = V[(int64_t)k * n + q];
        V[(int64_t)k * n + p] = c * vp - s * vq;
        V[(int64_t)k * n + q] = s * vp + c * vq;
      }
      __syncthreads();
    }
  }
  if (tid == 0 && sweep >= max_sweeps) atomicCAS(status, 0, 1);
  // sort eigenvalues descending (rank by counting; ties by index), permute V
  for (int i = tid; i < n; i += nt) {
    const double li = G[(int64_t)i * n + i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double lj = G[(int64_t)j * n + j];
      if (lj > li || (lj == li && j < i)) ++rank;
    }
    lam_all[job.lam_off + rank] = li * gs;
    // column i of V -> column rank of the output
    for (int k = 0; k < n; ++k) V_all[job.g_off + (int64_t)k * n + rank] = V[(int64_t)k * n + i];
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

int run_jacobi_eig(Ctx &ctx, const std::vector<EigJob> &jobs_in, double *G, double *V,
                   double *W, double *lam) {
  if (jobs_in.empty()) return 0;
  std::vector<EigJob> jobs = jobs_in;
  int max_n = 0;
  for (auto &j : jobs) max_n = std::max(max_n, j.n);
  UDMRG_REQUIRE(max_n <= 1024, "svd: bond sector larger than 1024 rows is not supported yet");
  size_t smem = 0;
  for (auto &j : jobs) {
    size_t need = 2 * (size_t)j.n * j.n * sizeof(double);
    j.smem = need <= kJacobiSmemBytes ? 1 : 0;
    if (j.smem) smem = std::max(smem, need);
  }
  UDMRG_CHECK_CUDA(cudaFuncSetAttribute(jacobi_eig_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)kJacobiSmemBytes));
  EigJob *d = (EigJob *)ctx.alloc(jobs.size() * sizeof(EigJob));
  int *dstat = (int *)ctx.alloc(sizeof(int));
  UDMRG_CHECK_CUDA(cudaMemsetAsync(dstat, 0, sizeof(int), ctx.stream));
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(d, jobs.data(), jobs.size() * sizeof(EigJob),
                                   cudaMemcpyHostToDevice, ctx.stream));
  jacobi_eig_kernel<<<(int)jobs.size(), 512, smem, ctx.stream>>>(d, G, V, lam, W, 40, 4e-16,
                                                                  dstat);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
  int hstat = 0;
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(&hstat, dstat, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  ctx.free(d);
  ctx.free(dstat);
  return hstat;
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
