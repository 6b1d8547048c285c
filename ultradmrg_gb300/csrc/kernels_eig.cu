// Batched symmetric eigen-solver of the truncated SVD (Gram matrices of the
// bond sectors and the Rayleigh-Ritz matrices of the randomized SVD).
//
// FP64 throughput per SM is low on this GPU, so the solver does as little
// FP64 work as the problem allows:
//   1. Householder reduction to tridiagonal form (about 2 n^3 flops; one CTA
//      per matrix held in shared memory, several co-resident CTAs per larger
//      matrix; the reflectors stay in the matrix's upper triangle);
//   2. every eigenvalue by Sturm-sequence bisection (O(n) per step and
//      eigenvalue, all eigenvalues of all matrices in parallel);
//   3. only the eigenvectors the caller needs, by inverse iteration on the
//      tridiagonal matrix (one thread per cluster of close eigenvalues;
//      modified Gram-Schmidt inside a cluster);
//   4. orthonormalisation by Newton-Schulz steps (grouped GEMMs, host side);
//   5. back-transformation by the Householder reflectors (one CTA per matrix).
// These are the textbook methods (Golub & Van Loan ch. 8; Wilkinson's
// inverse iteration; the Sturm count of Barth, Martin & Wilkinson), written
// for this batch layout.
#include <algorithm>
#include <cmath>

#include "svd.hpp"
#include "vecops.hpp"

namespace udmrg {

namespace {

constexpr int kTriThreads = 512;
constexpr int kBackThreads = 256;

__device__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < nw; ++i) s += red[i];
    red[32] = s;
  }
  __syncthreads();
  return red[32];
}

// Householder tridiagonalisation of the symmetric n x n matrix of each job
// that fits in shared memory (row-major at G + g_off; the matrix is first
// scaled to unit max-abs, the scale goes to scale[job]).  Step j reflects
// row/column j: v (v_0 = 1) is stored in row j right of the first
// superdiagonal, tau in tau[lam_off + j], the diagonal in d[lam_off + i] and
// the off-diagonal in e[lam_off + i].
__global__ void tridiag_kernel(const EigJob *__restrict__ jobs, double *__restrict__ G_all,
                               double *__restrict__ d_all, double *__restrict__ e_all,
                               double *__restrict__ tau_all, double *__restrict__ scale_all,
                               int *__restrict__ status) {
  extern __shared__ double sm[];
  __shared__ double red[33];
  __shared__ int bad;
  const EigJob job = jobs[blockIdx.x];
  const int n = job.n;
  if (n == 0 || !job.smem) return;  // larger matrices: tridiag_mc_kernel
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  double *A = sm;
  double *v = sm + (int64_t)n * n;
  double *w = v + n;
  double *d = d_all + job.lam_off, *e = e_all + job.lam_off, *tau = tau_all + job.lam_off;

  for (int64_t x = tid; x < (int64_t)n * n; x += nt) A[x] = G_all[job.g_off + x];
  // scale to unit max-abs; non-finite input is reported
  double mx = 0.0;
  int nf = 0;
  if (tid == 0) bad = 0;
  for (int64_t x = tid; x < (int64_t)n * n; x += nt) {
    const double g = A[x];
    nf |= !isfinite(g);
    mx = fmax(mx, fabs(g));
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    nf |= __shfl_down_sync(0xffffffffu, nf, o);
  }
  __syncthreads();
  if (lane == 0) {
    red[warp] = mx;
    if (nf) atomicOr(&bad, 1);
  }
  __syncthreads();
  if (tid == 0) {
    double m = 0.0;
    for (int i = 0; i < nwarp; ++i) m = fmax(m, red[i]);
    red[32] = m;
  }
  __syncthreads();
  if (bad) {
    if (tid == 0) atomicExch(status, 2);
    return;
  }
  const double scale = red[32];
  if (tid == 0) scale_all[blockIdx.x] = scale;
  // scale and symmetrise (a GEMM-made Gram matrix is symmetric only up to rounding)
  const double inv = scale > 0.0 ? 1.0 / scale : 0.0;
  for (int64_t x = tid; x < (int64_t)n * n; x += nt) {
    const int r = (int)(x / n), c = (int)(x - (int64_t)r * n);
    if (r < c) {
      const double g = 0.5 * inv * (A[x] + A[(int64_t)c * n + r]);
      A[x] = g;
      A[(int64_t)c * n + r] = g;
    } else if (r == c) {
      A[x] *= inv;
    }
  }
  __syncthreads();

  for (int j = 0; j + 2 < n; ++j) {
    const int m = n - j - 1;  // length of the reflected vector (rows j+1 .. n-1)
    double *rowj = A + (int64_t)j * n;
    const double alpha = rowj[j + 1];
    double x2 = 0.0;
    for (int c = j + 2 + tid; c < n; c += nt) x2 += rowj[c] * rowj[c];
    x2 = block_sum(x2, red);
    double t = 0.0, beta = alpha, vs = 0.0;
    if (x2 > 0.0) {
      beta = -copysign(sqrt(alpha * alpha + x2), alpha);
      t = (beta - alpha) / beta;
      vs = 1.0 / (alpha - beta);
    }
    for (int r = tid; r < m; r += nt) {
      const double vr = r == 0 ? 1.0 : rowj[j + 1 + r] * vs;
      v[r] = t == 0.0 ? (r == 0 ? 1.0 : 0.0) : vr;
      if (r > 0) rowj[j + 1 + r] = v[r];
    }
    if (tid == 0) {
      d[j] = rowj[j];
      e[j] = beta;
      tau[j] = t;
    }
    __syncthreads();
    if (t == 0.0) continue;
    // w = t * A_t v, A_t = trailing block rows/cols j+1 .. n-1 (one warp per row)
    for (int r = warp; r < m; r += nwarp) {
      const double *ar = A + (int64_t)(j + 1 + r) * n + (j + 1);
      double s = 0.0;
      for (int c = lane; c < m; c += 32) s += ar[c] * v[c];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) w[r] = t * s;
    }
    __syncthreads();
    double wv = 0.0;
    for (int r = tid; r < m; r += nt) wv += w[r] * v[r];
    wv = block_sum(wv, red);
    const double K = -0.5 * t * wv;
    for (int r = tid; r < m; r += nt) w[r] += K * v[r];
    __syncthreads();
    // A_t -= v w^T + w v^T
    for (int64_t x = tid; x < (int64_t)m * m; x += nt) {
      const int r = (int)(x / m), c = (int)(x - (int64_t)r * m);
      A[(int64_t)(j + 1 + r) * n + (j + 1 + c)] -= v[r] * w[c] + w[r] * v[c];
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (n >= 2) {
      d[n - 2] = A[(int64_t)(n - 2) * n + (n - 2)];
      e[n - 2] = A[(int64_t)(n - 2) * n + (n - 1)];
      tau[n - 2] = 0.0;
    }
    d[n - 1] = A[(int64_t)(n - 1) * n + (n - 1)];
    e[n - 1] = 0.0;
    tau[n - 1] = 0.0;
  }
  __syncthreads();
  // the reflectors live in the rows' upper parts
  for (int64_t x = tid; x < (int64_t)n * n; x += nt) G_all[job.g_off + x] = A[x];
}

// Number of eigenvalues of the tridiagonal (d, e) below x (Sturm count).
__device__ __forceinline__ int sturm_count(const double *d, const double *e, int n, double x,
                                           double pivmin) {
  int cnt = 0;
  double q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  if (q < 0.0) ++cnt;
  for (int k = 1; k < n; ++k) {
    q = d[k] - x - e[k - 1] * e[k - 1] / q;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0.0) ++cnt;
  }
  return cnt;
}

// Eigenvalues by multisection; lam[lam_off + i] (descending) = scale * value.
// A warp handles kBisectEigs eigenvalues of one job, kBisectLanes lanes each:
// per step the lanes of an eigenvalue take Sturm counts at the kBisectLanes
// interior points that cut its interval into kBisectLanes + 1 equal parts,
// and the part holding the eigenvalue is kept (the division chain of a Sturm
// count is serial, so points side by side shorten the chain of steps).
// Block b handles eigenvalues i0 .. i0 + kBisectEigs - 1 (ascending index) of
// job chunk[b].x, i0 = chunk[b].y.
// With the threshold grid of the leading-eigenvalue path (top, cnt; see
// grid_count_kernel) each eigenvalue starts from its grid cell, a factor 1.34
// wide, instead of the Gershgorin interval: up to ~40% fewer steps for the
// small eigenvalues of a Gram matrix.
constexpr int kBisectLanes = 8;
constexpr int kBisectEigs = 32 / kBisectLanes;
constexpr int kGrid = 256;             // grid points
constexpr double kGridDecades = 32.0;  // the grid spans top .. top * 1e-32
__device__ __forceinline__ double grid_point(double top, int k) {
  return top * exp10(-(double)k * kGridDecades / (kGrid - 1));
}
__global__ void __launch_bounds__(32)
    bisect_kernel(const EigJob *__restrict__ jobs, const int2 *__restrict__ chunk,
                  const double *__restrict__ d_all, const double *__restrict__ e_all,
                  const double *__restrict__ scale_all, double *__restrict__ lam_all,
                  const double *__restrict__ grid_top, const int *__restrict__ grid_cnt) {
  extern __shared__ double sm[];
  const int jb = chunk[blockIdx.x].x, i0 = chunk[blockIdx.x].y;
  const EigJob job = jobs[jb];
  const int n = job.n;
  if (n == 0) return;
  const int lane = threadIdx.x, grp = lane / kBisectLanes, k = lane % kBisectLanes;
  double *d = sm, *e = sm + n;
  for (int i = lane; i < n; i += 32) {
    d[i] = d_all[job.lam_off + i];
    e[i] = i + 1 < n ? e_all[job.lam_off + i] : 0.0;
  }
  __syncwarp();
  // Gershgorin interval and the largest off-diagonal (warp reduction)
  double glo = 1e308, ghi = -1e308, em = 0.0;
  for (int i = lane; i < n; i += 32) {
    const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0);
    glo = fmin(glo, d[i] - r);
    ghi = fmax(ghi, d[i] + r);
    if (i + 1 < n) em = fmax(em, fabs(e[i]));
  }
  for (int o = 16; o > 0; o >>= 1) {
    glo = fmin(glo, __shfl_xor_sync(0xffffffffu, glo, o));
    ghi = fmax(ghi, __shfl_xor_sync(0xffffffffu, ghi, o));
    em = fmax(em, __shfl_xor_sync(0xffffffffu, em, o));
  }
  const double pad = 2.2e-16 * fmax(fabs(glo), fabs(ghi)) * n + 1e-300;
  const double lo0 = glo - pad, hi0 = ghi + pad;
  const double pivmin = 1e-290 * fmax(1.0, em * em);
  const double scale = scale_all[jb];
  // absolute accuracy far below the eps * |T| the reduction itself achieves
  const double atol = 1e-18 * fmax(fabs(lo0), fabs(hi0));
  const int i = i0 + grp;  // i-th smallest
  double lo = lo0, hi = hi0;
  bool done = i >= n;
  if (grid_cnt && !done && scale > 0.0 && grid_top[0] > 0.0) {
    // cnt[k] = eigenvalues not below x_k (decreasing x_k); the first k with
    // cnt[k] >= n - i bounds eigenvalue i from below by x_k, and x_{k-1}
    // from above (the counts come from the same Sturm sequence)
    const int *cnt = grid_cnt + (int64_t)jb * (kGrid + 1);
    int k = 0;
    while (k < kGrid && cnt[k] < n - i) ++k;
    if (k < kGrid) lo = fmax(lo, grid_point(grid_top[0], k) / scale);
    if (k > 0) hi = fmin(hi, grid_point(grid_top[0], k - 1) / scale);
    if (!(lo < hi)) {  // inconsistent rounding at a cell edge: the full interval
      lo = lo0;
      hi = hi0;
    }
  }
  for (int it = 0; it < 64; ++it) {
    if (!done && hi - lo <= 4.4e-16 * fmax(fabs(lo), fabs(hi)) + atol) done = true;
    if (__all_sync(0xffffffffu, done)) break;
    const double w = (hi - lo) / (kBisectLanes + 1);
    const double x = lo + w * (k + 1);
    const bool above = !done && x > lo && x < hi && sturm_count(d, e, n, x, pivmin) > i;
    const unsigned m = (__ballot_sync(0xffffffffu, above) >> (grp * kBisectLanes)) &
                       ((1u << kBisectLanes) - 1);
    if (!done) {
      // first point with more than i eigenvalues below it bounds eigenvalue i
      const int f = m ? __ffs(m) - 1 : kBisectLanes;
      const double nlo = f == 0 ? lo : lo + w * f, nhi = f == kBisectLanes ? hi : lo + w * (f + 1);
      if (nlo <= lo && nhi >= hi) {
        done = true;  // no representable point inside the interval
      } else {
        lo = nlo;
        hi = nhi;
      }
    }
  }
  if (i < n && k == 0) lam_all[job.lam_off + (n - 1 - i)] = scale * 0.5 * (lo + hi);
}

// ---- leading eigenvalues only (positive semi-definite jobs) ----
//
// A truncated SVD keeps at most Dmax states of all bond sectors together, and
// the weight of the discarded ones follows from each Gram matrix's trace, so
// only the leading eigenvalues of every sector need bisection.  A common
// threshold is read off Sturm counts at a logarithmic grid of points below
// the largest Gershgorin bound of all jobs.
// top[0] = max over jobs of scale * (Gershgorin upper bound of its tridiagonal)
__global__ void grid_top_kernel(const EigJob *__restrict__ jobs, int nj,
                                const double *__restrict__ d_all, const double *__restrict__ e_all,
                                const double *__restrict__ scale_all, double *__restrict__ top) {
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  double m = 0.0;
  for (int q = warp; q < nj; q += nwarp) {
    const EigJob job = jobs[q];
    const int n = job.n;
    const double *d = d_all + job.lam_off, *e = e_all + job.lam_off;
    double h = 0.0;
    for (int i = lane; i < n; i += 32)
      h = fmax(h, d[i] + (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0));
    for (int o = 16; o > 0; o >>= 1) h = fmax(h, __shfl_down_sync(0xffffffffu, h, o));
    if (lane == 0) m = fmax(m, scale_all[q] * h);
  }
  if (lane == 0) red[warp] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < nwarp; ++w) t = fmax(t, red[w]);
    top[0] = t;
  }
}

// cnt[q * (kGrid + 1) + k] = number of eigenvalues of job q not below
// x_k = top * 10^(-k * kGridDecades / (kGrid - 1)) for k < kGrid, and n for
// k = kGrid; tr[q] = scale * sum of the diagonal (the trace).  One block per
// job, one grid point per thread.
__global__ void grid_count_kernel(const EigJob *__restrict__ jobs,
                                  const double *__restrict__ d_all,
                                  const double *__restrict__ e_all,
                                  const double *__restrict__ scale_all,
                                  const double *__restrict__ top, int *__restrict__ cnt,
                                  double *__restrict__ tr) {
  extern __shared__ double sm[];
  __shared__ double pm[2];
  const int q = blockIdx.x;
  const EigJob job = jobs[q];
  const int n = job.n;
  double *d = sm, *e = sm + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    d[i] = d_all[job.lam_off + i];
    e[i] = i + 1 < n ? e_all[job.lam_off + i] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = 0.0, em = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) {
      t += d[i];
      em = fmax(em, fabs(e[i]));
    }
    for (int o = 16; o > 0; o >>= 1) {
      t += __shfl_down_sync(0xffffffffu, t, o);
      em = fmax(em, __shfl_down_sync(0xffffffffu, em, o));
    }
    if (threadIdx.x == 0) {
      pm[0] = t;
      pm[1] = em;
    }
  }
  __syncthreads();
  const double sc = scale_all[q];
  if (threadIdx.x == 0) tr[q] = sc * pm[0];
  const double pivmin = 1e-290 * fmax(1.0, pm[1] * pm[1]);  // as in bisect_kernel
  for (int k = threadIdx.x; k <= kGrid; k += blockDim.x) {
    int c;
    if (k == kGrid || n == 0) {
      c = n;
    } else if (sc <= 0.0 || top[0] <= 0.0) {
      c = 0;  // a zero matrix: no eigenvalue reaches x_k > 0
    } else {
      c = n - sturm_count(d, e, n, grid_point(top[0], k) / sc, pivmin);
    }
    cnt[(int64_t)q * (kGrid + 1) + k] = c;
  }
}

__device__ __forceinline__ double start_entry(uint64_t seed, int i) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// Inverse iteration: one thread per cluster of eigenvalues (descending
// positions first .. first+count-1 of job `job`), each eigenvector found with
// an LU factorisation (partial pivoting) of T - lambda I and three solves,
// orthogonalised against the cluster's earlier vectors (modified
// Gram-Schmidt).  Vector of position p goes to column p of Z (row-major
// n x ld at z_off).  Work arrays are interleaved by thread (coalesced).
__global__ void invit_kernel(const EigCluster *__restrict__ cl, int ncl,
                             const EigJob *__restrict__ jobs, const double *__restrict__ d_all,
                             const double *__restrict__ e_all,
                             const double *__restrict__ scale_all,
                             const double *__restrict__ lam_all, double *__restrict__ Z,
                             double *__restrict__ work, int nmax) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncl) return;
  const EigCluster c = cl[t];
  const EigJob job = jobs[c.job];
  const int n = job.n;
  const double *d = d_all + job.lam_off, *e = e_all + job.lam_off;
  const int64_t T = ncl;
  double *l = work + 0 * (int64_t)nmax * T, *u0 = work + 1 * (int64_t)nmax * T;
  double *u1 = work + 2 * (int64_t)nmax * T, *u2 = work + 3 * (int64_t)nmax * T;
  double *y = work + 4 * (int64_t)nmax * T, *pv = work + 5 * (int64_t)nmax * T;
  auto at = [&](double *a, int i) -> double & { return a[(int64_t)i * T + t]; };
  double tnorm = 0.0;
  for (int i = 0; i < n; ++i)
    tnorm = fmax(tnorm, fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0) +
                            (i + 1 < n ? fabs(e[i]) : 0.0));
  const double tiny = 2.2e-16 * (tnorm > 0.0 ? tnorm : 1.0);  // zero matrix: any basis
  const double inv_scale = scale_all[c.job] > 0.0 ? 1.0 / scale_all[c.job] : 0.0;
  double *zc = Z + c.z_off;
  for (int k = 0; k < c.count; ++k) {
    const int p = c.first + k;
    const double lam = lam_all[job.lam_off + p] * inv_scale;
    if (n == 1) {
      zc[p] = 1.0;
      continue;
    }
    // LU of T - lam I with row interchanges: row i of U holds u0 (the
    // reciprocal of the diagonal, kept away from zero), u1, u2 (the two
    // superdiagonals); l the multipliers; pv the interchanges
    auto rinv = [&](double v) {
      return 1.0 / (fabs(v) > tiny ? v : (v < 0 ? -tiny : tiny));
    };
    double a = d[0] - lam, b = e[0];
    for (int i = 0; i + 1 < n; ++i) {
      const double sub = e[i], dn = d[i + 1] - lam, sup = i + 2 < n ? e[i + 1] : 0.0;
      if (fabs(a) >= fabs(sub)) {
        const double piv = a != 0.0 ? a : tiny;
        const double f = sub / piv;
        at(u0, i) = rinv(piv);
        at(u1, i) = b;
        at(u2, i) = 0.0;
        at(l, i) = f;
        at(pv, i) = 0.0;
        a = dn - f * b;
        b = sup;
      } else {
        const double f = a / sub;
        at(u0, i) = rinv(sub);
        at(u1, i) = dn;
        at(u2, i) = sup;
        at(l, i) = f;
        at(pv, i) = 1.0;
        a = b - f * dn;
        b = -f * sup;
      }
    }
    at(u0, n - 1) = rinv(a);
    for (int i = 0; i < n; ++i) at(y, i) = start_entry(c.seed + 7919ull * (uint64_t)p, i);
    for (int it = 0; it < 3; ++it) {
      // forward: apply the interchanges and multipliers
      for (int i = 0; i + 1 < n; ++i) {
        if (at(pv, i) != 0.0) {
          const double tmp = at(y, i);
          at(y, i) = at(y, i + 1);
          at(y, i + 1) = tmp - at(l, i) * at(y, i);
        } else {
          at(y, i + 1) -= at(l, i) * at(y, i);
        }
      }
      // back substitution with U
      for (int i = n - 1; i >= 0; --i) {
        double s = at(y, i);
        if (i + 1 < n) s -= at(u1, i) * at(y, i + 1);
        if (i + 2 < n) s -= at(u2, i) * at(y, i + 2);
        at(y, i) = s * at(u0, i);
      }
      // orthogonalise against the cluster's earlier vectors, normalise
      for (int q = c.first; q < p; ++q) {
        double s = 0.0;
        for (int i = 0; i < n; ++i) s += zc[(int64_t)i * c.ld + q] * at(y, i);
        for (int i = 0; i < n; ++i) at(y, i) -= s * zc[(int64_t)i * c.ld + q];
      }
      double nrm = 0.0;
      for (int i = 0; i < n; ++i) nrm += at(y, i) * at(y, i);
      nrm = sqrt(nrm);
      const double f = nrm > 0.0 ? 1.0 / nrm : 0.0;
      for (int i = 0; i < n; ++i) at(y, i) *= f;
    }
    for (int i = 0; i < n; ++i) zc[(int64_t)i * c.ld + p] = at(y, i);
  }
}

// Back transformation: Z (row-major n x k, leading dimension ld, at z_off)
// <- Q Z with Q = H_0 H_1 ... H_{n-3}, H_j = I - tau_j v_j v_j^T acting on
// rows j+1 ...  Block b transforms columns c0 .. c0 + cw - 1 of job
// bt[b].job (columns are independent).
struct BackChunk {
  int64_t z_off, ld;
  int32_t job, c0, cw, pad;
};
// Real data: narrow column chunks (W = 8
// columns per block, 4 for matrices above 3,400 rows), so that the largest
// sector's columns spread over many SMs: this GPU issues about two FP64 FMAs
// per clock per SM, and one sector's 4 n^2 k flops on one SM would bound the
// whole kernel.  The chunk lives in shared memory (n x W doubles) for all
// reflectors; thread t owns column t % W and the rows congruent to t / W
// modulo kBackThreads / W.  Per reflector: partial dot products, a reduction
// over the row groups (shuffles inside a warp, one shared-memory stage across
// warps), the rank-1 update; two block barriers.
template <int W>
__global__ void __launch_bounds__(kBackThreads)
    backtransform_narrow_kernel(const EigJob *__restrict__ jobs,
                                const BackChunk *__restrict__ bt,
                                const double *__restrict__ G_all,
                                const double *__restrict__ tau_all, double *__restrict__ Z) {
  constexpr int RG = kBackThreads / W;  // row groups
  static_assert(RG * W == kBackThreads && W <= 32 && (32 % W) == 0, "back transformation layout");
  extern __shared__ double zs[];  // n x W
  __shared__ double part[kBackThreads / 32][W];
  const BackChunk ch = bt[blockIdx.x];
  const EigJob job = jobs[ch.job];
  const int n = job.n;
  if (n < 3 || ch.cw == 0) return;
  const int c = threadIdx.x % W, g = threadIdx.x / W;
  const int warp = threadIdx.x >> 5;
  double *z = Z + ch.z_off + ch.c0;
  const bool col = c < ch.cw;
  for (int r = g; r < n; r += RG) zs[r * W + c] = col ? z[(int64_t)r * ch.ld + c] : 0.0;
  __syncthreads();
  const double *A = G_all + job.g_off;
  for (int j = n - 3; j >= 0; --j) {
    const double t = tau_all[job.lam_off + j];
    if (t == 0.0) continue;  // uniform across the block
    const int m = n - j - 1;
    const double *vrow = A + (int64_t)j * n + j + 1;  // v[r] for r >= 1; v[0] = 1
    double *zj = zs + (j + 1) * W + c;
    double s0 = 0.0, s1 = 0.0;
    int r = g;
    for (; r + RG < m; r += 2 * RG) {
      const double v0 = r == 0 ? 1.0 : __ldg(vrow + r);
      const double v1 = __ldg(vrow + r + RG);
      s0 = fma(v0, zj[r * W], s0);
      s1 = fma(v1, zj[(r + RG) * W], s1);
    }
    if (r < m) s0 = fma(r == 0 ? 1.0 : __ldg(vrow + r), zj[r * W], s0);
    double sum = s0 + s1;
    // the row groups of this warp, then the warps
#pragma unroll
    for (int o = W; o < 32; o <<= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) < W) part[warp][c] = sum;
    __syncthreads();
    double w = 0.0;
#pragma unroll
    for (int q = 0; q < kBackThreads / 32; ++q) w += part[q][c];
    w *= t;
    for (int r2 = g; r2 < m; r2 += RG) zj[r2 * W] -= (r2 == 0 ? 1.0 : __ldg(vrow + r2)) * w;
    __syncthreads();
  }
  if (col)
    for (int r = g; r < n; r += RG) z[(int64_t)r * ch.ld + c] = zs[r * W + c];
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {  // conj(a) * b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}

// ---- Householder tridiagonalisation of one large matrix by several CTAs ----
//
// A matrix too large for shared memory is reduced by P co-resident CTAs (a
// cooperative launch): CTA p owns the rows i with i % P == p.  Step j uses
// the reflector v_j of row j and w_j = t_j A v_j - K v_j; one fused pass over
// each CTA's own rows applies the rank-2 update of step j and forms the
// matrix-vector product of step j + 1, so the trailing block is read and
// written once per step.  Per step the CTAs meet once, at a counter barrier
// (every w_j entry and partial sum is written); then every CTA applies step
// j's update to row j + 1 in its own shared memory (the same arithmetic in
// every CTA) and forms the next reflector from it.  The barrier gives up
// after kTriTimeoutNs and sets status 3.  Partial sums are added in CTA
// order, so the result does not depend on timing.
struct TriPart {
  int32_t job, p, P, slot;
  int64_t wb_off;  // 2 n scalars of w buffers (double-buffered by step parity)
};
struct TriSlot {  // one per matrix, zeroed before the launch
  unsigned int arrive;
  int pad[3];
};
constexpr int kTriMaxParts = 64;
constexpr unsigned long long kTriTimeoutNs = 2000000000ull;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ double cj(double a) { return a; }
__device__ __forceinline__ double2 cj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double smul(double a, double b) { return a * b; }
__device__ __forceinline__ double2 smul(double2 a, double2 b) { return cmul(a, b); }
__device__ __forceinline__ double sadd(double a, double b) { return a + b; }
__device__ __forceinline__ double2 sadd(double2 a, double2 b) { return cadd(a, b); }
__device__ __forceinline__ double ssub(double a, double b) { return a - b; }
__device__ __forceinline__ double2 ssub(double2 a, double2 b) {
  return make_double2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ double sre(double a) { return a; }
__device__ __forceinline__ double sre(double2 a) { return a.x; }
__device__ __forceinline__ double sim(double) { return 0.0; }
__device__ __forceinline__ double sim(double2 a) { return a.y; }
__device__ __forceinline__ double sabs2(double a) { return a * a; }
__device__ __forceinline__ double sabs2(double2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double samax(double a) { return fabs(a); }
__device__ __forceinline__ double samax(double2 a) { return fmax(fabs(a.x), fabs(a.y)); }
__device__ __forceinline__ bool sfinite(double a) { return isfinite(a); }
__device__ __forceinline__ bool sfinite(double2 a) { return isfinite(a.x) && isfinite(a.y); }
template <typename T> __device__ __forceinline__ T smake(double re, double im);
template <> __device__ __forceinline__ double smake<double>(double re, double) { return re; }
template <> __device__ __forceinline__ double2 smake<double2>(double re, double im) {
  return make_double2(re, im);
}
__device__ __forceinline__ double sscale(double s, double a) { return s * a; }
__device__ __forceinline__ double2 sscale(double s, double2 a) {
  return make_double2(s * a.x, s * a.y);
}
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double2 warp_sum(double2 v) {
  return make_double2(warp_sum(v.x), warp_sum(v.y));
}

// All CTAs of the matrix arrive; false (status 3) if the others do not
// arrive within the time limit.
__device__ bool tri_barrier(TriSlot *sl, unsigned target, int *status) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(&sl->arrive, 1u);
    const unsigned long long t0 = global_ns();
    int good = 1;
    while (*(volatile unsigned *)&sl->arrive < target) {
      if (global_ns() - t0 > kTriTimeoutNs) {
        good = 0;
        atomicExch(status, 3);
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Reflector of step j from row j, held in shared memory from its diagonal
// on (row[c - j] = A[j][c]): v (v_0 = 1) into v[0 .. m), returns tau; the CTA
// with writer set writes d[j], e[j], tau[j].  Same formulas as the
// single-CTA kernels.
template <typename T>
__device__ T tri_reflector(const T *row, int n, int j, T *v, double *red, bool writer, double *d,
                           double *e, T *tau) {
  const T *rowj = row - j;  // rowj[c] = A[j][c], c >= j
  const int m = n - j - 1;
  const T alpha = cj(rowj[j + 1]);
  double x2 = 0.0;
  for (int c = j + 2 + threadIdx.x; c < n; c += blockDim.x) x2 += sabs2(rowj[c]);
  x2 = block_sum(x2, red);
  T t = smake<T>(0.0, 0.0), sc = smake<T>(0.0, 0.0);
  double beta = sre(alpha);
  const bool refl = x2 > 0.0 || sim(alpha) != 0.0;
  if (refl) {
    beta = -copysign(sqrt(sabs2(alpha) + x2), sre(alpha));
    t = smake<T>((beta - sre(alpha)) / beta, -sim(alpha) / beta);
    const double dr = sre(alpha) - beta, di = sim(alpha), dd = dr * dr + di * di;
    sc = smake<T>(dr / dd, -di / dd);  // 1 / (alpha - beta)
  }
  for (int r = threadIdx.x; r < m; r += blockDim.x)
    v[r] = r == 0 ? smake<T>(1.0, 0.0)
                  : (refl ? smul(cj(rowj[j + 1 + r]), sc) : smake<T>(0.0, 0.0));
  if (writer && threadIdx.x == 0) {
    d[j] = sre(rowj[j]);
    e[j] = beta;
    tau[j] = t;
  }
  __syncthreads();
  return t;
}

template <typename T>
__global__ void __launch_bounds__(kTriThreads)
    tridiag_mc_kernel(const EigJob *__restrict__ jobs, const TriPart *__restrict__ parts,
                      T *__restrict__ G_all, double *__restrict__ d_all,
                      double *__restrict__ e_all, T *__restrict__ tau_all,
                      double *__restrict__ scale_all, TriSlot *__restrict__ slots,
                      T *__restrict__ wbuf_all, T *__restrict__ red_all,
                      int *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char tri_sm[];
  __shared__ double red[33];
  __shared__ T ksum;
  const TriPart pt = parts[blockIdx.x];
  const EigJob job = jobs[pt.job];
  const int n = job.n, p = pt.p, P = pt.P;
  TriSlot *sl = slots + pt.slot;
  T *A = G_all + job.g_off;
  T *wb = wbuf_all + pt.wb_off;
  T *rd = red_all + (int64_t)pt.slot * 2 * kTriMaxParts;
  double *d = d_all + job.lam_off, *e = e_all + job.lam_off;
  T *tau = tau_all + job.lam_off;
  T *vA = (T *)tri_sm, *vB = vA + n, *wA = vB + n, *rb = wA + n;  // rb: the next pivot row
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int nwarp = nt >> 5;
  unsigned nbar = 0;
  // first row >= lo owned by this CTA
  auto first_own = [&](int lo) { return lo + ((p - lo % P) + P) % P; };

  // 1. max-abs and finiteness of the own rows; partials in the w buffer
  double mx = 0.0;
  int nf = 0;
  for (int i = first_own(0) + P * warp; i < n; i += P * nwarp)
    for (int c = lane; c < n; c += 32) {
      const T g = A[(int64_t)i * n + c];
      nf |= !sfinite(g);
      mx = fmax(mx, samax(g));
    }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    nf |= __shfl_down_sync(0xffffffffu, nf, o);
  }
  __syncthreads();
  if (lane == 0) red[warp] = nf ? -1.0 : mx;
  __syncthreads();
  double *pw = (double *)wb;  // 2 P doubles (P <= n / 4)
  if (tid == 0) {
    double m = 0.0;
    int bad = 0;
    for (int i = 0; i < nwarp; ++i) {
      bad |= red[i] < 0.0;
      m = fmax(m, red[i]);
    }
    pw[p] = m;
    pw[P + p] = bad;
  }
  if (!tri_barrier(sl, ++nbar * P, status)) return;
  if (warp == 0) {
    double m = 0.0;
    int bad = 0;
    for (int q = lane; q < P; q += 32) {
      m = fmax(m, __ldcg(&pw[q]));
      bad |= __ldcg(&pw[P + q]) != 0.0;
    }
    for (int o = 16; o > 0; o >>= 1) {
      m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
      bad |= __shfl_down_sync(0xffffffffu, bad, o);
    }
    if (lane == 0) red[32] = bad ? -1.0 : m;
  }
  __syncthreads();
  const double scale = red[32];
  if (scale < 0.0) {  // every CTA sees the same flag and leaves
    if (tid == 0 && p == 0) atomicExch(status, 2);
    return;
  }
  if (tid == 0 && p == 0) scale_all[pt.job] = scale;
  const double inv = scale > 0.0 ? 1.0 / scale : 0.0;
  // 2. lower triangle of the own rows <- scaled conjugate of the upper triangle
  //    (exactly Hermitian; the upper triangle is not written in this phase)
  for (int i = first_own(0) + P * warp; i < n; i += P * nwarp) {
    T *ar = A + (int64_t)i * n;
    for (int c = lane; c < i; c += 32) ar[c] = sscale(inv, cj(__ldcg(&A[(int64_t)c * n + i])));
    if (lane == 0) ar[i] = smake<T>(inv * sre(ar[i]), 0.0);
  }
  if (!tri_barrier(sl, ++nbar * P, status)) return;
  // 3. upper triangle of the own rows scaled
  for (int i = first_own(0) + P * warp; i < n; i += P * nwarp) {
    T *ar = A + (int64_t)i * n;
    for (int c = i + 1 + lane; c < n; c += 32) ar[c] = sscale(inv, ar[c]);
  }
  if (!tri_barrier(sl, ++nbar * P, status)) return;

  // Own rows i >= lo: optional rank-2 update with (vA, wA) of step j = lo - 2,
  // then w[i - lo] = t * (row i, columns lo ..) . vn into wbuf, and the CTA's
  // partial sum of conj(w_i) vn_i into rd.
  auto rows_pass = [&](int lo, bool upd, const T *vn, T t, T *wout, T *rout) {
    const int j = lo - 2;
    T acc = smake<T>(0.0, 0.0);
    for (int i = first_own(lo) + P * warp; i < n; i += P * nwarp) {
      T *ar = A + (int64_t)i * n;
      T s = smake<T>(0.0, 0.0);
      if (upd) {
        const T vi = vA[i - j - 1], wi = wA[i - j - 1];
        for (int c = lo + lane; c < n; c += 32) {
          const T a = ssub(ar[c], sadd(smul(vi, cj(wA[c - j - 1])), smul(wi, cj(vA[c - j - 1]))));
          ar[c] = a;
          s = sadd(s, smul(a, vn[c - lo]));
        }
      } else {
        for (int c = lo + lane; c < n; c += 32) s = sadd(s, smul(ar[c], vn[c - lo]));
      }
      s = warp_sum(s);
      if (lane == 0) {
        const T wi = smul(t, s);
        wout[i - lo] = wi;
        acc = sadd(acc, smul(cj(wi), vn[i - lo]));
      }
    }
    // CTA partial, summed over warps in order
    __syncthreads();
    T *wp = (T *)(tri_sm + 4 * (size_t)n * sizeof(T));  // nwarp scalars
    if (lane == 0) wp[warp] = acc;
    __syncthreads();
    if (tid == 0) {
      T s = smake<T>(0.0, 0.0);
      for (int q = 0; q < nwarp; ++q) s = sadd(s, wp[q]);
      rout[p] = s;
    }
  };

  // step 0: reflector and products of the own rows
  for (int c = tid; c < n; c += nt) rb[c] = __ldcg(&A[c]);
  __syncthreads();
  T t = tri_reflector(rb, n, 0, vA, red, p == 0, d, e, tau);
  rows_pass(1, false, vA, t, wb, rd);
  for (int j = 0; j + 1 < n; ++j) {
    const int m = n - j - 1, par = j & 1;
    if (!tri_barrier(sl, ++nbar * P, status)) return;
    if (j % P == p)  // reflector storage; every CTA has read row j by now
      for (int c = j + 2 + tid; c < n; c += nt) A[(int64_t)j * n + c] = vA[c - j - 1];
    if (warp == 0) {  // the P partials: lane q holds q and q + 32, tree sum in lane order
      T s = smake<T>(0.0, 0.0);
      if (lane < P) s = __ldcg(&rd[par * kTriMaxParts + lane]);
      if (lane + 32 < P) s = sadd(s, __ldcg(&rd[par * kTriMaxParts + lane + 32]));
      s = warp_sum(s);
      if (lane == 0) ksum = smul(sscale(-0.5, t), s);  // K = -t (w^H v) / 2
    }
    __syncthreads();
    const T K = ksum;
    for (int r = tid; r < m; r += nt) wA[r] = sadd(__ldcg(&wb[par * n + r]), smul(K, vA[r]));
    __syncthreads();
    if (j + 2 == n) {  // the trailing block is the last diagonal entry
      if ((n - 1) % P == p && tid == 0) {
        T *a = A + (int64_t)(n - 1) * n + (n - 1);
        const T v0 = vA[0], w0 = wA[0];
        const T an = ssub(*a, sadd(smul(v0, cj(w0)), smul(w0, cj(v0))));
        *a = an;
        d[n - 1] = sre(an);
        e[n - 1] = 0.0;
        tau[n - 1] = smake<T>(0.0, 0.0);
      }
      break;
    }
    // row j + 1 (updated through step j - 1 by its owner) with step j's update
    {
      const T *ar = A + (int64_t)(j + 1) * n;
      const T v0 = vA[0], w0 = wA[0];
      for (int c = j + 1 + tid; c < n; c += nt)
        rb[c - j - 1] =
            ssub(__ldcg(&ar[c]), sadd(smul(v0, cj(wA[c - j - 1])), smul(w0, cj(vA[c - j - 1]))));
      __syncthreads();
    }
    const T tn = tri_reflector(rb, n, j + 1, vB, red, p == 0, d, e, tau);
    rows_pass(j + 2, true, vB, tn, wb + (par ^ 1) * n, rd + (par ^ 1) * kTriMaxParts);
    T *x = vA;
    vA = vB;
    vB = x;
    t = tn;
  }
}

// Complex Hermitian version of tridiag_kernel.  Step j (0 <= j <= n-2)
// reflects the column x = A[j+1.., j] (read as conj of row j) with
// H = I - tau v v^H, v_0 = 1, beta real, so that H^H x = beta e_0 and the
// tridiagonal matrix is real; v (r >= 1) is stored in row j at column j+1+r,
// tau (complex) in tau[lam_off + j].
__global__ void tridiag_c_kernel(const EigJob *__restrict__ jobs, double2 *__restrict__ G_all,
                                 double *__restrict__ d_all, double *__restrict__ e_all,
                                 double2 *__restrict__ tau_all, double *__restrict__ scale_all,
                                 int *__restrict__ status) {
  extern __shared__ double2 smc[];
  __shared__ double red[33];
  __shared__ double redi[33];
  __shared__ int bad;
  const EigJob job = jobs[blockIdx.x];
  const int n = job.n;
  if (n == 0 || !job.smem) return;  // larger matrices: tridiag_mc_kernel
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  double2 *A = smc;
  double2 *v = smc + (int64_t)n * n;
  double2 *w = v + n;
  double *d = d_all + job.lam_off, *e = e_all + job.lam_off;
  double2 *tau = tau_all + job.lam_off;

  for (int64_t x = tid; x < (int64_t)n * n; x += nt) A[x] = G_all[job.g_off + x];
  double mx = 0.0;
  int nf = 0;
  if (tid == 0) bad = 0;
  for (int64_t x = tid; x < (int64_t)n * n; x += nt) {
    const double2 g = A[x];
    nf |= !isfinite(g.x) || !isfinite(g.y);
    mx = fmax(mx, fmax(fabs(g.x), fabs(g.y)));
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    nf |= __shfl_down_sync(0xffffffffu, nf, o);
  }
  __syncthreads();
  if (lane == 0) {
    red[warp] = mx;
    if (nf) atomicOr(&bad, 1);
  }
  __syncthreads();
  if (tid == 0) {
    double m = 0.0;
    for (int i = 0; i < nwarp; ++i) m = fmax(m, red[i]);
    red[32] = m;
  }
  __syncthreads();
  if (bad) {
    if (tid == 0) atomicExch(status, 2);
    return;
  }
  const double scale = red[32];
  if (tid == 0) scale_all[blockIdx.x] = scale;
  // scale and make exactly Hermitian
  const double inv = scale > 0.0 ? 1.0 / scale : 0.0;
  for (int64_t x = tid; x < (int64_t)n * n; x += nt) {
    const int r = (int)(x / n), c = (int)(x - (int64_t)r * n);
    if (r < c) {
      const double2 a = A[x], b = A[(int64_t)c * n + r];
      const double2 g = make_double2(0.5 * inv * (a.x + b.x), 0.5 * inv * (a.y - b.y));
      A[x] = g;
      A[(int64_t)c * n + r] = make_double2(g.x, -g.y);
    } else if (r == c) {
      A[x] = make_double2(A[x].x * inv, 0.0);
    }
  }
  __syncthreads();

  for (int j = 0; j + 1 < n; ++j) {
    const int m = n - j - 1;
    double2 *rowj = A + (int64_t)j * n;
    const double2 alpha = make_double2(rowj[j + 1].x, -rowj[j + 1].y);  // x_0
    double x2 = 0.0;
    for (int c = j + 2 + tid; c < n; c += nt) x2 += rowj[c].x * rowj[c].x + rowj[c].y * rowj[c].y;
    x2 = block_sum(x2, red);
    double2 t = make_double2(0.0, 0.0), sc = make_double2(0.0, 0.0);
    double beta = alpha.x;
    if (x2 > 0.0 || alpha.y != 0.0) {
      beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + x2), alpha.x);
      t = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
      const double2 den = make_double2(alpha.x - beta, alpha.y);  // 1 / (alpha - beta)
      const double dd = den.x * den.x + den.y * den.y;
      sc = make_double2(den.x / dd, -den.y / dd);
    }
    const bool refl = t.x != 0.0 || t.y != 0.0;
    for (int r = tid; r < m; r += nt) {
      double2 vr;
      if (r == 0)
        vr = make_double2(1.0, 0.0);
      else if (!refl)
        vr = make_double2(0.0, 0.0);
      else
        vr = cmul(make_double2(rowj[j + 1 + r].x, -rowj[j + 1 + r].y), sc);
      v[r] = vr;
      if (r > 0) rowj[j + 1 + r] = vr;
    }
    if (tid == 0) {
      d[j] = rowj[j].x;
      e[j] = beta;
      tau[j] = t;
    }
    __syncthreads();
    if (!refl) continue;
    // w = t * A_t v (one warp per row)
    for (int r = warp; r < m; r += nwarp) {
      const double2 *ar = A + (int64_t)(j + 1 + r) * n + (j + 1);
      double2 acc = make_double2(0.0, 0.0);
      for (int c = lane; c < m; c += 32) acc = cadd(acc, cmul(ar[c], v[c]));
      for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
      }
      if (lane == 0) w[r] = cmul(t, acc);
    }
    __syncthreads();
    // K = -1/2 t (w^H v); w += K v
    double kr = 0.0, ki = 0.0;
    for (int r = tid; r < m; r += nt) {
      const double2 q = cmulc(w[r], v[r]);
      kr += q.x;
      ki += q.y;
    }
    kr = block_sum(kr, red);
    ki = block_sum(ki, redi);
    const double2 K = cmul(make_double2(-0.5 * t.x, -0.5 * t.y), make_double2(kr, ki));
    for (int r = tid; r < m; r += nt) w[r] = cadd(w[r], cmul(K, v[r]));
    __syncthreads();
    // A_t -= v w^H + w v^H
    for (int64_t x = tid; x < (int64_t)m * m; x += nt) {
      const int r = (int)(x / m), c = (int)(x - (int64_t)r * m);
      const double2 a = cmul(v[r], make_double2(w[c].x, -w[c].y));
      const double2 b = cmul(w[r], make_double2(v[c].x, -v[c].y));
      double2 &g = A[(int64_t)(j + 1 + r) * n + (j + 1 + c)];
      g = make_double2(g.x - a.x - b.x, g.y - a.y - b.y);
    }
    __syncthreads();
  }
  if (tid == 0) {
    d[n - 1] = A[(int64_t)(n - 1) * n + (n - 1)].x;
    e[n - 1] = 0.0;
    tau[n - 1] = make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int64_t x = tid; x < (int64_t)n * n; x += nt) G_all[job.g_off + x] = A[x];
}

// Complex back-transformation: Z <- H_0 H_1 ... H_{n-2} Z, H_j = I - tau_j v_j v_j^H.
__global__ void backtransform_c_kernel(const EigJob *__restrict__ jobs,
                                       const BackChunk *__restrict__ bt,
                                       const double2 *__restrict__ G_all,
                                       const double2 *__restrict__ tau_all,
                                       double2 *__restrict__ Z) {
  extern __shared__ double2 smc[];
  __shared__ double2 part[8][33];
  const BackChunk ch = bt[blockIdx.x];
  const EigJob job = jobs[ch.job];
  const int n = job.n;
  if (n < 2 || ch.cw == 0) return;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  double2 *z = Z + ch.z_off + ch.c0;
  double2 *v = smc;
  const double2 *A = G_all + job.g_off;
  const bool col = tx < ch.cw;
  for (int j = n - 2; j >= 0; --j) {
    const double2 t = tau_all[job.lam_off + j];
    if (t.x == 0.0 && t.y == 0.0) continue;
    const int m = n - j - 1;
    for (int r = threadIdx.x; r < m; r += blockDim.x)
      v[r] = r == 0 ? make_double2(1.0, 0.0) : A[(int64_t)j * n + j + 1 + r];
    __syncthreads();
    double2 s = make_double2(0.0, 0.0);
    if (col)
      for (int r = ty; r < m; r += 8) s = cadd(s, cmulc(v[r], z[(int64_t)(j + 1 + r) * ch.ld + tx]));
    part[ty][tx] = s;
    __syncthreads();
    double2 w = make_double2(0.0, 0.0);
    for (int g = 0; g < 8; ++g) w = cadd(w, part[g][tx]);
    w = cmul(t, w);
    if (col)
      for (int r = ty; r < m; r += 8) {
        double2 &zz = z[(int64_t)(j + 1 + r) * ch.ld + tx];
        const double2 q = cmul(v[r], w);
        zz = make_double2(zz.x - q.x, zz.y - q.y);
      }
    __syncthreads();
  }
}

}  // namespace

constexpr size_t kTriSmemBytes = 200 * 1024;

// Reduces the jobs without shared-memory residence with tridiag_mc_kernel.
// The SMs are shared out in proportion to n^3 (the flop count), at most
// kTriMaxParts and n / 8 CTAs per matrix; jobs that do not fit one
// cooperative launch go to the next.
template <typename T>
void tridiag_multi_cta(Ctx &ctx, DeviceScratch &scratch, const std::vector<EigJob> &jobs,
                       const SymEigWork &wk, double *G, int *dstat) {
  std::vector<int> big;
  double work = 0.0;
  int nmax = 0;
  for (int q = 0; q < (int)jobs.size(); ++q)
    if (!jobs[q].smem && jobs[q].n > 0) {
      big.push_back(q);
      work += std::pow((double)jobs[q].n, 3);
      nmax = std::max(nmax, jobs[q].n);
    }
  if (big.empty()) return;
  std::sort(big.begin(), big.end(), [&](int a, int b) { return jobs[a].n > jobs[b].n; });
  const void *kern = (const void *)tridiag_mc_kernel<T>;
  const size_t msmem = (4 * (size_t)nmax + kTriThreads / 32) * sizeof(T);
  UDMRG_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)msmem));
  int per_sm = 0;
  UDMRG_CHECK_CUDA(
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTriThreads, msmem));
  const int budget = std::min(ctx.num_sms, per_sm * ctx.num_sms);
  UDMRG_REQUIRE(budget >= 1, "eigensolver: the reduction kernel does not fit an SM");
  size_t at = 0;
  while (at < big.size()) {
    std::vector<TriPart> parts;
    int64_t wb_tot = 0;
    int slot = 0;
    for (; at < big.size(); ++at) {
      const int q = big[at], n = jobs[q].n;
      const double share = std::pow((double)n, 3) / work;
      int P = std::max(1, (int)(budget * share));
      P = std::min({P, kTriMaxParts, std::max(1, n / 8)});
      if (!parts.empty() && (int)parts.size() + P > budget) break;
      P = std::min(P, budget);
      for (int p = 0; p < P; ++p) parts.push_back(TriPart{q, p, P, slot, wb_tot});
      wb_tot += 2 * (int64_t)n;
      ++slot;
    }
    TriPart *dparts = scratch.get<TriPart>(parts.size());
    TriSlot *dslots = scratch.get<TriSlot>(slot);
    T *dwb = scratch.get<T>(wb_tot);
    T *dred = scratch.get<T>((int64_t)slot * 2 * kTriMaxParts);
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(dparts, parts.data(), parts.size() * sizeof(TriPart),
                                     cudaMemcpyHostToDevice, ctx.stream));
    UDMRG_CHECK_CUDA(cudaMemsetAsync(dslots, 0, slot * sizeof(TriSlot), ctx.stream));
    const EigJob *djobs = wk.jobs;
    T *g = (T *)G, *tau = (T *)wk.tau;
    double *d = wk.d, *e = wk.e, *sc = wk.scale;
    void *args[] = {&djobs, &dparts, &g, &d, &e, &tau, &sc, &dslots, &dwb, &dred, &dstat};
    UDMRG_CHECK_CUDA(cudaLaunchCooperativeKernel(kern, dim3((unsigned)parts.size()),
                                                 dim3(kTriThreads), args, msmem, ctx.stream));
    ctx.launches++;
    ctx.sync();  // `parts` must outlive the upload
  }
}

// Lower triangle of each job's matrix from its upper one: G[i][j] = conj(G[j][i]).
// One block per job walks the 32 x 32 tiles on and below the diagonal; each
// tile is read transposed from the upper triangle through shared memory, so
// both the reads and the writes are coalesced rows.
template <typename T>
__global__ void __launch_bounds__(256)
    sym_mirror_kernel(const EigJob *__restrict__ jobs, T *__restrict__ G) {
  __shared__ T tile[32][33];
  const EigJob job = jobs[blockIdx.x];
  const int n = job.n;
  const int nt = (n + 31) / 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  T *A = G + job.g_off;
  for (int t = 0; t < nt * (nt + 1) / 2; ++t) {
    // tile (bi, bj) with bi >= bj: row block bi of the lower triangle
    int bi = 0;
    while ((bi + 1) * (bi + 2) / 2 <= t) ++bi;
    const int bj = t - bi * (bi + 1) / 2;
    // source: rows bj*32.., columns bi*32.. (upper triangle)
    for (int r = ty; r < 32; r += 8) {
      const int i = bj * 32 + r, j = bi * 32 + tx;
      if (i < n && j < n) tile[r][tx] = A[(int64_t)i * n + j];
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
      const int i = bi * 32 + r, j = bj * 32 + tx;  // destination (i, j), i > j
      if (i < n && j < n && i > j) A[(int64_t)i * n + j] = cj(tile[tx][r]);
    }
    __syncthreads();
  }
}

int sym_eig_values(Ctx &ctx, DeviceScratch &scratch, std::vector<EigJob> &jobs, double *G,
                   double *lam, SymEigWork &wk, bool cplx, int64_t need, int64_t floor,
                   const std::vector<int64_t> *rank_cap, bool mirror) {
  const int nj = (int)jobs.size();
  if (nj == 0) return 0;
  int64_t ltot = 0;
  int nmax = 0;
  for (auto &j : jobs) {
    ltot = std::max<int64_t>(ltot, j.lam_off + j.n);
    nmax = std::max(nmax, j.n);
  }
  UDMRG_REQUIRE(nmax <= 4096, "eigensolver: matrix larger than 4096 is not supported");
  wk.d = scratch.get<double>(std::max<int64_t>(ltot, 1));
  wk.e = scratch.get<double>(std::max<int64_t>(ltot, 1));
  wk.tau = scratch.get<double>((cplx ? 2 : 1) * std::max<int64_t>(ltot, 1));
  wk.scale = scratch.get<double>(nj);
  wk.cplx = cplx;
  const size_t es = (cplx ? 2 : 1) * sizeof(double);
  size_t smem = 0;
  for (auto &j : jobs) {
    const size_t base = 2 * (size_t)j.n * es;
    const size_t full = base + (size_t)j.n * j.n * es;
    j.smem = full <= kTriSmemBytes ? 1 : 0;
    if (j.smem) smem = std::max(smem, full);
  }
  UDMRG_CHECK_CUDA(cudaFuncSetAttribute(tridiag_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)kTriSmemBytes));
  UDMRG_CHECK_CUDA(cudaFuncSetAttribute(tridiag_c_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)kTriSmemBytes));
  wk.jobs = scratch.get<EigJob>(nj);
  int *dstat = scratch.get<int>(1);
  UDMRG_CHECK_CUDA(cudaMemsetAsync(dstat, 0, sizeof(int), ctx.stream));
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(wk.jobs, jobs.data(), nj * sizeof(EigJob),
                                   cudaMemcpyHostToDevice, ctx.stream));
  if (mirror) {
    if (cplx)
      sym_mirror_kernel<double2><<<nj, 256, 0, ctx.stream>>>(wk.jobs, (double2 *)G);
    else
      sym_mirror_kernel<double><<<nj, 256, 0, ctx.stream>>>(wk.jobs, G);
    UDMRG_CHECK_CUDA(cudaGetLastError());
    ctx.launches++;
  }
  if (cplx)
    tridiag_c_kernel<<<nj, kTriThreads, smem, ctx.stream>>>(
        wk.jobs, (double2 *)G, wk.d, wk.e, (double2 *)wk.tau, wk.scale, dstat);
  else
    tridiag_kernel<<<nj, kTriThreads, smem, ctx.stream>>>(wk.jobs, G, wk.d, wk.e, wk.tau,
                                                          wk.scale, dstat);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  if (cplx)
    tridiag_multi_cta<double2>(ctx, scratch, jobs, wk, G, dstat);
  else
    tridiag_multi_cta<double>(ctx, scratch, jobs, wk, G, dstat);
  const size_t bsmem = 2 * (size_t)nmax * sizeof(double);
  if (bsmem > 48 * 1024) {
    UDMRG_CHECK_CUDA(cudaFuncSetAttribute(bisect_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bsmem));
    UDMRG_CHECK_CUDA(cudaFuncSetAttribute(grid_count_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bsmem));
  }
  // how many leading eigenvalues of each job to compute
  wk.computed.assign(nj, 0);
  wk.trace.clear();
  int64_t ntot = 0;
  for (int q = 0; q < nj; ++q) {
    wk.computed[q] = jobs[q].n;
    ntot += jobs[q].n;
  }
  double *dtop = nullptr;
  int *dcnt = nullptr;
  if (need > 0 && need < ntot) {
    dtop = scratch.get<double>(1);
    double *dtr = scratch.get<double>(nj);
    dcnt = scratch.get<int>((size_t)nj * (kGrid + 1));
    grid_top_kernel<<<1, 1024, 0, ctx.stream>>>(wk.jobs, nj, wk.d, wk.e, wk.scale, dtop);
    grid_count_kernel<<<nj, kGrid, bsmem, ctx.stream>>>(wk.jobs, wk.d, wk.e, wk.scale, dtop, dcnt,
                                                        dtr);
    UDMRG_CHECK_CUDA(cudaGetLastError());
    ctx.launches += 2;
    std::vector<int> cnt((size_t)nj * (kGrid + 1));
    wk.trace.assign(nj, 0.0);
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(cnt.data(), dcnt, cnt.size() * sizeof(int),
                                     cudaMemcpyDeviceToHost, ctx.stream));
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(wk.trace.data(), dtr, nj * sizeof(double),
                                     cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    // the first grid point with `need` eigenvalues above it, then one point
    // lower (a factor 1.34: near-ties and rounding at the threshold)
    int ks = -1;
    for (int k = 0; k <= kGrid; ++k) {
      int64_t t = 0;
      for (int q = 0; q < nj; ++q) {
        const int64_t c = cnt[(size_t)q * (kGrid + 1) + k];
        t += rank_cap ? std::min<int64_t>(c, (*rank_cap)[q]) : c;
      }
      if (t >= need) {
        ks = k;
        break;
      }
    }
    // fewer than `need` usable eigenvalues above the lowest grid point (a
    // rank-deficient set, and a Dmin asking for its null states too): every
    // eigenvalue
    if (ks >= 0) {
      ks = std::min(ks + 1, kGrid);
      for (int q = 0; q < nj; ++q) {
        const int64_t n = jobs[q].n;
        const int64_t c =
            std::max<int64_t>(cnt[(size_t)q * (kGrid + 1) + ks], std::min(n, floor));
        wk.computed[q] = std::min(c, n);
      }
    }
  }
  std::vector<int2> chunks;
  for (int q = 0; q < nj; ++q)
    for (int i0 = jobs[q].n - (int)wk.computed[q]; i0 < jobs[q].n; i0 += kBisectEigs)
      chunks.push_back(make_int2(q, i0));
  int2 *dch = scratch.get<int2>(chunks.size());
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(dch, chunks.data(), chunks.size() * sizeof(int2),
                                   cudaMemcpyHostToDevice, ctx.stream));
  if (!chunks.empty())
    bisect_kernel<<<(int)chunks.size(), 32, bsmem, ctx.stream>>>(
        wk.jobs, dch, wk.d, wk.e, wk.scale, lam, dtop, dcnt);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches += 2;
  int hstat = 0;
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(&hstat, dstat, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  return hstat;
}

void sym_eig_vectors(Ctx &ctx, DeviceScratch &scratch, const std::vector<EigJob> &jobs,
                     const double *G, const double *lam, const std::vector<double> &hlam,
                     const std::vector<int64_t> &k, const std::vector<int64_t> &z_off_out,
                     const std::vector<int64_t> &z_ld_out, double *Zout, const SymEigWork &wk,
                     uint64_t seed) {
  const int nj = (int)jobs.size();
  // the eigenvectors of the (real) tridiagonal matrix: in place for real
  // matrices, in a packed real buffer for complex ones
  double *Z = Zout;
  std::vector<int64_t> z_off = z_off_out, z_ld = z_ld_out;
  int64_t zr_tot = 0;
  if (wk.cplx) {
    for (int q = 0; q < nj; ++q) {
      z_off[q] = zr_tot;
      z_ld[q] = std::max<int64_t>(k[q], 1);
      zr_tot += (int64_t)jobs[q].n * k[q];
    }
    Z = scratch.get<double>(std::max<int64_t>(zr_tot, 1));
  }
  // clusters: descending neighbours closer than 1e-9 of the matrix's largest |eigenvalue|
  std::vector<EigCluster> cl;
  int nmax = 0;
  for (int q = 0; q < nj; ++q) {
    const int n = jobs[q].n;
    nmax = std::max(nmax, n);
    if (k[q] == 0) continue;
    const double *h = hlam.data() + jobs[q].lam_off;
    const int64_t nc = q < (int)wk.computed.size() ? wk.computed[q] : n;  // computed values
    const double big = std::max(std::fabs(h[0]), std::fabs(h[std::max<int64_t>(nc, 1) - 1]));
    const double tol = 1e-9 * big;
    int first = 0;
    for (int p = 1; p <= k[q]; ++p) {
      if (p == k[q] || h[p - 1] - h[p] > tol) {
        cl.push_back(EigCluster{z_off[q], z_ld[q], seed + 1000003ull * (uint64_t)q, q, first,
                                p - first, 0});
        first = p;
      }
    }
  }
  if (!cl.empty()) {
    const int ncl = (int)cl.size();
    EigCluster *dcl = scratch.get<EigCluster>(ncl);
    double *work = scratch.get<double>(6 * (int64_t)nmax * ncl);
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(dcl, cl.data(), ncl * sizeof(EigCluster),
                                     cudaMemcpyHostToDevice, ctx.stream));
    invit_kernel<<<(ncl + 63) / 64, 64, 0, ctx.stream>>>(dcl, ncl, wk.jobs, wk.d, wk.e, wk.scale,
                                                        lam, Z, work, nmax);
    UDMRG_CHECK_CUDA(cudaGetLastError());
    ctx.launches++;
  }
  // Newton-Schulz: Z <- 1.5 Z - 0.5 Z (Z^T Z), twice (grouped GEMMs)
  {
    int64_t stot = 0, ztot = 0;
    std::vector<int64_t> soff(nj), zc_off(nj);
    for (int q = 0; q < nj; ++q) {
      soff[q] = stot;
      stot += k[q] * k[q];
      zc_off[q] = ztot;
      ztot += (int64_t)jobs[q].n * k[q];
    }
    if (stot > 0) {
      DeviceScratch ns(ctx);
      double *S = ns.get<double>(stot), *Zc = ns.get<double>(ztot);
      GemmPlan gs, gz, gc;
      gs.ctx = gz.ctx = gc.ctx = &ctx;
      for (int q = 0; q < nj; ++q) {
        if (k[q] == 0) continue;
        const int64_t n = jobs[q].n, kk = k[q];
        // S = Z^T Z (k x k): A = Z^T (ms 1, ks ld), B = Z (ks ld, ns 1)
        gemm_add_simple(gs, soff[q], kk, kk, n, z_off[q], 1, z_ld[q], z_off[q], z_ld[q], 1, false);
        // Zc = Z S (n x k, packed): accumulated as Zc = -0.5 Z S + 1.5 Zc
        gemm_add_simple(gz, zc_off[q], n, kk, kk, z_off[q], z_ld[q], 1, soff[q], kk, 1, false);
      }
      gemm_finalize(gs);
      gemm_finalize(gz);
      std::vector<Copy2D> to_c, from_c;
      for (int q = 0; q < nj; ++q) {
        if (k[q] == 0) continue;
        to_c.push_back(Copy2D{z_off[q], zc_off[q], jobs[q].n, (int32_t)k[q], z_ld[q], 1, k[q], 1});
        from_c.push_back(
            Copy2D{zc_off[q], z_off[q], jobs[q].n, (int32_t)k[q], k[q], 1, z_ld[q], 1});
      }
      for (int it = 0; it < 2; ++it) {
        (ctx.svd_dw ? run_gemm_dw : run_gemm)(ctx, gs, kF64, Z, Z, S, 1.0, 0.0);
        run_copy2d(ctx, to_c, Z, Zc, false);
        (ctx.svd_dw ? run_gemm_dw : run_gemm)(ctx, gz, kF64, Z, S, Zc, -0.5, 1.5);
        run_copy2d(ctx, from_c, Zc, Z, false);
      }
    }
  }
  if (wk.cplx && zr_tot > 0) {  // real eigenvectors of T -> complex, into the caller's layout
    double *Zc = scratch.get<double>(2 * zr_tot);
    real_to_complex(ctx, Z, Zc, zr_tot);
    std::vector<Copy2D> ops;
    for (int q = 0; q < nj; ++q)
      if (k[q] > 0)
        ops.push_back(Copy2D{z_off[q], z_off_out[q], jobs[q].n, (int32_t)k[q], k[q], 1,
                             z_ld_out[q], 1});
    run_copy2d(ctx, ops, Zc, Zout, true);
  }
  // back-transformation by the reflectors: complex data 32 columns per block,
  // real data kBackCols columns per block (the chunk in shared memory)
  {
    const int narrow = nmax * 8 * (int)sizeof(double) <= 218 * 1024 ? 8 : 4;
    const int width = wk.cplx ? 32 : narrow;
    std::vector<BackChunk> bt;
    for (int q = 0; q < nj; ++q)
      for (int64_t c0 = 0; c0 < k[q]; c0 += width)
        bt.push_back(BackChunk{z_off_out[q], z_ld_out[q], q, (int32_t)c0,
                               (int32_t)std::min<int64_t>(width, k[q] - c0), 0});
    if (!bt.empty()) {
      BackChunk *dbt = scratch.get<BackChunk>(bt.size());
      UDMRG_CHECK_CUDA(cudaMemcpyAsync(dbt, bt.data(), bt.size() * sizeof(BackChunk),
                                       cudaMemcpyHostToDevice, ctx.stream));
      const size_t smem = wk.cplx ? (size_t)nmax * 2 * sizeof(double)
                                  : (size_t)nmax * narrow * sizeof(double);
      UDMRG_REQUIRE(smem <= 227 * 1024, "back transformation: matrix too large");
      if (smem > 48 * 1024) {
        UDMRG_CHECK_CUDA(cudaFuncSetAttribute(backtransform_narrow_kernel<8>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
        UDMRG_CHECK_CUDA(cudaFuncSetAttribute(backtransform_narrow_kernel<4>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
        UDMRG_CHECK_CUDA(cudaFuncSetAttribute(backtransform_c_kernel,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
      }
      if (wk.cplx)
        backtransform_c_kernel<<<(int)bt.size(), kBackThreads, smem, ctx.stream>>>(
            wk.jobs, dbt, (const double2 *)G, (const double2 *)wk.tau, (double2 *)Zout);
      else if (narrow == 8)
        backtransform_narrow_kernel<8><<<(int)bt.size(), kBackThreads, smem, ctx.stream>>>(
            wk.jobs, dbt, G, wk.tau, Zout);
      else
        backtransform_narrow_kernel<4><<<(int)bt.size(), kBackThreads, smem, ctx.stream>>>(
            wk.jobs, dbt, G, wk.tau, Zout);
      UDMRG_CHECK_CUDA(cudaGetLastError());
      ctx.launches++;
    }
  }
  ctx.sync();  // host vectors above must outlive the uploads
}

}  // namespace udmrg
