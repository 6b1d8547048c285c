// Truncated block SVD of a block tensor viewed as (left axes) x (right axes).
#pragma once

#include "gemm.hpp"
#include "vecops.hpp"

namespace udmrg {

struct Copy2D {
  int64_t src_off, dst_off;
  int32_t rows, cols;
  int64_t src_ld, src_cs, dst_ld, dst_cs;
};

struct EigJob {
  int64_t g_off;    // offset of the n x n matrix in the G / V / W buffers
  int64_t lam_off;  // offset of the n eigenvalues
  int32_t n;
  int32_t smem;     // set by sym_eig_values (matrix held in shared memory)
};

// Batched symmetric eigen-solver (Householder tridiagonalisation, bisection,
// inverse iteration, Newton-Schulz orthonormalisation, back-transformation).
struct EigCluster {  // eigenvalues close enough to share a Gram-Schmidt sweep
  int64_t z_off, ld;
  uint64_t seed;
  int32_t job, first, count, pad;
};
struct SymEigWork {
  EigJob *jobs = nullptr;  // device copy of the jobs
  double *d = nullptr, *e = nullptr, *tau = nullptr, *scale = nullptr;
  bool cplx = false;  // complex Hermitian matrices (interleaved re, im; tau complex)
  // host: eigenvalues computed per job (the leading ones; all by default) and
  // each job's trace (the sum of all its eigenvalues)
  std::vector<int64_t> computed;
  std::vector<double> trace;
};

struct ScaleJob {
  int64_t x_off, f_off;
  int32_t rows, cols;
  int32_t by_row, pad;
};


void run_copy2d(Ctx &ctx, const std::vector<Copy2D> &ops, const double *src, double *dst,
                bool cplx);
void run_scale(Ctx &ctx, const std::vector<ScaleJob> &jobs, double *X, const double *f, bool cplx);

// Kept-state selection over all bond sectors (the rule of the oracle):
// singular values ordered by descending size, ties within rtol*s_max ordered by
// (sector, position); keep the smallest D in [min(Dmin,n), min(Dmax,n)] whose
// discarded weight sum_{discarded} s^2 / sum s^2 <= trunc_err.
// Phase 1: reduce every job's symmetric n x n matrix in G to tridiagonal form
// (G keeps the reflectors) and put its eigenvalues, descending, at
// lam[lam_off ...].  Returns 0, 2 for non-finite input, 3 if the multi-CTA
// reduction timed out.  jobs[].smem is set.  With cplx, G holds complex
// Hermitian matrices (offsets in complex elements) and phase 2 returns
// complex eigenvectors.
// need > 0 (positive semi-definite matrices, e.g. Gram matrices): only the
// leading eigenvalues of every job down to a common threshold below which
// fewer than `need` eigenvalues of all jobs together lie above, at least
// min(n, floor) per job, are computed (wk.computed); wk.trace holds each job's
// trace, so the weight of the rest is known exactly.  rank_cap (optional, one
// per job): the caller uses at most that many of the job's eigenvalues (a Gram
// matrix of rank min(rows, cols)), so no more of them count towards `need`.
// mirror: only the upper triangles of the matrices hold data; the lower ones
// are filled from them first (conjugated for complex data).
int sym_eig_values(Ctx &ctx, DeviceScratch &scratch, std::vector<EigJob> &jobs, double *G,
                   double *lam, SymEigWork &wk, bool cplx = false, int64_t need = 0,
                   int64_t floor = 0, const std::vector<int64_t> *rank_cap = nullptr,
                   bool mirror = false);
// Phase 2: the leading k[q] eigenvectors of job q (hlam: host copy of lam) as
// the columns of Z (row-major n x k[q], leading dimension z_ld[q], at z_off[q]),
// orthonormal to FP64 accuracy.
void sym_eig_vectors(Ctx &ctx, DeviceScratch &scratch, const std::vector<EigJob> &jobs,
                     const double *G, const double *lam, const std::vector<double> &hlam,
                     const std::vector<int64_t> &k, const std::vector<int64_t> &z_off,
                     const std::vector<int64_t> &z_ld, double *Z, const SymEigWork &wk,
                     uint64_t seed = 0x5EED5EEDull);

void select_kept(const std::vector<std::vector<double>> &svals, double trunc_err, int64_t Dmin,
                 int64_t Dmax, std::vector<int64_t> &kept, int64_t &D, double &err,
                 double rtol = 1e-12, double extra_mass = 0.0);

void fill_normal(Ctx &ctx, double *x, int64_t n, uint64_t seed);
// out[f_off + j] = sum_i X[x_off + i * cols + j]^2 for every job (by_row unused)
void run_col_sumsq(Ctx &ctx, const std::vector<ScaleJob> &jobs, const double *X, double *out);
// S (per job, n x n PSD) -> R^{-T} (row-major, i.e. R^{-1} column-major) with
// S = R^T R (pivots below rel_tol drop)
void run_chol_inv(Ctx &ctx, const std::vector<EigJob> &jobs, double *S, double *Rinv,
                  double rel_tol);

enum SvdMode : int {
  kSvdFull = 0,        // u, s, vt with M = u s vt
  kSvdSplitLeft = 1,   // u (isometry) and vt := s vt (centre moves right)
  kSvdSplitRight = 2,  // vt (isometry) and u := u s (centre moves left)
};

struct SvdResult {
  TensorPtr u, s, vt;
  double trunc_err = 0;
  int64_t D = 0;
  std::vector<double> svals;  // kept singular values, bond-sector order
  double ee = 0;              // -sum s^2 log s^2 over kept values
  // per bond sector (ascending QN): QN, matrix shape, kept count, sketch size
  // (randomized path; 0 for the exact one) and the leading singular values
  std::vector<QN> sector_qn;
  std::vector<int64_t> sector_rows, sector_cols, sector_kept, sector_sketch;
  std::vector<std::vector<double>> sector_svals;
  int64_t grow_rounds = 0;  // randomized path: sketch enlargements after a miss
};

// Leading singular values per sector that the rank model reads.
constexpr int64_t kSpectrumFloor = 64;

// Exact truncated SVD.  Only the leading singular values of the sectors are
// computed (all of them when Dmax does not truncate); spectrum_floor: at
// least that many per sector (the leading values the rank model reads).
SvdResult svd_trunc(Ctx &ctx, const BTensor &T, int ldims, const QN &ldiv, double trunc_err,
                    int64_t Dmin, int64_t Dmax, int mode, int64_t spectrum_floor = 0);

// Sector-wise randomized truncated SVD.  For every bond sector a Gaussian
// sketch of `sketch[q]` columns (default: full rank, i.e. exact) spans the
// dominant subspace after `power_iters` power iterations with Cholesky-QR
// re-orthonormalisation; the projected problem is solved exactly (FP64 Gram +
// Jacobi).  Discarded weight counts the exact residual mass outside the
// sketches.  A sector whose sketch is entirely kept is a miss: its sketch
// grows (x2) and the decomposition is repeated, up to full rank, so the kept
// set never depends on a too-small sketch.
struct SketchParams {
  std::vector<std::pair<QN, int64_t>> sketch;  // requested sketch size per bond QN
  int64_t oversample = 8;
  int power_iters = 4;
  uint64_t seed = 1;
  // cost rule: if the total sketch exceeds this fraction of the total sector
  // dimension, the exact SVD is cheaper and runs instead (1: never)
  double max_fraction = 1.0;
};
SvdResult svd_trunc_sketch(Ctx &ctx, const BTensor &T, int ldims, const QN &ldiv,
                           double trunc_err, int64_t Dmin, int64_t Dmax, int mode,
                           const SketchParams &sp);

}  // namespace udmrg
