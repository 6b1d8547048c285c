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
  int32_t smem;     // set by run_jacobi_eig
};

struct ScaleJob {
  int64_t x_off, f_off;
  int32_t rows, cols;
  int32_t by_row, pad;
};

constexpr size_t kJacobiSmemBytes = 200 * 1024;

void run_copy2d(Ctx &ctx, const std::vector<Copy2D> &ops, const double *src, double *dst,
                bool cplx);
// Returns 0, or 1 when some sector did not converge within the sweep limit.
int run_jacobi_eig(Ctx &ctx, const std::vector<EigJob> &jobs, double *G, double *V, double *W,
                   double *lam);
void run_scale(Ctx &ctx, const std::vector<ScaleJob> &jobs, double *X, const double *f, bool cplx);

// Kept-state selection over all bond sectors (the rule of the oracle):
// singular values ordered by descending size, ties within rtol*s_max ordered by
// (sector, position); keep the smallest D in [min(Dmin,n), min(Dmax,n)] whose
// discarded weight sum_{discarded} s^2 / sum s^2 <= trunc_err.
void select_kept(const std::vector<std::vector<double>> &svals, double trunc_err, int64_t Dmin,
                 int64_t Dmax, std::vector<int64_t> &kept, int64_t &D, double &err,
                 double rtol = 1e-12);

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
};

SvdResult svd_trunc(Ctx &ctx, const BTensor &T, int ldims, const QN &ldiv, double trunc_err,
                    int64_t Dmin, int64_t Dmax, int mode);

}  // namespace udmrg
