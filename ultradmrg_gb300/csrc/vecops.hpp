// Krylov vector operations on device buffers.
#pragma once

#include <cstring>

#include "btensor.hpp"

namespace udmrg {

constexpr int kMaxVecs = 512;

struct VecWork {
  Ctx &ctx;
  double *partial = nullptr;  // reduction partials
  double *result = nullptr;   // small device results
  const double **ptrs = nullptr;
  double *coefs = nullptr;
  explicit VecWork(Ctx &c);
  ~VecWork();
};

// <x|y> = sum conj(x_i) y_i over n elements (complex when cplx).
std::complex<double> dot(VecWork &w, const double *x, const double *y, int64_t n, bool cplx);
void dot_async(VecWork &w, const double *x, const double *y, int64_t n, bool cplx, double *dres);
// g -= c1*v1 + c2*v2 over n doubles (v2 may be null); writes |g|^2 to dnorm2.
void lanczos_update_async(VecWork &w, double *g, const double *v1, const double *v2, double c1,
                          double c2, int64_t n_doubles, double *dnorm2);
double norm2(VecWork &w, const double *x, int64_t n_doubles);
void scale(Ctx &ctx, double *x, int64_t n_doubles, double s);
// out = sum_j coef_j vecs_j; coef interleaved (re, im) pairs when cplx, else plain reals.
void lincomb(VecWork &w, double *out, const std::vector<const double *> &vecs,
             const std::vector<double> &coef, int64_t n, bool cplx);
void conj_inplace(Ctx &ctx, double *x, int64_t n_cplx);
void real_to_complex(Ctx &ctx, const double *x, double *y, int64_t n);

}  // namespace udmrg
