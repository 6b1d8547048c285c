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
double norm2(VecWork &w, const double *x, int64_t n_doubles);
void scale(Ctx &ctx, double *x, int64_t n_doubles, double s);
// out = sum_j coef_j vecs_j; coef interleaved (re, im) pairs when cplx, else plain reals.
void lincomb(VecWork &w, double *out, const std::vector<const double *> &vecs,
             const std::vector<double> &coef, int64_t n, bool cplx);
void conj_inplace(Ctx &ctx, double *x, int64_t n_cplx);
void real_to_complex(Ctx &ctx, const double *x, double *y, int64_t n);

// Krylov basis with device-resident step scalars: the three-term update, the
// projection against the whole basis and the normalisation read their
// coefficients from device memory, so a Lanczos step needs one host
// synchronisation (to read alpha and |gamma|^2 for the tridiagonal matrix).
struct KrylovWork {
  Ctx &ctx;
  int64_t n = 0;  // elements (complex or real)
  bool cplx = false;
  int nb = 0;                       // blocks of the multi-dot kernel
  double *partial = nullptr;        // kMaxVecs x nb x 2 multi-dot partials
  double *red = nullptr;            // reduction partials of the fused norms
  double *gate = nullptr;           // |gamma|^2 before / after the first projection
  double *coef = nullptr;           // kMaxVecs x 2 projection coefficients
  double *alpha = nullptr;          // kMaxVecs x 2: <v_j | H v_j>
  double *nrm2 = nullptr;           // kMaxVecs: |gamma_j|^2
  const double **ptrs = nullptr;    // device array of the basis pointers
  const double **hptrs = nullptr;   // pinned mirror (entries written once)
  double *hres = nullptr;           // pinned host results
  KrylovWork(Ctx &c, int64_t n_elems, bool complex_data);
  ~KrylovWork();
  // registers basis vector j (j = number of vectors so far)
  void push(int j, const double *v);
};
// Scalars on the device: alpha[j] = <v_j | H v_j>; nrm2[i] = |gamma|^2 of the
// vector that becomes v_i.
// alpha[j] = <v_j | y>
void krylov_alpha(KrylovWork &k, int j, const double *y);
// g (= H v_j on entry) -= Re(alpha[j]) v_j + sqrt(nrm2[j]) v_{j-1} (the
// second term when j > 0); nrm2[j+1] = |g|^2
void krylov_update(KrylovWork &k, int j, double *g);
// g -= sum_{i <= j} <v_i | g> v_i (one classical Gram-Schmidt pass);
// nrm2[j+1] = |g|^2.  The second pass runs (decided on the device) only if
// the first one reduced |g|^2 below half its value.
void krylov_project(KrylovWork &k, int j, double *g, bool second);
// g /= sqrt(nrm2[j+1]) (unchanged when that norm is zero)
void krylov_normalise(KrylovWork &k, int j, double *g);
// hres[0] = Re alpha[j], hres[1] = nrm2[j+1]; synchronises the stream
void krylov_fetch(KrylovWork &k, int j);

}  // namespace udmrg
