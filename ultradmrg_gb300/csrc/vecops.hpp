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

// Krylov basis with device-resident step scalars.  Every kernel of a step
// reads the step index s from device memory (KrylovWork::step) and works on
// two fixed buffers (X = v_s, the matvec input; Y = H v_s, which becomes
// gamma_s), so the launch sequence of a step is the same for every s and is
// captured once as a CUDA graph.  One host synchronisation per step reads
// alpha_s and |gamma_s|^2 for the tridiagonal matrix.
struct KrylovWork {
  Ctx &ctx;
  int64_t n = 0;  // elements (complex or real)
  bool cplx = false;
  int mcap = 0;                     // largest basis a projection sees (steps + 1)
  int nb = 0;                       // blocks of the multi-dot kernel
  double *partial = nullptr;        // mcap x nb x 2 multi-dot partials
  double *red = nullptr;            // reduction partials of the fused norms
  double *gate = nullptr;           // |gamma|^2 before / after the first projection
  double *coef = nullptr;           // kMaxVecs x 2 projection coefficients
  double *alpha = nullptr;          // kMaxVecs x 2: <v_s | H v_s>
  double *nrm2 = nullptr;           // kMaxVecs + 2: nrm2[s] = |gamma_{s-1}|^2 (s = 0: |v0|^2)
  const double **ptrs = nullptr;    // device array of the basis pointers
  const double **hptrs = nullptr;   // pinned mirror (entries written once)
  int *step = nullptr;              // device: the step the next launch sequence runs
  double *X = nullptr, *Y = nullptr;
  double *hres = nullptr;  // mapped pinned: {alpha_s, |gamma_s|^2, |gamma_{s-1}|^2}
  double *dres = nullptr;  // device alias of hres
  // max_steps: the most steps a solve may run (its Krylov dimension cap)
  KrylovWork(Ctx &c, int64_t n_elems, bool complex_data, int64_t max_steps);
  ~KrylovWork();
  // registers basis vector j; the step j normalisation writes it
  void push(int j, const double *v);
};
// Y = v0 (a copy), nrm2[0] = |v0|^2, step = 0
void krylov_begin(KrylovWork &k, const double *v0);
// v_s = Y / sqrt(nrm2[s]) (Y itself when that norm is zero), written to the
// registered basis vector s and to X
void krylov_normalise(KrylovWork &k);
// alpha[s] = <X | Y>
void krylov_alpha(KrylovWork &k);
// Y -= Re(alpha[s]) X + sqrt(nrm2[s]) v_{s-1} (the second term when s > 0);
// nrm2[s+1] = |Y|^2
void krylov_update(KrylovWork &k);
// Y -= sum_{i <= s} <v_i | Y> v_i (one classical Gram-Schmidt pass);
// nrm2[s+1] = |Y|^2.  The second pass runs (decided on the device) only if
// the first one reduced |Y|^2 below half its value.
void krylov_project(KrylovWork &k, bool second);
// hres = {Re alpha[s], nrm2[s+1], nrm2[s]}; step = s + 1
void krylov_publish(KrylovWork &k);
// Device times (best of four, ms) of one Krylov step's vector kernels at
// step s on vectors of n doubles: ms[0] normalise, ms[1] alpha, ms[2]
// three-term update, ms[3] the first projection pass (multi-dot and
// projection against v_0 .. v_s), ms[4] the second (gated) pass; bytes[]
// the HBM bytes each moves (0 for a second pass the gate skipped).
void krylov_step_probe(Ctx &ctx, int64_t n, int s, double ms[5], double bytes[5],
                       int *second_ran);

}  // namespace udmrg
