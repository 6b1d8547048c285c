// Two-site update: matvec plan, Lanczos solvers, environment updates, sweeps.
#pragma once

#include "mpo_step.hpp"
#include "rank_mlp.hpp"
#include "sg_matvec.hpp"
#include "svd.hpp"

namespace udmrg {

// Matvec precision: plain FP64 block GEMMs, or split-BF16 tcgen05 GEMMs with
// FP32 accumulation (Krylov vectors, dots and the tridiagonal problem stay FP64).
enum Precision : int { kPrecFP64 = 0, kPrecMixed = 1 };

// Block-sparse ops built on plan + run.
TensorPtr contract_axes(Ctx &ctx, const BTensor &A, const BTensor &B, const std::vector<int> &ca,
                        const std::vector<int> &cb);
TensorPtr contract_cyclic(Ctx &ctx, const BTensor &A, const BTensor &B, int a_start, int b_start,
                          int n, bool dw = false);
TensorPtr dag(Ctx &ctx, const BTensor &A);
TensorPtr to_complex(Ctx &ctx, const BTensor &A);
// Same data laid out in the (superset) structure `dst` (missing blocks zero).
TensorPtr embed(Ctx &ctx, const BTensor &src, const BTensor &dst_struct);
// Union of two block structures over identical indexes (structure only).
TensorPtr struct_union(const BTensor &a, const BTensor &b);

// H_eff * psi for fixed (L, W1, W2, R), with psi and the result in one
// "Krylov structure": the smallest block set containing psi0's blocks that is
// closed under the matvec.  Reference: eff_ham_mul_two_site_state,
// algorithm/vmps/lanczos_vmps_solver_impl.h:260-289 (same four contractions).
struct MatvecPlan {
  Ctx *ctx = nullptr;
  const BTensor *L = nullptr, *W1 = nullptr, *W2 = nullptr, *R = nullptr;
  TensorPtr sstruct;  // the Krylov structure (no data)
  std::unique_ptr<ContractPlan> p1, p2, p3, p4;
  std::vector<int64_t> missing;  // blocks of sstruct the matvec does not write
  double *t1 = nullptr, *t2 = nullptr, *t3 = nullptr;
  double flops = 0;  // algorithmic flops of one matvec
  int precision = kPrecFP64;
  int sites = 2;  // 1: single-site form (L, W1, R; p3 unused)
  std::unique_ptr<SgMatvecPlan> sg;  // the mixed-precision form
  // real two-site FP64 form: the two MPO steps as one sparse channel map
  // (p2, p3 then only describe the intermediate structures)
  std::unique_ptr<MpoStep64> m64;
  // host seconds of the plan's construction: 0 Krylov closure (and the W1 W2
  // download), 1 the host tables built on host threads (contraction plans,
  // FP64 MPO step, mixed form when its tiles are known), 2 their uploads,
  // 3 the mixed form's tables alone (a part of 1, or of 4), 4 the mixed
  // form's device part (with the tile trials of a new shape class), 5 FP64
  // workspaces and GEMM tile tuning
  double build_sec[6] = {0, 0, 0, 0, 0, 0};
  ~MatvecPlan();
  void apply(const double *in, double *out);       // device buffers in sstruct layout
  // always an FP64-accurate form: the plain FP64 GEMMs, or (dw) the
  // double-word FP32 ones for real data
  void apply_fp64(const double *in, double *out, bool dw = false);
  // the mixed solver's anchor: apply_fp64 with the context's anchor_dw
  void apply_anchor(const double *in, double *out) { apply_fp64(in, out, ctx->anchor_dw); }
};

std::unique_ptr<MatvecPlan> plan_matvec2(Ctx &ctx, const BTensor &L, const BTensor &W1,
                                         const BTensor &W2, const BTensor &R,
                                         const BTensor &psi0, int precision = kPrecFP64);

// H_eff * psi of one site (eff_ham_mul_single_site_state,
// lanczos_vmps_solver_impl.h:291-304): L * psi, * W (cyclic 1,0,2), * R
// (cyclic 3,1,2).  FP64 form only.
std::unique_ptr<MatvecPlan> plan_matvec1(Ctx &ctx, const BTensor &L, const BTensor &W,
                                         const BTensor &R, const BTensor &psi0);

struct LanczosParams {
  double error = 1e-7;
  int64_t max_iterations = 200;
  int precision = kPrecFP64;
};

struct LanczosResult {
  int64_t iters = 0;
  double gs_eng = 0;
  TensorPtr gs_vec;
  double matvec_seconds = 0;  // device time spent in matvecs (CUDA events)
  int64_t matvecs = 0;
  double ritz_eng = 0;       // mixed precision: the Ritz value before the refinement
  int64_t fp64_matvecs = 0;  // mixed precision: FP64 matvecs (the refinement's first step)
};

// Ground state by Lanczos (lanczos_vmps_solver_impl.h:114-248): three-term
// recurrence (FP64 form: without reorthogonalisation, as the reference),
// all bases kept on the device, FP64 tridiagonal eigenproblem on the host.
// With the mixed-precision matvec the solve is followed by a refinement run
// started from its Ritz vector whose first step is an FP64 matvec; gs_eng is
// that run's Ritz value (ritz_eng: the first run's).
LanczosResult lanczos_gs(Ctx &ctx, MatvecPlan &mv, const BTensor &init_state,
                         const LanczosParams &p);

// exp(-i dt H_eff) psi (lanczos_expmv_solver_impl.h:70-184).
struct ExpmvResult {
  int64_t iters = 0;
  TensorPtr expmv;
};
ExpmvResult lanczos_expmv(Ctx &ctx, MatvecPlan &mv, const BTensor &init_state, double step,
                          const LanczosParams &p);

// Host tridiagonal eigen-solver (implicit QL with shifts).  Returns the lowest
// eigenvalue; if vec != nullptr, the matching normalised eigenvector.
double tridiag_lowest(const std::vector<double> &a, const std::vector<double> &b, int64_t n,
                      std::vector<double> *vec);
// All eigenpairs (ascending); z is row-major n x n with eigenvectors as columns.
void tridiag_eig(const std::vector<double> &a, const std::vector<double> &b, int64_t n,
                 std::vector<double> &w, std::vector<double> &z);
// exp(-i dt T) e1 for tridiagonal T (interleaved complex output).
std::vector<double> tridiag_expme1(const std::vector<double> &a, const std::vector<double> &b,
                                   int64_t n, double dt);

// Environment updates (algorithm/vmps/vmps_init.h:343-373).
// dw: the contractions of real data in double-word FP32 arithmetic (the
// mixed-precision sweep's environments, 2^-48 relative per product).
TensorPtr update_site_lenv(Ctx &ctx, const BTensor &lenv, const BTensor &A, const BTensor &W,
                           bool dw = false);
TensorPtr update_site_renv(Ctx &ctx, const BTensor &renv, const BTensor &A, const BTensor &W,
                           bool dw = false);
TensorPtr trivial_renv(Ctx &ctx, const BTensor &mps_last, const BTensor &mpo_last);
TensorPtr trivial_lenv(Ctx &ctx, const BTensor &mps_first, const BTensor &mpo_first);

enum SvdChoice : int { kSvdExact = 0, kSvdSketchPrev = 1, kSvdSketchLearned = 2 };

struct SweepParams {
  int64_t sweeps = 1;
  int64_t Dmin = 1, Dmax = 1;
  double trunc_err = 0;
  LanczosParams lancz;
  int svd_mode = kSvdExact;
  int64_t svd_oversample = 8;
  bool svd_audit = false;  // judge every randomized SVD by the exact one
  double svd_sketch_max_fraction = 1.0;  // cost rule of the randomized SVD (1: off)
};

struct SiteLog {
  int64_t site;
  double e0, trunc_err;
  int64_t D, iters;
  double ee, lancz_sec, svd_sec, env_sec, tot_sec;
  double matvec_flops;
  int64_t svd_sketch_total;  // sum of the final sketch sizes (0: exact SVD)
  int64_t svd_grow_rounds;   // sketch enlargements after a miss
  double svd_audit_err;      // |trunc_err - exact SVD's| (-1: not audited)
  int64_t svd_audit_kept_diff;  // kept states differing from the exact SVD's
  double plan_sec = 0.0;     // host time building the matvec plan (part of lancz_sec)
};

// Sketch sizes of the randomized SVD per bond QN.
using SketchHint = std::vector<std::pair<QN, int64_t>>;
// Spectra of the last SVD at a bond: bond QN -> leading singular values.
using BondSpectra = std::vector<std::pair<QN, std::vector<double>>>;

// One local update (TwoSiteFiniteVMPSUpdate, two_site_update_finite_vmps_impl.h:232-373):
// Lanczos on the bond (l, l+1), truncated SVD, MPS split by direction, and the
// environment grown by one site in that direction.
struct LocalUpdate {
  TensorPtr mps_l, mps_r, env;
};
// hint: sketch sizes for the randomized SVD (learned mode); spectra: receives
// the leading singular values of every bond sector of this update.
LocalUpdate two_site_update_local(Ctx &ctx, const BTensor &lenv, const BTensor &renv,
                                  const BTensor &mps_l, const BTensor &mps_r,
                                  const BTensor &mpo_l, const BTensor &mpo_r,
                                  const SweepParams &p, char dir, SiteLog *log,
                                  const SketchHint *hint = nullptr,
                                  BondSpectra *spectra = nullptr);

// Noise fields of FiniteVMPSSweepParams (finite_vmps_sweep_params.h:31-107):
// the starting noise of each sweep (the last one repeats) and its adaptation.
struct NoiseParams {
  std::vector<double> noises;
  // defaults: kVMPSNoiseDecreaseRate, kVMPSNoiseIncreaseRate, kVMPSMaxNoise,
  // kVMPSNoiseAlpha (finite_vmps_sweep_params.h:25-28)
  double noise_decrease = 0.95, noise_increase = 1.02, max_noise = 1.0, alpha = 0.3;
};

// TwoSiteFiniteVMPSWithNoise (two_site_update_noise_finite_vmps_impl.h:81-556):
// boundaries from the edges, adaptive noise, subspace expansion of every
// update's bond (noise.cpp).  No noises: the plain sweep.  noise_log: the
// noise applied at each update (0: no expansion).  The MPS centre must be at
// site 0 on entry.
double two_site_finite_vmps_noise(Ctx &ctx, std::vector<TensorPtr> &mps,
                                  const std::vector<const BTensor *> &mpo, const SweepParams &p,
                                  const NoiseParams &np, std::vector<SiteLog> *log,
                                  std::vector<double> *noise_log);

// Learned truncation state: the rank model (used when svd_mode ==
// kSvdSketchLearned), the spectra and kept counts of every bond at its last
// visit (kept across sweep calls on the same chain, so a schedule of sweeps
// with growing Dmax keeps its history), and (when record) training samples:
// features of each bond sector from the previous visit and the label
// log2(1 + kept now).
struct LearnState {
  RankModel *model = nullptr;
  bool record = false;
  std::vector<BondSpectra> prev;
  std::vector<std::vector<std::pair<QN, int64_t>>> prev_kept;
  std::vector<float> x, y;
};

// TwoSiteFiniteVMPS (two_site_update_finite_vmps_impl.h:95-494), device
// resident: mps tensors are replaced in place; returns the last energy.
double two_site_finite_vmps(Ctx &ctx, std::vector<TensorPtr> &mps,
                            const std::vector<const BTensor *> &mpo, const SweepParams &p,
                            std::vector<SiteLog> *log, LearnState *learn = nullptr);

// Two-site TDVP (two_site_update_finite_tdvp_impl.h:123-531), device
// resident.  One step is one sweep: two-site forward evolution by tau/2 and
// single-site backward evolution by -tau/2 from left to right, the pair at the
// right end by tau, the same from right to left, and the first pair by tau/2.
struct TdvpParams {
  double tau = 0.01;
  int64_t Dmin = 1, Dmax = 1;
  double trunc_err = 0;
  LanczosParams lancz;
};
struct TdvpLog {
  int64_t step, site, kind;  // kind 2: two-site forward, 1: single-site backward
  double trunc_err;
  int64_t D, iters;
  double ee, lancz_sec, tot_sec;
};
// The MPS is brought to right-canonical form (centre at site 0) first;
// tensors are complex (real ones are promoted) and replaced in place.
void two_site_finite_tdvp(Ctx &ctx, std::vector<TensorPtr> &mps,
                          const std::vector<const BTensor *> &mpo, const TdvpParams &p,
                          int64_t steps, std::vector<TdvpLog> *log);

}  // namespace udmrg
