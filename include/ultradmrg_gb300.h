/*
 * C ABI of the GB300-native two-site DMRG/TDVP local update.
 *
 * Every entry point returns 0 on success or a nonzero status code; the
 * message of the last failure on the calling thread is udmrg_last_error().
 * Tensors live on the device of their context; host data crosses the
 * boundary only through udmrg_tensor_upload / udmrg_tensor_download as the
 * packed block data (blocks in lexicographic order of their sector-id
 * tuples, each block row-major; complex data interleaved re, im).
 *
 * The block-sparse model is the QLTensor model of QuantumLiquids/TensorToolkit
 * used by qlmps: an index is a list of quantum-number sectors (qn, dim) plus a
 * direction (OUT = +1, IN = -1); a block exists only if
 * sum_i dir_i * qn_i == divergence.
 */
#ifndef ULTRADMRG_GB300_H
#define ULTRADMRG_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct udmrg_ctx udmrg_ctx;
typedef struct udmrg_tensor udmrg_tensor;
typedef struct udmrg_matvec_plan udmrg_matvec_plan;

enum { UDMRG_F64 = 0, UDMRG_C128 = 1 };
enum { UDMRG_SVD_FULL = 0, UDMRG_SVD_SPLIT_LEFT = 1, UDMRG_SVD_SPLIT_RIGHT = 2 };

enum { UDMRG_PREC_FP64 = 0, UDMRG_PREC_MIXED = 1 };

/* LanczosParams (include/qlmps/algorithm/lanczos_params.h:27-46), plus the
 * matvec precision: UDMRG_PREC_FP64 (plain FP64 block GEMMs) or
 * UDMRG_PREC_MIXED (split-BF16 tcgen05 GEMMs with FP32 accumulation; Krylov
 * vectors, dot products and the tridiagonal problem stay FP64). */
typedef struct {
  double error;           /* absolute energy change that stops the iteration */
  int64_t max_iterations; /* maximal Krylov dimension, at least 2 */
  int64_t matvec_precision;
} udmrg_lanczos_params;

/* LanczosRes (include/qlmps/algorithm/vmps/lanczos_vmps_solver_impl.h:98-103).
 * gs_vec is a new tensor owned by the caller. */
typedef struct {
  int64_t iters;
  double gs_eng;
  udmrg_tensor *gs_vec;
  double matvec_seconds; /* device time of the matvecs (CUDA events) */
  int64_t matvecs;
  /* mixed precision: the mixed-precision solve is followed by a refinement
   * run from its Ritz vector whose first step is one FP64 matvec (an exact
   * first row of the tridiagonal matrix); gs_eng and gs_vec are that run's
   * Ritz value and vector, ritz_eng the Ritz value before it, and iters
   * counts the steps of both runs.  FP64: ritz_eng = 0, fp64_matvecs = 0. */
  double ritz_eng;
  int64_t fp64_matvecs;
} udmrg_lanczos_res;

/* FiniteVMPSSweepParams without the noise and path fields
 * (include/qlmps/algorithm/finite_vmps_sweep_params.h:31-107). */
enum { UDMRG_SVD_EXACT = 0, UDMRG_SVD_SKETCH_PREV = 1, UDMRG_SVD_SKETCH_LEARNED = 2 };

typedef struct {
  int64_t sweeps;
  int64_t Dmin;
  int64_t Dmax;
  double trunc_err;
  udmrg_lanczos_params lancz_params;
  /* truncated SVD of the local update: UDMRG_SVD_EXACT, or the sector-wise
   * randomized SVD with sketch sizes from the bond's current sector
   * dimensions (SKETCH_PREV) or from the learned rank predictor
   * (SKETCH_LEARNED, see udmrg_rank_model_*); svd_oversample extra columns */
  int64_t svd_mode;
  int64_t svd_oversample;
  /* nonzero: the exact block SVD also runs on every randomized SVD's input
   * and judges it (svd_audit_* of the site log; its time is not counted) */
  int64_t svd_audit;
  /* cost rule: when a randomized SVD's total sketch exceeds this fraction of
   * the total sector dimension, the exact SVD runs instead (<= 0 or >= 1: off) */
  double svd_sketch_max_fraction;
} udmrg_sweep_params;

/* One line of the per-site log printed by TwoSiteFiniteVMPSUpdate
 * (two_site_update_finite_vmps_impl.h:362-371). */
typedef struct {
  int64_t site;
  double e0, trunc_err;
  int64_t D, iters;
  double ee, lancz_sec, svd_sec, env_sec, tot_sec, matvec_flops;
  int64_t svd_sketch_total; /* randomized SVD: sum of sketch sizes (0: exact) */
  int64_t svd_grow_rounds;  /* randomized SVD: enlargements after a miss */
  /* audit (svd_audit): |truncation error - exact SVD's| (-1: not audited)
   * and the number of kept states that differ from the exact SVD's */
  double svd_audit_err;
  int64_t svd_audit_kept_diff;
  double plan_sec; /* host seconds building the matvec plan (part of lancz_sec) */
} udmrg_site_log;

const char *udmrg_last_error(void);

/* ---- context -------------------------------------------------------- */
int udmrg_ctx_create(int device, udmrg_ctx **out);
int udmrg_ctx_destroy(udmrg_ctx *ctx);
int udmrg_ctx_sync(udmrg_ctx *ctx);
/* Number of device kernels this library launched through ctx so far. */
int udmrg_ctx_launches(udmrg_ctx *ctx, uint64_t *out);
/* Krylov steps (Lanczos ground state, Lanczos exponential) as CUDA graphs:
 * enable != 0 (the default) captures each solve's step launch sequence once
 * and replays it per step; 0 launches the kernels directly.  Both run the
 * same kernels on the same data (identical results).  Replaces nothing in
 * qlmps: the reference loop calls the matvec function pointer per step
 * (lanczos_vmps_solver_impl.h:148, 213). */
int udmrg_ctx_set_krylov_graph(udmrg_ctx *ctx, int enable);
/* The mixed-precision Lanczos ends with a refinement run whose first step is
 * one FP64-accurate matvec (the anchor).  dw != 0 (the default): its two
 * block-GEMM stages, and the mixed-precision sweep's environment updates, in
 * double-word FP32 arithmetic (each FP64 operand split into two floats, 48
 * significant bits, error-free products and sums; about 2^-48 relative per
 * product, on this GPU's FP32 pipe instead of its narrow FP64 pipe) for real
 * data; 0: on the FP64 pipe.  Complex data always uses the FP64 pipe.  The
 * plain FP64 form is not affected.  Replaces nothing in qlmps (its matvec
 * is FP64 throughout). */
int udmrg_ctx_set_anchor_dw(udmrg_ctx *ctx, int dw);
/* Host buffers of udmrg_matvec_plan_apply_host that are page-locked and
 * mapped into the device's address space (cudaMallocHost, cudaHostAlloc,
 * cudaHostRegister with mapping) are used in place by a mixed-precision
 * plan: mode 0 never (one copy each way through device buffers), 1 the input
 * (read by the psi pack over the host link), 2 input and output (the result
 * written by the last GEMM's epilogue).  Pageable memory is always copied.
 * No counterpart in the reference (its matvec takes host tensors). */
int udmrg_ctx_set_host_mapped(udmrg_ctx *ctx, int mode);
int udmrg_ctx_host_mapped(const udmrg_ctx *ctx, int *mode);
/* Mixed matvec: rows of the B tiles of the two tcgen05 GEMMs (L.psi: bn1,
 * .R: bn3), 64 or 128, or 0 for the tile autotuner (the default): the first
 * plan of a shape class is built with both tiles, matvecs of the two alternate
 * over four trials timed stage by stage (best of four), each GEMM keeps its
 * faster tile and later plans of the class
 * reuse the choice.  udmrg_ctx_tc_tuning reports the trials run and the shape
 * classes decided.  No counterpart in the reference (tile tuning of the GB300
 * kernels). */
int udmrg_ctx_set_tc_tiles(udmrg_ctx *ctx, int bn1, int bn3);
int udmrg_ctx_tc_tuning(udmrg_ctx *ctx, int64_t *trials, int64_t *classes);
/* Tile policy of the grouped FP64 (and double-word) block GEMMs of a
 * two-site matvec plan's FP64-accurate product: 0 least padded work per
 * output block, 1 fewer 32 x 32 tiles (taken only where larger tiles would
 * pad more than twice as much), or -1 (the default) for the autotuner: the
 * first plan of a shape class times one product under each policy and later
 * plans of the class reuse the faster.  Results do not depend on the policy
 * (the same summation order).  udmrg_ctx_gemm_tuning reports the trials run
 * and the classes decided.  No counterpart in the reference. */
int udmrg_ctx_set_gemm_tiles(udmrg_ctx *ctx, int policy);
int udmrg_ctx_gemm_tuning(udmrg_ctx *ctx, int64_t *trials, int64_t *classes);
/* Profiler range: waits for ctx's stream, then starts (start != 0) or stops
 * the CUDA profiler's collection (cudaProfilerStart / cudaProfilerStop), so
 * a profiler run with collection off at start records only the bracketed
 * work.  No counterpart in the reference (measurement). */
int udmrg_ctx_profiler_range(udmrg_ctx *ctx, int start);

/* ---- tensors (QLTensor storage model) -------------------------------- */
/* nsec[rank]: sectors per index; qns[sum(nsec)*nq]; dims[sum(nsec)];
 * dirs[rank] (+1 OUT / -1 IN); keys[nblocks*rank] sector ids of the blocks
 * (any order; stored sorted).  Data is uninitialised until uploaded. */
int udmrg_tensor_create(udmrg_ctx *ctx, int dtype, int nq, int rank, const int32_t *nsec,
                        const int32_t *qns, const int64_t *dims, const int32_t *dirs,
                        int64_t nblocks, const int32_t *keys, udmrg_tensor **out);
int udmrg_tensor_destroy(udmrg_tensor *t);
int udmrg_tensor_info(const udmrg_tensor *t, int *dtype, int *nq, int *rank, int64_t *nblocks,
                      int64_t *size);
/* Index of one axis.  Call with qns == dims == NULL to read *nsec first. */
int udmrg_tensor_index(const udmrg_tensor *t, int axis, int32_t *nsec, int32_t *qns,
                       int64_t *dims, int32_t *dir);
int udmrg_tensor_keys(const udmrg_tensor *t, int32_t *keys);
int udmrg_tensor_upload(udmrg_tensor *t, const double *host);
int udmrg_tensor_download(const udmrg_tensor *t, double *host);
/* Device address of the packed data (for device-resident callers). */
int udmrg_tensor_device_ptr(const udmrg_tensor *t, double **dptr);
/* 2-norm of the data, and in-place scaling by a real factor
 * (the Normalize()/QuasiNormalize() building blocks of qlten). */
int udmrg_tensor_norm(udmrg_ctx *ctx, const udmrg_tensor *t, double *norm);
int udmrg_tensor_scale(udmrg_ctx *ctx, udmrg_tensor *t, double alpha);

/* ---- block-sparse operations ---------------------------------------- */
/* Contract(A, B, {axes_a, axes_b}, C): output = A's free axes then B's. */
int udmrg_contract(udmrg_ctx *ctx, const udmrg_tensor *a, const udmrg_tensor *b, int n,
                   const int32_t *axes_a, const int32_t *axes_b, udmrg_tensor **out);
/* Contract<T, Q, a_tail, b_head>(A, B, a_start, b_start, n, C): cyclic axes. */
int udmrg_contract_cyclic(udmrg_ctx *ctx, const udmrg_tensor *a, const udmrg_tensor *b,
                          int a_start, int b_start, int n, udmrg_tensor **out);
int udmrg_dag(udmrg_ctx *ctx, const udmrg_tensor *a, udmrg_tensor **out);

/* ---- the hot path ---------------------------------------------------- */
/* eff_ham_mul_two_site_state (lanczos_vmps_solver_impl.h:260-289):
 * eff_ham = {L, W_l, W_r, R}; returns a new tensor H_eff * state. */
int udmrg_eff_ham_mul_two_site_state(udmrg_ctx *ctx, udmrg_tensor *const *eff_ham,
                                     const udmrg_tensor *state, udmrg_tensor **out);
/* eff_ham_mul_single_site_state (lanczos_vmps_solver_impl.h:291-304):
 * eff_ham = {L, W, R}; returns a new tensor H_eff * state (rank-3 state). */
int udmrg_eff_ham_mul_single_site_state(udmrg_ctx *ctx, udmrg_tensor *const *eff_ham,
                                        const udmrg_tensor *state, udmrg_tensor **out);
/* LanczosSolver with eff_ham_mul_two_site_state
 * (lanczos_vmps_solver_impl.h:114-248). init_state is not modified. */
int udmrg_lanczos_solver(udmrg_ctx *ctx, udmrg_tensor *const *eff_ham,
                         const udmrg_tensor *init_state, const udmrg_lanczos_params *params,
                         udmrg_lanczos_res *res);
/* LanczosExpmvSolver (algorithm/tdvp/lanczos_expmv_solver_impl.h:70-184):
 * exp(-i step H_eff) state for complex tensors; iters returned.  A rank-4
 * state uses eff_ham_mul_two_site_state (eff_ham = {L, W_l, W_r, R}), a
 * rank-3 state eff_ham_mul_single_site_state (eff_ham = {L, W, R}). */
int udmrg_lanczos_expmv_solver(udmrg_ctx *ctx, udmrg_tensor *const *eff_ham,
                               const udmrg_tensor *init_state, double step,
                               const udmrg_lanczos_params *params, int64_t *iters,
                               udmrg_tensor **out);
/* UpdateSiteLenvs / UpdateSiteRenvs (algorithm/vmps/vmps_init.h:343-373). */
int udmrg_update_site_lenvs(udmrg_ctx *ctx, const udmrg_tensor *lenv, const udmrg_tensor *mps_ten,
                            const udmrg_tensor *mpo_ten, udmrg_tensor **out);
int udmrg_update_site_renvs(udmrg_ctx *ctx, const udmrg_tensor *renv, const udmrg_tensor *mps_ten,
                            const udmrg_tensor *mpo_ten, udmrg_tensor **out);
/* SVD(T, ldims, ldiv, trunc_err, Dmin, Dmax, &u, &s, &vt, &err, &D)
 * (call site two_site_update_finite_vmps_impl.h:302-307).  mode selects the
 * plain factors (FULL) or the fused MPS splits of :320-334 (SPLIT_LEFT:
 * vt := s*vt; SPLIT_RIGHT: u := u*s). ldiv has nq entries. */
int udmrg_svd(udmrg_ctx *ctx, const udmrg_tensor *t, int ldims, const int32_t *ldiv,
              double trunc_err, int64_t Dmin, int64_t Dmax, int mode, udmrg_tensor **u,
              udmrg_tensor **s, udmrg_tensor **vt, double *actual_trunc_err, int64_t *D);
/* Sector-wise randomized truncated SVD (same outputs as udmrg_svd).
 * sketch_qns[nsk*nq] / sketch_sizes[nsk]: requested sketch size per bond QN
 * (sectors not listed use their full rank, i.e. are exact); a sector whose
 * sketch is entirely kept grows x2 and is redone (grow_rounds counts these
 * passes).  No counterpart in the reference (its SVD is exact). */
int udmrg_svd_randomized(udmrg_ctx *ctx, const udmrg_tensor *t, int ldims, const int32_t *ldiv,
                         double trunc_err, int64_t Dmin, int64_t Dmax, int mode, int64_t nsk,
                         const int32_t *sketch_qns, const int64_t *sketch_sizes,
                         int64_t oversample, int power_iters, uint64_t seed, udmrg_tensor **u,
                         udmrg_tensor **s, udmrg_tensor **vt, double *actual_trunc_err,
                         int64_t *D, int64_t *grow_rounds);
/* TwoSiteFiniteVMPSUpdate (two_site_update_finite_vmps_impl.h:232-373) on one
 * bond: lenv = left environment of sites [0, l), renv = right environment of
 * sites (l+1, N), the two MPS tensors and MPO tensors of sites l, l+1.  dir is
 * 'r' or 'l'.  Returns the new MPS tensors (isometry on the side of dir's
 * origin) and the environment grown by one site (left env of [0, l] for 'r',
 * right env of [l+1, N) for 'l').  log may be NULL. */
int udmrg_two_site_update(udmrg_ctx *ctx, const udmrg_tensor *lenv, const udmrg_tensor *renv,
                          const udmrg_tensor *mps_l, const udmrg_tensor *mps_r,
                          const udmrg_tensor *mpo_l, const udmrg_tensor *mpo_r,
                          const udmrg_sweep_params *params, char dir, udmrg_tensor **new_l,
                          udmrg_tensor **new_r, udmrg_tensor **new_env, udmrg_site_log *log);
/* TwoSiteFiniteVMPS (two_site_update_finite_vmps_impl.h:95-494), device
 * resident.  mps[N] is read and replaced by the updated tensors (the old
 * handles are destroyed); mpo[N] is borrowed.  log may be NULL. */
int udmrg_two_site_finite_vmps(udmrg_ctx *ctx, int64_t N, udmrg_tensor **mps,
                               udmrg_tensor *const *mpo, const udmrg_sweep_params *params,
                               double *e0, udmrg_site_log *log, int64_t log_cap,
                               int64_t *log_len);

/* ---- FiniteDMRG over a matrix-representation MPO ------------------------ */
/* One site of MatReprMPO (one_dim_tn/mpo/mat_repr_mpo.h:21, a SparMat of
 * one-site operators): rows x cols, nnz non-null elements at (x[n], y[n])
 * holding the operator tensors {pb_in, pb_out} ops[n]. */
typedef struct {
  int64_t rows, cols, nnz;
  const int64_t *x, *y;
  udmrg_tensor *const *ops;
} udmrg_mat_repr_site;
/* FiniteDMRG(mps, mat_repr_mpo, sweep_params) (algorithm/dmrg/dmrg_impl.h:504-511):
 * the super-block matvec sum_j sum_k (W_r(j,k) x R_k)[sum_i (L_i x W_l(i,j)) psi]
 * is the two-site matvec with the MPO bond split into channels, so the matrix
 * representation becomes MPO tensors (channels of equal quantum number in one
 * bond sector) and the two-site sweep runs on them; returns the last energy. */
int udmrg_finite_dmrg(udmrg_ctx *ctx, int64_t N, udmrg_tensor **mps,
                      const udmrg_mat_repr_site *mro, const udmrg_sweep_params *params,
                      double *e0, udmrg_site_log *log, int64_t log_cap, int64_t *log_len);

/* ---- two-site TDVP ----------------------------------------------------- */
/* TDVPEvolveParams (algorithm/tdvp/tdvp_evolve_params.h:20-85), the part the
 * time evolution itself uses: time step tau, number of steps (sweeps), bond
 * dimension bounds, truncation error and Krylov parameters.  The operator
 * insertion and the measurements of TwoSiteFiniteTDVP are the caller's.
 * lancz_params.matvec_precision selects the two-site Krylov matvec (mixed:
 * the split-BF16 form through its real embedding of the complex data; the
 * MPO's coefficients must be real); the single-site backward steps are FP64. */
typedef struct {
  double tau;
  int64_t steps;
  int64_t Dmin, Dmax;
  double trunc_err;
  udmrg_lanczos_params lancz_params;
} udmrg_tdvp_params;
typedef struct {
  int64_t step, site, kind; /* kind 2: two-site forward, 1: single-site backward */
  double trunc_err;
  int64_t D, iters;
  double ee, lancz_sec, tot_sec;
} udmrg_tdvp_log;
/* TwoSiteFiniteTDVP time stepping (two_site_update_finite_tdvp_impl.h:123-531):
 * brings the MPS to right-canonical form (centre at site 0), then `steps`
 * TwoSiteFiniteTDVPSweep sweeps; tensors become complex and are replaced in
 * place. */
int udmrg_two_site_finite_tdvp(udmrg_ctx *ctx, int64_t N, udmrg_tensor **mps,
                               udmrg_tensor *const *mpo, const udmrg_tdvp_params *params,
                               udmrg_tdvp_log *log, int64_t log_cap, int64_t *log_len);

/* ---- learned rank predictor (no counterpart in the reference) --------------- */
/* Two-layer MLP (n_in = 70 features -> 128 ReLU -> 1) predicting, for one
 * bond sector, y = log2(1 + kept states) from the sector's spectrum at the
 * previous visit of its bond.  Features per sample: log10 of the leading 64
 * singular values (floor 1e-20) / 10, the two QN components relative to the
 * bond's dominant sector / 4, log10(trunc_err) / 10, log2(1 + previous
 * kept) / 10, log10 of the bond's smallest kept singular value at the
 * previous visit / 10, log2(Dmax / previous bond dimension).  FP32; trained
 * and evaluated on the device.  The handle also holds the bond history
 * (spectra and kept counts per bond) of the chain it last swept, kept across
 * sweep calls until udmrg_rank_model_forget. */
typedef struct udmrg_rank_model udmrg_rank_model;
int udmrg_rank_model_sizes(int *n_in, int *n_hidden, int *n_params);
int udmrg_rank_model_create(udmrg_ctx *ctx, uint64_t seed, udmrg_rank_model **out);
int udmrg_rank_model_destroy(udmrg_rank_model *m);
int udmrg_rank_model_forget(udmrg_rank_model *m);
/* dst takes a copy of src's bond history (to run several sweeps from one state). */
int udmrg_rank_model_copy_history(udmrg_rank_model *dst, const udmrg_rank_model *src);
/* Parameters: W1 (hidden x in, row-major) | b1 | w2 | b2, n_params floats. */
int udmrg_rank_model_get_params(udmrg_rank_model *m, float *params);
int udmrg_rank_model_set_params(udmrg_rank_model *m, const float *params);
int udmrg_rank_model_predict(udmrg_rank_model *m, int64_t n, const float *x, float *y);
/* Mean squared error over n samples and its gradient (grad may be NULL). */
int udmrg_rank_model_loss_grad(udmrg_rank_model *m, int64_t n, const float *x, const float *t,
                               float *loss, float *grad);
/* Adam on shuffled minibatches; returns the loss over all samples after training. */
int udmrg_rank_model_train(udmrg_rank_model *m, int64_t n, const float *x, const float *t,
                           int epochs, int batch, float lr, uint64_t seed, float *final_loss);
/* TwoSiteFiniteVMPS with learned truncation: like udmrg_two_site_finite_vmps;
 * with params->svd_mode == UDMRG_SVD_SKETCH_LEARNED the model sizes the
 * randomized SVD's sketches of every bond it has seen before (exact SVD on a
 * bond's first visit; a sector whose whole sketch is kept is a miss and is
 * regrown, up to its full dimension, until the kept set is exact);
 * with record != 0 the training samples of every update (features of each
 * bond sector at its previous visit, label log2(1 + kept now)) are written to
 * samples_x (cap x n_in) and samples_y (cap), their total number to
 * *nsamples.  model may be NULL only without learning (plain sweep). */
int udmrg_two_site_finite_vmps_learned(udmrg_ctx *ctx, int64_t N, udmrg_tensor **mps,
                                       udmrg_tensor *const *mpo, const udmrg_sweep_params *params,
                                       udmrg_rank_model *model, int record, float *samples_x,
                                       float *samples_y, int64_t cap, int64_t *nsamples,
                                       double *e0, udmrg_site_log *log, int64_t log_cap,
                                       int64_t *log_len);

/* Noise fields of FiniteVMPSSweepParams
 * (include/qlmps/algorithm/finite_vmps_sweep_params.h:31-107): the starting
 * noise of each sweep (n_noises values, the last one repeats) and the
 * adaptation factors. */
typedef struct {
  const double *noises;
  int64_t n_noises;
  double noise_decrease, noise_increase, max_noise, alpha;
} udmrg_noise_params;

/* TwoSiteFiniteVMPSWithNoise
 * (include/qlmps/algorithm/vmps/two_site_update_noise_finite_vmps_impl.h:81-556):
 * edge tensors whose bond holds the whole block space become index
 * combiners and the sweeps run between the first sites where Dmax binds
 * (CheckAndUpdateBoundaryMPSTensors, vmps_init.h:135-246); before each update
 * the noise adapts from the energy expectation of the current two-site
 * state; after Lanczos the bond is expanded by noise * (L psi W1 W2) (moving
 * right) or noise * (psi R W2 W1) (moving left) unless its quantum numbers
 * are already covered; exact truncated SVD.  The MPS centre must be at site 0
 * on entry; mps tensors are replaced.  noise_log (log_cap entries, may be
 * NULL) receives the noise applied at each update, 0 where the bond was not
 * expanded.  With n_noises = 0: the plain sweep.  Sector order of fused and
 * expanded indexes: see INTEGRATION.md. */
int udmrg_two_site_finite_vmps_noise(udmrg_ctx *ctx, int64_t N, udmrg_tensor **mps,
                                     udmrg_tensor *const *mpo, const udmrg_sweep_params *params,
                                     const udmrg_noise_params *noise, double *e0,
                                     udmrg_site_log *log, int64_t log_cap, int64_t *log_len,
                                     double *noise_log);

/* ---- reusable matvec plan (repeated H_eff * psi on device buffers) -------- */
/* The plan fixes {L, W_l, W_r, R} and the block structure closed under the
 * matvec that contains psi_struct's blocks (the Krylov structure). */
int udmrg_matvec_plan_create(udmrg_ctx *ctx, udmrg_tensor *const *eff_ham,
                             const udmrg_tensor *psi_struct, udmrg_matvec_plan **out);
/* Same with a matvec precision (UDMRG_PREC_FP64 / UDMRG_PREC_MIXED). */
int udmrg_matvec_plan_create_ex(udmrg_ctx *ctx, udmrg_tensor *const *eff_ham,
                                const udmrg_tensor *psi_struct, int precision,
                                udmrg_matvec_plan **out);
int udmrg_matvec_plan_info(const udmrg_matvec_plan *p, double *flops, int64_t *psi_size,
                           int64_t *workspace_bytes);
/* Tensor with the plan's Krylov structure holding `src` (zero elsewhere). */
int udmrg_matvec_plan_embed(udmrg_matvec_plan *p, const udmrg_tensor *src, udmrg_tensor **out);
/* out = H_eff * in on device buffers laid out in the Krylov structure. */
int udmrg_matvec_plan_apply(udmrg_matvec_plan *p, const double *d_in, double *d_out);
/* out = H_eff * in with host buffers of psi_size elements each (packed
 * Krylov-structure layout): one call copies in, applies and copies out on
 * the context's stream, then waits (pinned host memory gives full copy
 * bandwidth; with udmrg_ctx_set_host_mapped a mixed plan uses mapped pinned
 * buffers in place instead).  The plan keeps two device buffers for the
 * copies.  The host-facing form of eff_ham_mul_two_site_state
 * (lanczos_vmps_solver_impl.h:250-289). */
int udmrg_matvec_plan_apply_host(udmrg_matvec_plan *p, const double *h_in, double *h_out);
/* The same product in the mixed solver's anchor form (FP64 pipe or
 * double-word FP32, per udmrg_ctx_set_anchor_dw), whatever the plan's
 * precision. */
int udmrg_matvec_plan_apply_anchor(udmrg_matvec_plan *p, const double *d_in, double *d_out);
int udmrg_matvec_plan_destroy(udmrg_matvec_plan *p);
/* One matvec with CUDA events between its four stages (device ms, written to
 * ms[4]) and the work of each stage in FLOP (flops[4]: algorithmic for the
 * FP64 form; tensor-core work issued, six split products included, for the
 * mixed form).  Mixed stages: psi pack, GEMM L.psi, MPO step, GEMM .R (with
 * the fused MPO step: stage 2 is empty and stage 3 times the fused kernel);
 * FP64 stages: the four block contractions. */
int udmrg_matvec_plan_stage_times(udmrg_matvec_plan *p, const double *d_in, double *d_out,
                                  double *ms, double *flops);
/* Algorithmic HBM bytes of the mixed form's stages (bytes[4], same order as
 * the stage times): psi pack (FP64 read, three BF16 planes written per
 * element); GEMM L.psi (both split-BF16 images read, FP32 T1 entries
 * written); unfused: the MPO step (FP32 T1 entries read, three BF16 planes
 * written per T3 entry) and GEMM .R (T3 and R images read, FP64 result
 * written); fused: stage 3 reads each FP32 T1 entry and the R image once and
 * writes the FP64 result.  0 for the FP64 form. */
int udmrg_matvec_plan_stage_bytes(udmrg_matvec_plan *p, double *bytes);
/* Mixed form: run the MPO step inside the producers of the .R GEMM (enable =
 * 1) or as its own kernel writing the split-BF16 T3 image (enable = 0, the
 * default, faster on the measured workloads).  Both give bit-identical
 * results.  No counterpart in the reference (a kernel check used by the
 * tests). */
int udmrg_matvec_plan_set_fused(udmrg_matvec_plan *p, int enable);
/* Mixed form: the B-tile rows of its two GEMMs and whether the autotuner
 * chose them (*tuned = 1).  No counterpart in the reference. */
int udmrg_matvec_plan_tiles(const udmrg_matvec_plan *p, int *bn1, int *bn3, int *tuned);
/* The tile policy of the plan's FP64-accurate grouped GEMMs (0 or 1, see
 * udmrg_ctx_set_gemm_tiles).  No counterpart in the reference. */
int udmrg_matvec_plan_gemm_policy(const udmrg_matvec_plan *p, int *policy);
/* Host seconds spent building the plan, by phase: sec[0] the Krylov block
 * structure's closure, sec[1] the host tables, built on host threads (the
 * four contraction plans, the FP64 form's MPO step, the mixed form's tables
 * when its tile shapes are known), sec[2] their uploads, sec[3] the mixed
 * form's tables alone (a part of sec[1], or of sec[4]), sec[4] the mixed
 * form's device part (allocations, operand packing, uploads; the tile
 * trials of a new shape class), sec[5] FP64 workspaces and the GEMM tile
 * tuning.  Profiling aid with no qlmps counterpart (planning is implicit in
 * lanczos_vmps_solver_impl.h:114-248). */
int udmrg_matvec_plan_build_times(const udmrg_matvec_plan *p, double *sec);

/* ---- measurement ---------------------------------------------------- */
/* FP64 FMA throughput of the device (TFLOP/s), measured by a DFMA-bound
 * kernel; the roofline denominator of the plain FP64 block GEMMs. */
int udmrg_probe_fp64_tflops(udmrg_ctx *ctx, double *tflops);
/* HBM rates of the Lanczos vector kernels: one Krylov step's kernels at step
 * `step` (1 .. 509) on random vectors of n doubles, device-timed (best of
 * four): ms[0] normalisation, ms[1] alpha, ms[2] three-term update, ms[3]
 * the first re-orthogonalisation pass against v_0 .. v_step, ms[4] the
 * second, gated pass; bytes[i] the bytes each moves (0 where the gate
 * skipped the second pass, *second_pass_ran = 0).  Measurement aid, no
 * reference counterpart. */
int udmrg_probe_krylov_step(udmrg_ctx *ctx, int64_t n, int step, double *ms, double *bytes,
                            int *second_pass_ran);
/* CUDA events on the context's stream (slot in [0, 1024)), elapsed ms
 * between two recorded slots, and an L2 flush (a write of `bytes` bytes to
 * a scratch buffer, stream ordered) for cold-cache timing. */
int udmrg_ctx_event_record(udmrg_ctx *ctx, int slot);
/* Self-test of the tcgen05 split-BF16 GEMM: C = A * B for dense row-major
 * host matrices A (M x K), B (K x N), C (M x N).  No counterpart in the
 * reference (a kernel check used by the tests). */
int udmrg_selftest_tc_gemm(udmrg_ctx *ctx, int64_t M, int64_t N, int64_t K, const double *hA,
                           const double *hB, double *hC);
/* Self-test of the batched symmetric eigensolver used by the SVD: for nmat
 * row-major symmetric host matrices (sizes n[i], concatenated in mats), all
 * eigenvalues (descending, concatenated in lam) and the leading k[i]
 * eigenvectors (row-major n[i] x k[i], concatenated in vecs).  No counterpart
 * in the reference (a kernel check used by the tests). */
int udmrg_selftest_sym_eig(udmrg_ctx *ctx, int64_t nmat, const int32_t *n, const double *mats,
                           const int32_t *k, double *lam, double *vecs);
int udmrg_ctx_event_elapsed(udmrg_ctx *ctx, int slot_a, int slot_b, float *ms);
int udmrg_ctx_flush_l2(udmrg_ctx *ctx, int64_t bytes);

/* ---- allocation-free entry point ---------------------------------------- */
/* No counterpart in the reference.  2-norm of n_doubles device doubles at
 * d_x, written to the device double *d_norm, stream ordered on `stream` (a
 * cudaStream_t; NULL is the legacy default stream) on the current device.
 * For callers that cannot allocate device memory when they need it (their
 * device memory belongs to another allocator or is fully reserved, or they
 * run loops that must not touch an allocator): it calls no cudaMalloc/cudaFree
 * or allocating routine; its scratch is a fixed 32 KB device array held by
 * every GPU that loads the library until exit.  At most 16,777,216 doubles
 * per call (status 1 above that); devices 0..63.  The first call on a device
 * sets up the scratch address, so make it before any stream capture; that
 * address is cached for the life of the device's primary context (the
 * process).  A CUDA error pending from the caller's earlier launches is
 * reported (status 2) and not cleared.  Calls that overlap on the GPU race on
 * the shared scratch. */
int udmrg_norm_noalloc(const double *d_x, int64_t n_doubles, double *d_norm, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ULTRADMRG_GB300_H */
