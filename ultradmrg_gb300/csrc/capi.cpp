// extern "C" boundary: plain pointers and sizes, status codes, no exceptions.
#include <cmath>
#include <algorithm>
#include <cstring>
#include <memory>

#include <cuda_profiler_api.h>

#include "../../include/ultradmrg_gb300.h"
#include "dmrg.hpp"
#include "matrepr.hpp"
#include "svd.hpp"
#include "tc_gemm.hpp"

using namespace udmrg;

namespace udmrg {
double probe_fp64_tflops(Ctx &ctx);
}

struct udmrg_ctx {
  Ctx ctx;
  std::vector<cudaEvent_t> events;
  void *flush_buf = nullptr;
  int64_t flush_bytes = 0;
  explicit udmrg_ctx(int dev) : ctx(dev) {}
  ~udmrg_ctx() {
    for (auto e : events)
      if (e) cudaEventDestroy(e);
    if (flush_buf) ctx.free(flush_buf);
  }
};
struct udmrg_tensor {
  TensorPtr t;
};
struct udmrg_matvec_plan {
  Ctx *ctx;
  std::unique_ptr<MatvecPlan> plan;
  TensorPtr promoted[4];  // complex copies of real operators, when needed
  double *host_in = nullptr, *host_out = nullptr;  // device buffers of apply_host
  ~udmrg_matvec_plan() {
    if (host_in) ctx->free(host_in);
    if (host_out) ctx->free(host_out);
  }
};

namespace {

thread_local std::string g_err;

template <typename F>
int guarded(F &&f) {
  try {
    f();
    return kOk;
  } catch (const Error &e) {
    g_err = e.what();
    return e.code;
  } catch (const std::exception &e) {
    g_err = e.what();
    return kErrInternal;
  } catch (...) {
    g_err = "unknown error";
    return kErrInternal;
  }
}

udmrg_tensor *wrap(TensorPtr t) {
  auto *h = new udmrg_tensor;
  if (t && t->ctx) t->ctx->live_handles++;
  h->t = std::move(t);
  return h;
}

// A handle on `c` went away: delete the context if its destroy was requested
// and this was the last handle.
void release_ctx(Ctx *c) {
  if (!c) return;
  c->live_handles--;
  if (c->closing && c->live_handles <= 0) delete (udmrg_ctx *)c->owner;
}

const BTensor &T(const udmrg_tensor *h) {
  UDMRG_REQUIRE(h && h->t, "null tensor handle");
  return *h->t;
}

}  // namespace

namespace udmrg {
// Error reporting for entry points defined in other translation units.
const char *set_last_error_noalloc(const char *msg) {
  g_err = msg;
  return g_err.c_str();
}
}  // namespace udmrg

extern "C" {

const char *udmrg_last_error(void) { return g_err.c_str(); }

int udmrg_ctx_create(int device, udmrg_ctx **out) {
  return guarded([&] {
    UDMRG_REQUIRE(out, "null output");
    *out = new udmrg_ctx(device);
    (*out)->ctx.owner = *out;
  });
}

int udmrg_ctx_destroy(udmrg_ctx *c) {
  return guarded([&] {
    if (!c) return;
    // tensors and plans still alive keep the context until they are destroyed
    c->ctx.closing = true;
    if (c->ctx.live_handles <= 0) delete c;
  });
}

int udmrg_ctx_sync(udmrg_ctx *c) {
  return guarded([&] { c->ctx.sync(); });
}

int udmrg_ctx_launches(udmrg_ctx *c, uint64_t *out) {
  return guarded([&] { *out = c->ctx.launches; });
}

int udmrg_ctx_set_tc_tiles(udmrg_ctx *c, int bn1, int bn3) {
  return guarded([&] {
    auto ok = [](int b) { return b == 0 || b == 64 || b == 128; };
    UDMRG_REQUIRE(ok(bn1) && ok(bn3) && ((bn1 == 0) == (bn3 == 0)),
                  "tc tiles: 64 or 128 each, or both 0 (autotuner)");
    c->ctx.tc_bn1 = bn1;
    c->ctx.tc_bn3 = bn3;
  });
}

int udmrg_ctx_tc_tuning(udmrg_ctx *c, int64_t *trials, int64_t *classes) {
  return guarded([&] {
    if (trials) *trials = c->ctx.tc_trials;
    if (classes) *classes = (int64_t)c->ctx.tc_tuned.size();
  });
}

int udmrg_ctx_set_gemm_tiles(udmrg_ctx *c, int policy) {
  return guarded([&] {
    UDMRG_REQUIRE(c && policy >= -1 && policy <= 1, "gemm tile policy: -1, 0 or 1");
    c->ctx.gemm_policy = policy;
  });
}

int udmrg_ctx_gemm_tuning(udmrg_ctx *c, int64_t *trials, int64_t *classes) {
  return guarded([&] {
    if (trials) *trials = c->ctx.gemm_trials;
    if (classes) *classes = (int64_t)c->ctx.gemm_tuned.size();
  });
}

int udmrg_ctx_profiler_range(udmrg_ctx *c, int start) {
  return guarded([&] {
    UDMRG_REQUIRE(c, "null argument");
    c->ctx.sync();
    UDMRG_CHECK_CUDA(start ? cudaProfilerStart() : cudaProfilerStop());
  });
}

int udmrg_ctx_set_anchor_dw(udmrg_ctx *c, int dw) {
  return guarded([&] {
    UDMRG_REQUIRE(c, "null argument");
    c->ctx.anchor_dw = dw != 0;
  });
}

int udmrg_ctx_set_host_mapped(udmrg_ctx *c, int mode) {
  return guarded([&] {
    UDMRG_REQUIRE(c, "null argument");
    UDMRG_REQUIRE(mode >= 0 && mode <= 2, "host_mapped: mode 0, 1 or 2");
    c->ctx.host_mapped = mode;
  });
}

int udmrg_ctx_host_mapped(const udmrg_ctx *c, int *mode) {
  return guarded([&] {
    UDMRG_REQUIRE(c && mode, "null argument");
    *mode = c->ctx.host_mapped;
  });
}

int udmrg_ctx_set_krylov_graph(udmrg_ctx *c, int enable) {
  return guarded([&] {
    UDMRG_REQUIRE(c, "null argument");
    c->ctx.krylov_graph = enable != 0;
  });
}

int udmrg_tensor_create(udmrg_ctx *c, int dtype, int nq, int rank, const int32_t *nsec,
                        const int32_t *qns, const int64_t *dims, const int32_t *dirs,
                        int64_t nblocks, const int32_t *keys, udmrg_tensor **out) {
  return guarded([&] {
    UDMRG_REQUIRE(c && out, "null argument");
    UDMRG_REQUIRE(dtype == kF64 || dtype == kC128, "dtype must be UDMRG_F64 or UDMRG_C128");
    UDMRG_REQUIRE(nq >= 1 && nq <= kMaxQ, "nq out of range");
    UDMRG_REQUIRE(rank >= 1, "rank must be positive");
    auto t = std::make_unique<BTensor>();
    t->ctx = &c->ctx;
    t->dtype = (DType)dtype;
    t->nq = nq;
    int64_t s = 0;
    for (int i = 0; i < rank; ++i) {
      Index ix;
      ix.dir = dirs[i];
      UDMRG_REQUIRE(ix.dir == 1 || ix.dir == -1, "direction must be +1 (OUT) or -1 (IN)");
      for (int j = 0; j < nsec[i]; ++j, ++s) {
        QN q;
        for (int k = 0; k < nq; ++k) q.v[k] = qns[s * nq + k];
        ix.qns.push_back(q);
        UDMRG_REQUIRE(dims[s] > 0, "sector dimensions must be positive");
        ix.dims.push_back(dims[s]);
      }
      t->idx.push_back(std::move(ix));
    }
    std::vector<int32_t> flat(keys, keys + nblocks * rank);
    auto sorted = sort_keys(flat, rank);
    UDMRG_REQUIRE((int64_t)sorted.size() == nblocks * rank, "duplicate block keys");
    t->set_blocks(std::move(sorted));
    if (t->nblocks() > 0) {
      const QN d = t->div();
      for (int64_t b = 1; b < t->nblocks(); ++b)
        UDMRG_REQUIRE(t->block_div(t->key(b)) == d, "blocks with different divergences");
    }
    t->alloc_data();
    *out = wrap(std::move(t));
  });
}

int udmrg_tensor_destroy(udmrg_tensor *t) {
  return guarded([&] {
    if (!t) return;
    Ctx *c = t->t ? t->t->ctx : nullptr;
    delete t;
    release_ctx(c);
  });
}

int udmrg_tensor_info(const udmrg_tensor *h, int *dtype, int *nq, int *rank, int64_t *nblocks,
                      int64_t *size) {
  return guarded([&] {
    const BTensor &t = T(h);
    if (dtype) *dtype = t.dtype;
    if (nq) *nq = t.nq;
    if (rank) *rank = t.rank();
    if (nblocks) *nblocks = t.nblocks();
    if (size) *size = t.size();
  });
}

int udmrg_tensor_index(const udmrg_tensor *h, int axis, int32_t *nsec, int32_t *qns,
                       int64_t *dims, int32_t *dir) {
  return guarded([&] {
    const BTensor &t = T(h);
    UDMRG_REQUIRE(axis >= 0 && axis < t.rank(), "axis out of range");
    const Index &ix = t.idx[axis];
    if (nsec) *nsec = ix.nsec();
    if (dir) *dir = ix.dir;
    for (int j = 0; j < ix.nsec(); ++j) {
      if (qns)
        for (int k = 0; k < t.nq; ++k) qns[j * t.nq + k] = ix.qns[j].v[k];
      if (dims) dims[j] = ix.dims[j];
    }
  });
}

int udmrg_tensor_keys(const udmrg_tensor *h, int32_t *keys) {
  return guarded([&] {
    const BTensor &t = T(h);
    std::memcpy(keys, t.keys.data(), t.keys.size() * sizeof(int32_t));
  });
}

int udmrg_tensor_upload(udmrg_tensor *h, const double *host) {
  return guarded([&] {
    BTensor &t = *h->t;
    if (t.size())
      UDMRG_CHECK_CUDA(
          cudaMemcpyAsync(t.data, host, t.bytes(), cudaMemcpyHostToDevice, t.ctx->stream));
    t.ctx->sync();
  });
}

int udmrg_tensor_download(const udmrg_tensor *h, double *host) {
  return guarded([&] {
    const BTensor &t = T(h);
    if (t.size())
      UDMRG_CHECK_CUDA(
          cudaMemcpyAsync(host, t.data, t.bytes(), cudaMemcpyDeviceToHost, t.ctx->stream));
    t.ctx->sync();
  });
}

int udmrg_tensor_device_ptr(const udmrg_tensor *h, double **dptr) {
  return guarded([&] { *dptr = T(h).data; });
}

int udmrg_tensor_norm(udmrg_ctx *c, const udmrg_tensor *h, double *norm) {
  return guarded([&] {
    const BTensor &t = T(h);
    VecWork w(c->ctx);
    *norm = std::sqrt(norm2(w, t.data, t.size() * elem_doubles(t.dtype)));
  });
}

int udmrg_tensor_scale(udmrg_ctx *c, udmrg_tensor *h, double alpha) {
  return guarded([&] {
    BTensor &t = *h->t;
    scale(c->ctx, t.data, t.size() * elem_doubles(t.dtype), alpha);
    c->ctx.sync();
  });
}

int udmrg_contract(udmrg_ctx *c, const udmrg_tensor *a, const udmrg_tensor *b, int n,
                   const int32_t *axes_a, const int32_t *axes_b, udmrg_tensor **out) {
  return guarded([&] {
    std::vector<int> ca(axes_a, axes_a + n), cb(axes_b, axes_b + n);
    *out = wrap(contract_axes(c->ctx, T(a), T(b), ca, cb));
  });
}

int udmrg_contract_cyclic(udmrg_ctx *c, const udmrg_tensor *a, const udmrg_tensor *b,
                          int a_start, int b_start, int n, udmrg_tensor **out) {
  return guarded([&] { *out = wrap(contract_cyclic(c->ctx, T(a), T(b), a_start, b_start, n)); });
}

int udmrg_dag(udmrg_ctx *c, const udmrg_tensor *a, udmrg_tensor **out) {
  return guarded([&] { *out = wrap(dag(c->ctx, T(a))); });
}

namespace {

// Operators with the element type of the state (real ones promoted).
struct EffHam {
  const BTensor *op[4];
  TensorPtr keep[4];
};

void prepare_eff_ham(Ctx &ctx, udmrg_tensor *const *eff_ham, DType dt, EffHam &e, int nops = 4) {
  for (int i = 0; i < nops; ++i) {
    const BTensor &t = T(eff_ham[i]);
    if (t.dtype == dt) {
      e.op[i] = &t;
    } else {
      UDMRG_REQUIRE(dt == kC128, "real state with complex operators is not supported");
      e.keep[i] = to_complex(ctx, t);
      e.op[i] = e.keep[i].get();
    }
  }
}

}  // namespace

int udmrg_eff_ham_mul_two_site_state(udmrg_ctx *c, udmrg_tensor *const *eff_ham,
                                     const udmrg_tensor *state, udmrg_tensor **out) {
  return guarded([&] {
    Ctx &ctx = c->ctx;
    const BTensor &psi = T(state);
    EffHam e;
    prepare_eff_ham(ctx, eff_ham, psi.dtype, e);
    auto mv = plan_matvec2(ctx, *e.op[0], *e.op[1], *e.op[2], *e.op[3], psi);
    auto in = embed(ctx, psi, *mv->sstruct);
    auto res = mv->sstruct->clone_struct();
    res->alloc_data();
    mv->apply(in->data, res->data);
    ctx.sync();
    *out = wrap(std::move(res));
  });
}

int udmrg_eff_ham_mul_single_site_state(udmrg_ctx *c, udmrg_tensor *const *eff_ham,
                                        const udmrg_tensor *state, udmrg_tensor **out) {
  return guarded([&] {
    Ctx &ctx = c->ctx;
    const BTensor &psi = T(state);
    EffHam e;
    prepare_eff_ham(ctx, eff_ham, psi.dtype, e, 3);
    auto mv = plan_matvec1(ctx, *e.op[0], *e.op[1], *e.op[2], psi);
    auto in = embed(ctx, psi, *mv->sstruct);
    auto res = mv->sstruct->clone_struct();
    res->alloc_data();
    mv->apply(in->data, res->data);
    ctx.sync();
    *out = wrap(std::move(res));
  });
}

int udmrg_lanczos_solver(udmrg_ctx *c, udmrg_tensor *const *eff_ham,
                         const udmrg_tensor *init_state, const udmrg_lanczos_params *params,
                         udmrg_lanczos_res *res) {
  return guarded([&] {
    Ctx &ctx = c->ctx;
    const BTensor &psi = T(init_state);
    EffHam e;
    prepare_eff_ham(ctx, eff_ham, psi.dtype, e);
    LanczosParams p{params->error, params->max_iterations, (int)params->matvec_precision};
    auto mv = plan_matvec2(ctx, *e.op[0], *e.op[1], *e.op[2], *e.op[3], psi, p.precision);
    auto r = lanczos_gs(ctx, *mv, psi, p);
    res->iters = r.iters;
    res->gs_eng = r.gs_eng;
    res->matvec_seconds = r.matvec_seconds;
    res->matvecs = r.matvecs;
    res->ritz_eng = r.ritz_eng;
    res->fp64_matvecs = r.fp64_matvecs;
    res->gs_vec = wrap(std::move(r.gs_vec));
  });
}

int udmrg_lanczos_expmv_solver(udmrg_ctx *c, udmrg_tensor *const *eff_ham,
                               const udmrg_tensor *init_state, double step,
                               const udmrg_lanczos_params *params, int64_t *iters,
                               udmrg_tensor **out) {
  return guarded([&] {
    Ctx &ctx = c->ctx;
    TensorPtr promoted;
    const BTensor *psi = &T(init_state);
    if (psi->dtype != kC128) {
      promoted = to_complex(ctx, *psi);
      psi = promoted.get();
    }
    EffHam e;
    const bool one = psi->rank() == 3;  // single-site form: eff_ham = {L, W, R}
    prepare_eff_ham(ctx, eff_ham, kC128, e, one ? 3 : 4);
    UDMRG_REQUIRE(!one || params->matvec_precision == kPrecFP64,
                  "expmv: the single-site form is FP64 only");
    auto mv = one ? plan_matvec1(ctx, *e.op[0], *e.op[1], *e.op[2], *psi)
                  : plan_matvec2(ctx, *e.op[0], *e.op[1], *e.op[2], *e.op[3], *psi,
                                 (int)params->matvec_precision);
    LanczosParams p{params->error, params->max_iterations, (int)params->matvec_precision};
    auto r = lanczos_expmv(ctx, *mv, *psi, step, p);
    if (iters) *iters = r.iters;
    *out = wrap(std::move(r.expmv));
  });
}

int udmrg_update_site_lenvs(udmrg_ctx *c, const udmrg_tensor *lenv, const udmrg_tensor *mps_ten,
                            const udmrg_tensor *mpo_ten, udmrg_tensor **out) {
  return guarded([&] {
    *out = wrap(update_site_lenv(c->ctx, T(lenv), T(mps_ten), T(mpo_ten)));
  });
}

int udmrg_update_site_renvs(udmrg_ctx *c, const udmrg_tensor *renv, const udmrg_tensor *mps_ten,
                            const udmrg_tensor *mpo_ten, udmrg_tensor **out) {
  return guarded([&] {
    *out = wrap(update_site_renv(c->ctx, T(renv), T(mps_ten), T(mpo_ten)));
  });
}

int udmrg_svd(udmrg_ctx *c, const udmrg_tensor *t, int ldims, const int32_t *ldiv,
              double trunc_err, int64_t Dmin, int64_t Dmax, int mode, udmrg_tensor **u,
              udmrg_tensor **s, udmrg_tensor **vt, double *actual_trunc_err, int64_t *D) {
  return guarded([&] {
    const BTensor &x = T(t);
    QN q;
    for (int k = 0; k < x.nq; ++k) q.v[k] = ldiv[k];
    UDMRG_REQUIRE(mode >= 0 && mode <= 2, "bad SVD mode");
    auto r = svd_trunc(c->ctx, x, ldims, q, trunc_err, Dmin, Dmax, mode);
    *u = wrap(std::move(r.u));
    *s = wrap(std::move(r.s));
    *vt = wrap(std::move(r.vt));
    if (actual_trunc_err) *actual_trunc_err = r.trunc_err;
    if (D) *D = r.D;
  });
}

int udmrg_svd_randomized(udmrg_ctx *c, const udmrg_tensor *t, int ldims, const int32_t *ldiv,
                         double trunc_err, int64_t Dmin, int64_t Dmax, int mode, int64_t nsk,
                         const int32_t *sketch_qns, const int64_t *sketch_sizes,
                         int64_t oversample, int power_iters, uint64_t seed, udmrg_tensor **u,
                         udmrg_tensor **s, udmrg_tensor **vt, double *actual_trunc_err,
                         int64_t *D, int64_t *grow_rounds) {
  return guarded([&] {
    const BTensor &x = T(t);
    QN q;
    for (int k = 0; k < x.nq; ++k) q.v[k] = ldiv[k];
    UDMRG_REQUIRE(mode >= 0 && mode <= 2, "bad SVD mode");
    SketchParams sp;
    sp.oversample = oversample;
    sp.power_iters = power_iters;
    sp.seed = seed;
    for (int64_t i = 0; i < nsk; ++i) {
      QN qi;
      for (int k = 0; k < x.nq; ++k) qi.v[k] = sketch_qns[i * x.nq + k];
      sp.sketch.push_back({qi, sketch_sizes[i]});
    }
    auto r = svd_trunc_sketch(c->ctx, x, ldims, q, trunc_err, Dmin, Dmax, mode, sp);
    *u = wrap(std::move(r.u));
    *s = wrap(std::move(r.s));
    *vt = wrap(std::move(r.vt));
    if (actual_trunc_err) *actual_trunc_err = r.trunc_err;
    if (D) *D = r.D;
    if (grow_rounds) *grow_rounds = r.grow_rounds;
  });
}

static udmrg_site_log site_log(const SiteLog &s) {
  return {s.site,    s.e0,      s.trunc_err, s.D,           s.iters,
          s.ee,      s.lancz_sec, s.svd_sec, s.env_sec,     s.tot_sec,
          s.matvec_flops, s.svd_sketch_total, s.svd_grow_rounds, s.svd_audit_err,
          s.svd_audit_kept_diff, s.plan_sec};
}

int udmrg_two_site_update(udmrg_ctx *c, const udmrg_tensor *lenv, const udmrg_tensor *renv,
                          const udmrg_tensor *mps_l, const udmrg_tensor *mps_r,
                          const udmrg_tensor *mpo_l, const udmrg_tensor *mpo_r,
                          const udmrg_sweep_params *params, char dir, udmrg_tensor **new_l,
                          udmrg_tensor **new_r, udmrg_tensor **new_env, udmrg_site_log *log) {
  return guarded([&] {
    SweepParams p;
    p.sweeps = 1;
    p.Dmin = params->Dmin;
    p.Dmax = params->Dmax;
    p.trunc_err = params->trunc_err;
    p.lancz = {params->lancz_params.error, params->lancz_params.max_iterations,
               (int)params->lancz_params.matvec_precision};
    p.svd_mode = (int)params->svd_mode;
    p.svd_oversample = params->svd_oversample;
    p.svd_audit = params->svd_audit != 0;
    p.svd_sketch_max_fraction = params->svd_sketch_max_fraction > 0.0 &&
                                        params->svd_sketch_max_fraction < 1.0
                                    ? params->svd_sketch_max_fraction
                                    : 1.0;
    SiteLog s{};
    auto r = two_site_update_local(c->ctx, T(lenv), T(renv), T(mps_l), T(mps_r), T(mpo_l),
                                   T(mpo_r), p, dir, &s);
    *new_l = wrap(std::move(r.mps_l));
    *new_r = wrap(std::move(r.mps_r));
    *new_env = wrap(std::move(r.env));
    if (log)
      *log = site_log(s);
  });
}

int udmrg_two_site_finite_vmps(udmrg_ctx *c, int64_t N, udmrg_tensor **mps,
                               udmrg_tensor *const *mpo, const udmrg_sweep_params *params,
                               double *e0, udmrg_site_log *log, int64_t log_cap,
                               int64_t *log_len) {
  return udmrg_two_site_finite_vmps_learned(c, N, mps, mpo, params, nullptr, 0, nullptr, nullptr,
                                            0, nullptr, e0, log, log_cap, log_len);
}

struct udmrg_rank_model {
  Ctx *ctx;
  std::unique_ptr<RankModel> m;
  LearnState hist;  // bond spectra of the chain it last swept
};

int udmrg_rank_model_sizes(int *n_in, int *n_hidden, int *n_params) {
  return guarded([&] {
    if (n_in) *n_in = kRankIn;
    if (n_hidden) *n_hidden = kRankHidden;
    if (n_params) *n_params = kRankParams;
  });
}

int udmrg_rank_model_create(udmrg_ctx *c, uint64_t seed, udmrg_rank_model **out) {
  return guarded([&] {
    auto *m = new udmrg_rank_model;
    m->ctx = &c->ctx;
    m->m = std::make_unique<RankModel>(c->ctx, seed);
    c->ctx.live_handles++;
    *out = m;
  });
}

int udmrg_rank_model_forget(udmrg_rank_model *m) {
  return guarded([&] {
    m->hist.prev.clear();
    m->hist.prev_kept.clear();
  });
}

int udmrg_rank_model_copy_history(udmrg_rank_model *dst, const udmrg_rank_model *src) {
  return guarded([&] {
    dst->hist.prev = src->hist.prev;
    dst->hist.prev_kept = src->hist.prev_kept;
  });
}

int udmrg_rank_model_destroy(udmrg_rank_model *m) {
  return guarded([&] {
    if (!m) return;
    Ctx *c = m->ctx;
    delete m;
    release_ctx(c);
  });
}

int udmrg_rank_model_get_params(udmrg_rank_model *m, float *params) {
  return guarded([&] {
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(params, m->m->params, kRankParams * sizeof(float),
                                     cudaMemcpyDeviceToHost, m->ctx->stream));
    m->ctx->sync();
  });
}

int udmrg_rank_model_set_params(udmrg_rank_model *m, const float *params) {
  return guarded([&] {
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(m->m->params, params, kRankParams * sizeof(float),
                                     cudaMemcpyHostToDevice, m->ctx->stream));
    m->ctx->sync();
  });
}

int udmrg_rank_model_predict(udmrg_rank_model *m, int64_t n, const float *x, float *y) {
  return guarded([&] {
    Ctx &ctx = *m->ctx;
    DeviceScratch s(ctx);
    float *dx = s.get<float>(n * kRankIn), *dy = s.get<float>(n);
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(dx, x, n * kRankIn * sizeof(float), cudaMemcpyHostToDevice,
                                     ctx.stream));
    m->m->predict(dx, n, dy);
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(y, dy, n * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
  });
}

int udmrg_rank_model_loss_grad(udmrg_rank_model *m, int64_t n, const float *x, const float *t,
                               float *loss, float *grad) {
  return guarded([&] {
    Ctx &ctx = *m->ctx;
    DeviceScratch s(ctx);
    float *dx = s.get<float>(n * kRankIn), *dt = s.get<float>(n);
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(dx, x, n * kRankIn * sizeof(float), cudaMemcpyHostToDevice,
                                     ctx.stream));
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(dt, t, n * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    const float l = m->m->loss_grad(dx, dt, n);
    if (loss) *loss = l;
    if (grad) {
      UDMRG_CHECK_CUDA(cudaMemcpyAsync(grad, m->m->grad, kRankParams * sizeof(float),
                                       cudaMemcpyDeviceToHost, ctx.stream));
      ctx.sync();
    }
  });
}

int udmrg_rank_model_train(udmrg_rank_model *m, int64_t n, const float *x, const float *t,
                           int epochs, int batch, float lr, uint64_t seed, float *final_loss) {
  return guarded([&] {
    UDMRG_REQUIRE(n > 0 && batch > 0 && epochs >= 0, "rank model: bad training arguments");
    Ctx &ctx = *m->ctx;
    DeviceScratch s(ctx);
    float *dx = s.get<float>(n * kRankIn), *dt = s.get<float>(n);
    float *bx = s.get<float>((int64_t)batch * kRankIn), *bt = s.get<float>(batch);
    // shuffled copies per epoch are assembled on the host (the data set is small)
    std::vector<int64_t> ord(n);
    for (int64_t i = 0; i < n; ++i) ord[i] = i;
    uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
    std::vector<float> hx((size_t)batch * kRankIn), ht(batch);
    for (int e = 0; e < epochs; ++e) {
      for (int64_t i = n - 1; i > 0; --i) {  // Fisher-Yates with an LCG
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        std::swap(ord[i], ord[(int64_t)((st >> 33) % (uint64_t)(i + 1))]);
      }
      for (int64_t b0 = 0; b0 < n; b0 += batch) {
        const int64_t nb = std::min<int64_t>(batch, n - b0);
        for (int64_t i = 0; i < nb; ++i) {
          std::memcpy(hx.data() + i * kRankIn, x + ord[b0 + i] * kRankIn, kRankIn * sizeof(float));
          ht[i] = t[ord[b0 + i]];
        }
        UDMRG_CHECK_CUDA(cudaMemcpyAsync(bx, hx.data(), nb * kRankIn * sizeof(float),
                                         cudaMemcpyHostToDevice, ctx.stream));
        UDMRG_CHECK_CUDA(cudaMemcpyAsync(bt, ht.data(), nb * sizeof(float), cudaMemcpyHostToDevice,
                                         ctx.stream));
        m->m->loss_grad(bx, bt, nb);
        m->m->adam(lr);
      }
    }
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(dx, x, n * kRankIn * sizeof(float), cudaMemcpyHostToDevice,
                                     ctx.stream));
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(dt, t, n * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    const float l = m->m->loss_grad(dx, dt, n);
    if (final_loss) *final_loss = l;
  });
}

int udmrg_two_site_finite_vmps_learned(udmrg_ctx *c, int64_t N, udmrg_tensor **mps,
                                       udmrg_tensor *const *mpo, const udmrg_sweep_params *params,
                                       udmrg_rank_model *model, int record, float *samples_x,
                                       float *samples_y, int64_t cap, int64_t *nsamples,
                                       double *e0, udmrg_site_log *log, int64_t log_cap,
                                       int64_t *log_len) {
  return guarded([&] {
    LearnState scratch_state;
    LearnState &learn = model ? model->hist : scratch_state;
    learn.model = model ? model->m.get() : nullptr;
    learn.record = record != 0;
    learn.x.clear();
    learn.y.clear();
    const bool use_learn = learn.model || learn.record;
    std::vector<TensorPtr> m(N);
    for (int64_t i = 0; i < N; ++i) m[i] = T(mps[i]).clone();
    std::vector<const BTensor *> w(N);
    for (int64_t i = 0; i < N; ++i) w[i] = &T(mpo[i]);
    SweepParams p;
    p.sweeps = params->sweeps;
    p.Dmin = params->Dmin;
    p.Dmax = params->Dmax;
    p.trunc_err = params->trunc_err;
    p.lancz = {params->lancz_params.error, params->lancz_params.max_iterations,
               (int)params->lancz_params.matvec_precision};
    p.svd_mode = (int)params->svd_mode;
    p.svd_oversample = params->svd_oversample;
    p.svd_audit = params->svd_audit != 0;
    p.svd_sketch_max_fraction = params->svd_sketch_max_fraction > 0.0 &&
                                        params->svd_sketch_max_fraction < 1.0
                                    ? params->svd_sketch_max_fraction
                                    : 1.0;
    std::vector<SiteLog> lg;
    const double e = two_site_finite_vmps(c->ctx, m, w, p, &lg, use_learn ? &learn : nullptr);
    c->ctx.sync();
    for (int64_t i = 0; i < N; ++i) mps[i]->t = std::move(m[i]);
    if (nsamples) *nsamples = (int64_t)learn.y.size();
    if (samples_x && samples_y) {
      const int64_t ns = std::min<int64_t>(cap, (int64_t)learn.y.size());
      std::memcpy(samples_x, learn.x.data(), ns * kRankIn * sizeof(float));
      std::memcpy(samples_y, learn.y.data(), ns * sizeof(float));
    }
    if (e0) *e0 = e;
    if (log_len) *log_len = (int64_t)lg.size();
    if (log)
      for (int64_t i = 0; i < std::min<int64_t>(log_cap, (int64_t)lg.size()); ++i) {
        log[i] = site_log(lg[i]);
      }
  });
}

int udmrg_two_site_finite_vmps_noise(udmrg_ctx *c, int64_t N, udmrg_tensor **mps,
                                     udmrg_tensor *const *mpo, const udmrg_sweep_params *params,
                                     const udmrg_noise_params *noise, double *e0,
                                     udmrg_site_log *log, int64_t log_cap, int64_t *log_len,
                                     double *noise_log) {
  return guarded([&] {
    UDMRG_REQUIRE(noise != nullptr && (noise->n_noises == 0 || noise->noises != nullptr),
                  "noise vmps: missing noise parameters");
    std::vector<TensorPtr> m(N);
    for (int64_t i = 0; i < N; ++i) m[i] = T(mps[i]).clone();
    std::vector<const BTensor *> w(N);
    for (int64_t i = 0; i < N; ++i) w[i] = &T(mpo[i]);
    SweepParams p;
    p.sweeps = params->sweeps;
    p.Dmin = params->Dmin;
    p.Dmax = params->Dmax;
    p.trunc_err = params->trunc_err;
    p.lancz = {params->lancz_params.error, params->lancz_params.max_iterations,
               (int)params->lancz_params.matvec_precision};
    NoiseParams np;
    np.noises.assign(noise->noises, noise->noises + noise->n_noises);
    np.noise_decrease = noise->noise_decrease;
    np.noise_increase = noise->noise_increase;
    np.max_noise = noise->max_noise;
    np.alpha = noise->alpha;
    std::vector<SiteLog> lg;
    std::vector<double> nl;
    const double e = two_site_finite_vmps_noise(c->ctx, m, w, p, np, &lg, &nl);
    c->ctx.sync();
    for (int64_t i = 0; i < N; ++i) mps[i]->t = std::move(m[i]);
    if (e0) *e0 = e;
    if (log_len) *log_len = (int64_t)lg.size();
    for (int64_t i = 0; i < std::min<int64_t>(log_cap, (int64_t)lg.size()); ++i) {
      if (log) log[i] = site_log(lg[i]);
      if (noise_log) noise_log[i] = i < (int64_t)nl.size() ? nl[i] : 0.0;
    }
  });
}

int udmrg_finite_dmrg(udmrg_ctx *c, int64_t N, udmrg_tensor **mps,
                      const udmrg_mat_repr_site *mro, const udmrg_sweep_params *params,
                      double *e0, udmrg_site_log *log, int64_t log_cap, int64_t *log_len) {
  return guarded([&] {
    std::vector<MatReprSite> sites(N);
    for (int64_t i = 0; i < N; ++i) {
      sites[i].rows = mro[i].rows;
      sites[i].cols = mro[i].cols;
      for (int64_t n = 0; n < mro[i].nnz; ++n) {
        sites[i].x.push_back(mro[i].x[n]);
        sites[i].y.push_back(mro[i].y[n]);
        sites[i].ops.push_back(&T(mro[i].ops[n]));
      }
    }
    auto W = mat_repr_to_mpo(c->ctx, sites);
    std::vector<const BTensor *> w(N);
    for (int64_t i = 0; i < N; ++i) w[i] = W[i].get();
    std::vector<TensorPtr> m(N);
    for (int64_t i = 0; i < N; ++i) m[i] = T(mps[i]).clone();
    SweepParams p;
    p.sweeps = params->sweeps;
    p.Dmin = params->Dmin;
    p.Dmax = params->Dmax;
    p.trunc_err = params->trunc_err;
    p.lancz = {params->lancz_params.error, params->lancz_params.max_iterations,
               (int)params->lancz_params.matvec_precision};
    p.svd_mode = (int)params->svd_mode;
    p.svd_oversample = params->svd_oversample;
    p.svd_audit = params->svd_audit != 0;
    p.svd_sketch_max_fraction = params->svd_sketch_max_fraction > 0.0 &&
                                        params->svd_sketch_max_fraction < 1.0
                                    ? params->svd_sketch_max_fraction
                                    : 1.0;
    std::vector<SiteLog> lg;
    const double e = two_site_finite_vmps(c->ctx, m, w, p, &lg, nullptr);
    c->ctx.sync();
    for (int64_t i = 0; i < N; ++i) mps[i]->t = std::move(m[i]);
    if (e0) *e0 = e;
    if (log_len) *log_len = (int64_t)lg.size();
    if (log)
      for (int64_t i = 0; i < std::min<int64_t>(log_cap, (int64_t)lg.size()); ++i)
        log[i] = site_log(lg[i]);
  });
}

int udmrg_two_site_finite_tdvp(udmrg_ctx *c, int64_t N, udmrg_tensor **mps,
                               udmrg_tensor *const *mpo, const udmrg_tdvp_params *params,
                               udmrg_tdvp_log *log, int64_t log_cap, int64_t *log_len) {
  return guarded([&] {
    UDMRG_REQUIRE(params->steps >= 0, "tdvp: negative step count");
    std::vector<TensorPtr> m(N);
    for (int64_t i = 0; i < N; ++i) m[i] = T(mps[i]).clone();
    std::vector<const BTensor *> w(N);
    for (int64_t i = 0; i < N; ++i) w[i] = &T(mpo[i]);
    TdvpParams p;
    p.tau = params->tau;
    p.Dmin = params->Dmin;
    p.Dmax = params->Dmax;
    p.trunc_err = params->trunc_err;
    p.lancz = {params->lancz_params.error, params->lancz_params.max_iterations,
               (int)params->lancz_params.matvec_precision};
    std::vector<TdvpLog> lg;
    two_site_finite_tdvp(c->ctx, m, w, p, params->steps, &lg);
    c->ctx.sync();
    for (int64_t i = 0; i < N; ++i) mps[i]->t = std::move(m[i]);
    if (log_len) *log_len = (int64_t)lg.size();
    if (log)
      for (int64_t i = 0; i < std::min<int64_t>(log_cap, (int64_t)lg.size()); ++i) {
        const TdvpLog &t = lg[i];
        log[i] = {t.step, t.site, t.kind, t.trunc_err, t.D, t.iters, t.ee, t.lancz_sec, t.tot_sec};
      }
  });
}

int udmrg_matvec_plan_create(udmrg_ctx *c, udmrg_tensor *const *eff_ham,
                             const udmrg_tensor *psi_struct, udmrg_matvec_plan **out) {
  return udmrg_matvec_plan_create_ex(c, eff_ham, psi_struct, kPrecFP64, out);
}

int udmrg_matvec_plan_create_ex(udmrg_ctx *c, udmrg_tensor *const *eff_ham,
                                const udmrg_tensor *psi_struct, int precision,
                                udmrg_matvec_plan **out) {
  return guarded([&] {
    Ctx &ctx = c->ctx;
    const BTensor &psi = T(psi_struct);
    auto p = new udmrg_matvec_plan;
    p->ctx = &ctx;
    ctx.live_handles++;
    const BTensor *op[4];
    for (int i = 0; i < 4; ++i) {
      const BTensor &t = T(eff_ham[i]);
      if (t.dtype == psi.dtype) {
        op[i] = &t;
      } else {
        p->promoted[i] = to_complex(ctx, t);
        op[i] = p->promoted[i].get();
      }
    }
    p->plan = plan_matvec2(ctx, *op[0], *op[1], *op[2], *op[3], psi, precision);
    *out = p;
  });
}

int udmrg_matvec_plan_info(const udmrg_matvec_plan *p, double *flops, int64_t *psi_size,
                           int64_t *workspace_bytes) {
  return guarded([&] {
    const MatvecPlan &m = *p->plan;
    if (flops) *flops = m.flops;
    if (psi_size) *psi_size = m.sstruct->size();
    if (workspace_bytes)
      *workspace_bytes = (m.p1->out->size() + m.p2->out->size() + m.p3->out->size()) *
                         elem_doubles(m.sstruct->dtype) * (int64_t)sizeof(double);
  });
}

int udmrg_matvec_plan_embed(udmrg_matvec_plan *p, const udmrg_tensor *src, udmrg_tensor **out) {
  return guarded([&] { *out = wrap(embed(*p->ctx, T(src), *p->plan->sstruct)); });
}

int udmrg_matvec_plan_apply(udmrg_matvec_plan *p, const double *d_in, double *d_out) {
  return guarded([&] { p->plan->apply(d_in, d_out); });
}

// Device address of a page-locked, device-mapped host buffer of `bytes`
// bytes, or null: its first and last bytes must both be page-locked host
// memory mapped at the same distance apart in the device's address space.
static void *mapped_host(const void *h, size_t bytes) {
  if (!h || !bytes) return nullptr;
  cudaPointerAttributes a{}, z{};
  const char *last = (const char *)h + bytes - 1;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess ||
      cudaPointerGetAttributes(&z, last) != cudaSuccess) {
    cudaGetLastError();  // not an address the runtime knows: copied
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || z.type != cudaMemoryTypeHost || !a.devicePointer ||
      !z.devicePointer)
    return nullptr;
  if ((const char *)z.devicePointer - (const char *)a.devicePointer != (ptrdiff_t)(bytes - 1))
    return nullptr;
  return a.devicePointer;
}

int udmrg_matvec_plan_apply_host(udmrg_matvec_plan *p, const double *h_in, double *h_out) {
  return guarded([&] {
    MatvecPlan &m = *p->plan;
    Ctx &ctx = *p->ctx;
    const size_t bytes = (size_t)m.sstruct->size() * elem_doubles(m.sstruct->dtype) * sizeof(double);
    // the mixed form reads its input once (the psi pack) and writes its
    // output once (the .R GEMM's epilogue, every entry): both may live in
    // mapped host memory
    const bool mixed = m.sg != nullptr;
    const double *d_in =
        mixed && ctx.host_mapped >= 1 ? (const double *)mapped_host(h_in, bytes) : nullptr;
    double *d_out = mixed && ctx.host_mapped >= 2 ? (double *)mapped_host(h_out, bytes) : nullptr;
    if ((!d_in || !d_out) && !p->host_in) {
      p->host_in = (double *)ctx.alloc(std::max<size_t>(bytes, 8));
      p->host_out = (double *)ctx.alloc(std::max<size_t>(bytes, 8));
    }
    if (!d_in) {
      if (bytes)
        UDMRG_CHECK_CUDA(
            cudaMemcpyAsync(p->host_in, h_in, bytes, cudaMemcpyHostToDevice, ctx.stream));
      d_in = p->host_in;
    }
    m.apply(d_in, d_out ? d_out : p->host_out);
    if (!d_out && bytes)
      UDMRG_CHECK_CUDA(
          cudaMemcpyAsync(h_out, p->host_out, bytes, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
  });
}

int udmrg_matvec_plan_apply_anchor(udmrg_matvec_plan *p, const double *d_in, double *d_out) {
  return guarded([&] { p->plan->apply_anchor(d_in, d_out); });
}

int udmrg_probe_fp64_tflops(udmrg_ctx *c, double *tflops) {
  return guarded([&] { *tflops = probe_fp64_tflops(c->ctx); });
}

int udmrg_probe_krylov_step(udmrg_ctx *c, int64_t n, int step, double *ms, double *bytes,
                            int *second_pass_ran) {
  return guarded([&] {
    UDMRG_REQUIRE(c && ms && bytes && second_pass_ran, "null argument");
    krylov_step_probe(c->ctx, n, step, ms, bytes, second_pass_ran);
  });
}

int udmrg_selftest_sym_eig(udmrg_ctx *c, int64_t nmat, const int32_t *n, const double *mats,
                           const int32_t *k, double *lam, double *vecs) {
  return guarded([&] {
    Ctx &ctx = c->ctx;
    std::vector<EigJob> jobs(nmat);
    std::vector<int64_t> kk(nmat), zoff(nmat), zld(nmat);
    int64_t gtot = 0, ltot = 0, ztot = 0;
    for (int64_t i = 0; i < nmat; ++i) {
      UDMRG_REQUIRE(n[i] >= 1 && k[i] >= 0 && k[i] <= n[i], "sym_eig: bad sizes");
      jobs[i] = EigJob{gtot, ltot, n[i], 0};
      kk[i] = k[i];
      zoff[i] = ztot;
      zld[i] = std::max<int64_t>(k[i], 1);
      gtot += (int64_t)n[i] * n[i];
      ltot += n[i];
      ztot += (int64_t)n[i] * k[i];
    }
    DeviceScratch s(ctx);
    double *G = s.get<double>(gtot), *L = s.get<double>(ltot), *Z = s.get<double>(ztot);
    UDMRG_CHECK_CUDA(
        cudaMemcpyAsync(G, mats, gtot * sizeof(double), cudaMemcpyHostToDevice, ctx.stream));
    SymEigWork wk;
    const int st = sym_eig_values(ctx, s, jobs, G, L, wk);
    UDMRG_REQUIRE(st == 0, "sym_eig: non-finite input");
    std::vector<double> hl(ltot);
    UDMRG_CHECK_CUDA(
        cudaMemcpyAsync(hl.data(), L, ltot * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    sym_eig_vectors(ctx, s, jobs, G, L, hl, kk, zoff, zld, Z, wk);
    std::memcpy(lam, hl.data(), ltot * sizeof(double));
    if (ztot > 0)
      UDMRG_CHECK_CUDA(
          cudaMemcpyAsync(vecs, Z, ztot * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
  });
}

int udmrg_selftest_tc_gemm(udmrg_ctx *c, int64_t M, int64_t N, int64_t K, const double *hA,
                           const double *hB, double *hC) {
  return guarded([&] {
    Ctx &ctx = c->ctx;
    UDMRG_REQUIRE(M > 0 && N > 0 && K > 0 && M * K < (1ll << 28) && K * N < (1ll << 28),
                  "selftest: bad sizes");
    double *dA = (double *)ctx.alloc(M * K * sizeof(double));
    double *dB = (double *)ctx.alloc(K * N * sizeof(double));
    double *dC = (double *)ctx.alloc(M * N * sizeof(double));
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(dA, hA, M * K * sizeof(double), cudaMemcpyHostToDevice, ctx.stream));
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(dB, hB, K * N * sizeof(double), cudaMemcpyHostToDevice, ctx.stream));
    const int64_t abytes = tc_image_bytes(M, K, kTcBM), bbytes = tc_image_bytes(N, K, kTcBN);
    uint8_t *ai = (uint8_t *)ctx.alloc(abytes), *bi = (uint8_t *)ctx.alloc(bbytes);
    UDMRG_CHECK_CUDA(cudaMemsetAsync(ai, 0, abytes, ctx.stream));
    UDMRG_CHECK_CUDA(cudaMemsetAsync(bi, 0, bbytes, ctx.stream));
    const int32_t kc = (int32_t)((K + kTcBK - 1) / kTcBK);
    PackOp pa{0, K, 1, 0, (int32_t)M, (int32_t)K, 0, 0, kc, kTcBM, 0, 0};
    PackOp pb{0, 1, N, 0, (int32_t)N, (int32_t)K, 0, 0, kc, kTcBN, 0, 0};
    run_pack(ctx, std::vector<PackOp>{pa}, dA, true, ai);
    run_pack(ctx, std::vector<PackOp>{pb}, dB, true, bi);
    TcPlan plan;
    plan.ctx = &ctx;
    std::vector<int64_t> rows(M);
    for (int64_t m = 0; m < M; ++m) rows[m] = m * N;
    plan.add_group(0, 0, (int32_t)M, (int32_t)N, (int32_t)K, rows);
    plan.finalize();
    run_tc_gemm(ctx, plan, ai, bi, dC, kTcOutF64, 1.0);
    const int st = tc_check(ctx, plan);
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(hC, dC, M * N * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    for (void *p : {(void *)dA, (void *)dB, (void *)dC, (void *)ai, (void *)bi}) ctx.free(p);
    if (st) throw Error(kErrTimeout, "tcgen05 GEMM: a bounded device wait ran out");
  });
}

int udmrg_ctx_event_record(udmrg_ctx *c, int slot) {
  return guarded([&] {
    UDMRG_REQUIRE(slot >= 0 && slot < 1024, "event slot out of range");
    if ((int)c->events.size() <= slot) c->events.resize(slot + 1, nullptr);
    if (!c->events[slot]) UDMRG_CHECK_CUDA(cudaEventCreate(&c->events[slot]));
    UDMRG_CHECK_CUDA(cudaEventRecord(c->events[slot], c->ctx.stream));
  });
}

int udmrg_ctx_event_elapsed(udmrg_ctx *c, int a, int b, float *ms) {
  return guarded([&] {
    UDMRG_REQUIRE(a >= 0 && b >= 0 && a < (int)c->events.size() && b < (int)c->events.size() &&
                      c->events[a] && c->events[b],
                  "event slot not recorded");
    UDMRG_CHECK_CUDA(cudaEventSynchronize(c->events[b]));
    UDMRG_CHECK_CUDA(cudaEventElapsedTime(ms, c->events[a], c->events[b]));
  });
}

int udmrg_ctx_flush_l2(udmrg_ctx *c, int64_t bytes) {
  return guarded([&] {
    UDMRG_REQUIRE(bytes > 0, "flush size must be positive");
    if (c->flush_bytes < bytes) {
      if (c->flush_buf) c->ctx.free(c->flush_buf);
      c->flush_buf = c->ctx.alloc(bytes);
      c->flush_bytes = bytes;
    }
    UDMRG_CHECK_CUDA(cudaMemsetAsync(c->flush_buf, c->flush_bytes & 0xff, bytes, c->ctx.stream));
  });
}

int udmrg_matvec_plan_stage_bytes(udmrg_matvec_plan *p, double *bytes) {
  return guarded([&] {
    MatvecPlan &m = *p->plan;
    for (int i = 0; i < 4; ++i) bytes[i] = 0.0;
    if (m.sg) {
      const SgMatvecPlan &g = *m.sg;
      const double es = g.cplx ? 2.0 : 1.0;
      const double nreal = (double)g.psi_size * es;
      // psi pack: 8 B read, 3 x 2 B written per real number
      bytes[0] = 14.0 * nreal;
      // L.psi: both images read, 4 B per (unpadded) T1 entry written
      bytes[1] = (double)g.l_bytes + (double)g.psi_bytes + 4.0 * (double)m.p1->out->size() * es;
      if (g.fused) {  // T1 read once, R image read, FP64 result written
        bytes[3] = g.t1_read_bytes + (double)g.r_bytes + 8.0 * nreal;
      } else {
        bytes[2] = g.mpo_bytes;
        bytes[3] = (double)g.t3_bytes + (double)g.r_bytes + 8.0 * nreal;
      }
    }
  });
}

int udmrg_matvec_plan_tiles(const udmrg_matvec_plan *p, int *bn1, int *bn3, int *tuned) {
  return guarded([&] {
    const MatvecPlan &m = *p->plan;
    UDMRG_REQUIRE(m.sg != nullptr, "plan tiles: not a mixed-precision plan");
    if (bn1) *bn1 = m.sg->bn1;
    if (bn3) *bn3 = m.sg->bn3;
    if (tuned) *tuned = m.sg->tuned ? 1 : 0;
  });
}

int udmrg_matvec_plan_gemm_policy(const udmrg_matvec_plan *p, int *policy) {
  return guarded([&] { *policy = p->plan->p1->gemm.policy; });
}

int udmrg_matvec_plan_build_times(const udmrg_matvec_plan *p, double *sec) {
  return guarded([&] {
    for (int k = 0; k < 6; ++k) sec[k] = p->plan->build_sec[k];
  });
}

int udmrg_matvec_plan_set_fused(udmrg_matvec_plan *p, int enable) {
  return guarded([&] {
    MatvecPlan &m = *p->plan;
    UDMRG_REQUIRE(m.sg != nullptr, "set_fused: not a mixed-precision plan");
    m.sg->fused = enable != 0;
  });
}

int udmrg_matvec_plan_stage_times(udmrg_matvec_plan *p, const double *d_in, double *d_out,
                                  double *ms, double *flops) {
  return guarded([&] {
    MatvecPlan &m = *p->plan;
    Ctx &ctx = *p->ctx;
    float t[4] = {0, 0, 0, 0};
    if (m.sg) {
      m.sg->apply_timed(d_in, d_out, t);
      flops[0] = 0;
      flops[1] = 6.0 * m.sg->g1.flops;
      flops[2] = 0;
      flops[3] = 6.0 * m.sg->g3.flops;
    } else {
      const DType dt = m.sstruct->dtype;
      const int es = elem_doubles(dt);
      cudaEvent_t ev[5];
      for (auto &e : ev) UDMRG_CHECK_CUDA(cudaEventCreate(&e));
      cudaEventRecord(ev[0], ctx.stream);
      run_gemm(ctx, m.p1->gemm, dt, m.L->data, d_in, m.t1, 1.0, 0.0);
      cudaEventRecord(ev[1], ctx.stream);
      if (m.m64) {  // both MPO steps in one channel map (stage 2; stage 3 empty)
        run_mpo_step64(ctx, *m.m64, m.t1, m.t3);
        cudaEventRecord(ev[2], ctx.stream);
      } else {
        run_gemm(ctx, m.p2->gemm, dt, m.t1, m.W1->data, m.t2, 1.0, 0.0);
        cudaEventRecord(ev[2], ctx.stream);
        run_gemm(ctx, m.p3->gemm, dt, m.t2, m.W2->data, m.t3, 1.0, 0.0);
      }
      cudaEventRecord(ev[3], ctx.stream);
      for (int64_t b : m.missing)
        UDMRG_CHECK_CUDA(cudaMemsetAsync(d_out + m.sstruct->offs[b] * es, 0,
                                         m.sstruct->block_elems(b) * es * sizeof(double),
                                         ctx.stream));
      run_gemm(ctx, m.p4->gemm, dt, m.t3, m.R->data, d_out, 1.0, 0.0);
      cudaEventRecord(ev[4], ctx.stream);
      UDMRG_CHECK_CUDA(cudaEventSynchronize(ev[4]));
      for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&t[i], ev[i], ev[i + 1]);
      for (auto &e : ev) cudaEventDestroy(e);
      flops[0] = m.p1->gemm.flops;
      flops[1] = m.p2->gemm.flops;
      flops[2] = m.p3->gemm.flops;
      flops[3] = m.p4->gemm.flops;
    }
    for (int i = 0; i < 4; ++i) ms[i] = t[i];
  });
}

int udmrg_matvec_plan_destroy(udmrg_matvec_plan *p) {
  return guarded([&] {
    if (!p) return;
    Ctx *c = p->ctx;
    delete p;
    release_ctx(c);
  });
}

}  // extern "C"
