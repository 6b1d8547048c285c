#include "dmrg.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <future>
#include <limits>
#include <map>

namespace udmrg {

static_assert(kSpectrumFloor == kRankSv, "the SVD keeps the spectrum the rank model reads");

TensorPtr contract_axes(Ctx &ctx, const BTensor &A, const BTensor &B, const std::vector<int> &ca,
                        const std::vector<int> &cb) {
  auto p = plan_contract_axes(A, B, ca, cb);
  return run_contract(ctx, *p, A, B);
}

TensorPtr contract_cyclic(Ctx &ctx, const BTensor &A, const BTensor &B, int a_start, int b_start,
                          int n, bool dw) {
  auto p = plan_contract_cyclic(A, B, a_start, b_start, n);
  return run_contract(ctx, *p, A, B, dw);
}

TensorPtr dag(Ctx &ctx, const BTensor &A) {
  auto t = A.clone();
  for (auto &i : t->idx) i.dir = -i.dir;
  if (t->dtype == kC128) conj_inplace(ctx, t->data, t->size());
  return t;
}

TensorPtr to_complex(Ctx &ctx, const BTensor &A) {
  auto t = A.clone_struct();
  t->dtype = kC128;
  t->alloc_data();
  if (A.dtype == kC128) {
    if (A.size())
      UDMRG_CHECK_CUDA(cudaMemcpyAsync(t->data, A.data, A.bytes(), cudaMemcpyDeviceToDevice,
                                       ctx.stream));
  } else {
    real_to_complex(ctx, A.data, t->data, A.size());
  }
  return t;
}

// Block lists are sorted and unique, so union and difference are merges.
static int key_cmp(const int32_t *x, const int32_t *y, int r) {
  for (int i = 0; i < r; ++i)
    if (x[i] != y[i]) return x[i] < y[i] ? -1 : 1;
  return 0;
}

TensorPtr struct_union(const BTensor &a, const BTensor &b) {
  UDMRG_REQUIRE(a.rank() == b.rank(), "union: rank mismatch");
  for (int i = 0; i < a.rank(); ++i) UDMRG_REQUIRE(a.idx[i] == b.idx[i], "union: index mismatch");
  const int r = a.rank();
  const int64_t na = a.nblocks(), nb = b.nblocks();
  std::vector<int32_t> flat;
  flat.reserve((size_t)(na + nb) * r);
  for (int64_t i = 0, j = 0; i < na || j < nb;) {
    const int c = i == na ? 1 : j == nb ? -1 : key_cmp(a.key(i), b.key(j), r);
    const int32_t *k = c <= 0 ? a.key(i) : b.key(j);
    flat.insert(flat.end(), k, k + r);
    if (c <= 0) ++i;
    if (c >= 0) ++j;
  }
  auto t = a.clone_struct();
  t->set_blocks(std::move(flat));
  return t;
}

// keys of b's blocks that a lacks (flat, sorted)
static std::vector<int32_t> struct_minus(const BTensor &b, const BTensor &a) {
  const int r = b.rank();
  std::vector<int32_t> out;
  for (int64_t i = 0, j = 0; j < b.nblocks(); ++j) {
    while (i < a.nblocks() && key_cmp(a.key(i), b.key(j), r) < 0) ++i;
    if (i == a.nblocks() || key_cmp(a.key(i), b.key(j), r) != 0)
      out.insert(out.end(), b.key(j), b.key(j) + r);
  }
  return out;
}

TensorPtr embed(Ctx &ctx, const BTensor &src, const BTensor &dst_struct) {
  auto t = dst_struct.clone_struct();
  t->dtype = src.dtype;
  t->alloc_data();
  t->zero_data();
  const int es = elem_doubles(src.dtype);
  for (int64_t b = 0; b < src.nblocks(); ++b) {
    const int64_t d = t->find(std::vector<int32_t>(src.key(b), src.key(b) + src.rank()));
    UDMRG_REQUIRE(d >= 0, "embed: block absent from destination structure");
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(t->data + t->offs[d] * es, src.data + src.offs[b] * es,
                                     src.block_elems(b) * es * sizeof(double),
                                     cudaMemcpyDeviceToDevice, ctx.stream));
  }
  return t;
}

// ---------------------------------------------------------------------------
// Matvec plan
// ---------------------------------------------------------------------------

MatvecPlan::~MatvecPlan() {
  if (!ctx) return;
  ctx->free(t1);
  ctx->free(t2);
  ctx->free(t3);
}

// Tile policy of the FP64-accurate product's grouped GEMMs (the plain FP64
// matvec, or the mixed plan's anchor): fixed by ctx.gemm_policy, else the
// faster of the two policies in timed trials (zero input, best of two; the
// kernels' work does not depend on the values), cached per shape class
// (element type, anchor form, log2 of the Krylov structure's size, log2 of
// its largest right-bond sector).
static void tune_gemm_tiles(Ctx &ctx, MatvecPlan &mv) {
  std::vector<GemmPlan *> gp = {&mv.p1->gemm, &mv.p4->gemm};
  if (!mv.m64) {
    gp.push_back(&mv.p2->gemm);
    if (mv.p3) gp.push_back(&mv.p3->gemm);
  }
  auto retile = [&](int pol) {
    for (GemmPlan *g : gp) gemm_retile(*g, pol);
  };
  if (ctx.gemm_policy >= 0) {
    retile(ctx.gemm_policy);
    return;
  }
  const BTensor &S = *mv.sstruct;
  auto lg2 = [](int64_t x) {
    int64_t k = 0;
    while ((int64_t(1) << k) < x) ++k;
    return k;
  };
  int64_t maxb = 1;
  for (int64_t d : S.idx[S.rank() - 1].dims) maxb = std::max(maxb, d);
  const bool dw = mv.precision == kPrecMixed && ctx.anchor_dw;
  const std::array<int64_t, 4> key = {S.dtype == kC128 ? 1 : 0, dw ? 1 : 0, lg2(S.size()),
                                      lg2(maxb)};
  auto it = ctx.gemm_tuned.find(key);
  if (it != ctx.gemm_tuned.end()) {
    retile(it->second);
    return;
  }
  const int64_t nd = S.size() * elem_doubles(S.dtype);
  DeviceScratch sc(ctx);
  double *x = sc.get<double>(std::max<int64_t>(nd, 1)), *y = sc.get<double>(std::max<int64_t>(nd, 1));
  UDMRG_CHECK_CUDA(cudaMemsetAsync(x, 0, std::max<int64_t>(nd, 1) * sizeof(double), ctx.stream));
  cudaEvent_t e0, e1;
  UDMRG_CHECK_CUDA(cudaEventCreate(&e0));
  UDMRG_CHECK_CUDA(cudaEventCreate(&e1));
  float best[2] = {0, 0};
  for (int pol = 0; pol < 2; ++pol) {
    retile(pol);
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0, ctx.stream);
      mv.apply_fp64(x, y, dw);
      cudaEventRecord(e1, ctx.stream);
      UDMRG_CHECK_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      best[pol] = rep == 0 ? ms : std::min(best[pol], ms);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const int choice = best[1] < best[0] ? 1 : 0;
  retile(choice);
  ctx.gemm_tuned[key] = choice;
  ctx.gemm_trials++;
}

std::unique_ptr<MatvecPlan> plan_matvec2(Ctx &ctx, const BTensor &L, const BTensor &W1,
                                         const BTensor &W2, const BTensor &R,
                                         const BTensor &psi0, int precision) {
  UDMRG_REQUIRE(psi0.rank() == 4 && L.rank() == 3 && R.rank() == 3 && W1.rank() == 4 &&
                    W2.rank() == 4,
                "matvec: expects L(3), W1(4), W2(4), R(3), psi(4)");
  auto mv = std::make_unique<MatvecPlan>();
  mv->ctx = &ctx;
  mv->L = &L;
  mv->W1 = &W1;
  mv->W2 = &W2;
  mv->R = &R;
  using clk = std::chrono::steady_clock;
  auto tmark = clk::now();
  auto lap = [&] {
    const auto t = clk::now();
    const double s = std::chrono::duration<double>(t - tmark).count();
    tmark = t;
    return s;
  };
  // the Krylov structure: block structures only until it closes.  A
  // contraction's block set is the union over its operands' blocks, so each
  // round propagates only the blocks the previous one added (D) and the
  // intermediates' structures grow by union.
  TensorPtr S = psi0.clone_struct(), D = psi0.clone_struct();
  TensorPtr s1, s2, s3;  // the three intermediates' structures for the closed S
  std::vector<int> ca1, cb1, fa1, fb1, ca2, cb2, fa2, fb2, ca3, cb3, fa3, fb3, ca, cb, fa, fb;
  cyclic_axes(3, 4, 2, 0, 1, ca1, cb1, fa1, fb1);  // L(a', w, a) . psi(a, s1, s2, b)
  cyclic_axes(5, 4, 1, 0, 2, ca2, cb2, fa2, fb2);
  cyclic_axes(5, 4, 4, 0, 2, ca3, cb3, fa3, fb3);
  cyclic_axes(5, 3, 4, 1, 2, ca, cb, fa, fb);
  auto grow = [](TensorPtr &acc, TensorPtr d) {
    acc = acc ? struct_union(*acc, *d) : std::move(d);
  };
  for (int it = 0;; ++it) {
    UDMRG_REQUIRE(it < 16, "matvec: Krylov block structure did not close");
    auto d1 = contract_struct(L, *D, ca1, cb1, fa1, fb1);
    auto d2 = contract_struct(*d1, W1, ca2, cb2, fa2, fb2);
    auto d3 = contract_struct(*d2, W2, ca3, cb3, fa3, fb3);
    auto d4 = contract_struct(*d3, R, ca, cb, fa, fb);
    grow(s1, std::move(d1));
    grow(s2, std::move(d2));
    grow(s3, std::move(d3));
    std::vector<int32_t> fresh = struct_minus(*d4, *S);  // blocks not in S yet
    if (fresh.empty()) break;
    D = S->clone_struct();
    D->set_blocks(fresh);
    S = struct_union(*S, *D);
  }
  mv->build_sec[0] = lap();
  mv->precision = precision;
  UDMRG_REQUIRE(precision == kPrecFP64 || precision == kPrecMixed, "matvec: unknown precision");
  // real tensors: the two MPO steps as one sparse channel map (FP64 form) and
  // the same fused coefficients for the mixed form
  const bool real = L.dtype == kF64 && W1.dtype == kF64 && W2.dtype == kF64 &&
                    R.dtype == kF64 && psi0.dtype == kF64;
  const bool mixed = precision == kPrecMixed;
  std::unique_ptr<FusedMpo> fm, fm_sg;  // host copies of W1 W2 (one per thread)
  if (real || mixed) {
    fm = std::make_unique<FusedMpo>(ctx, W1, W2);
    if (real && mixed) fm_sg = std::make_unique<FusedMpo>(*fm);
  }
  FusedMpo *fmx = fm_sg ? fm_sg.get() : fm.get();
  int bn1 = 0, bn3 = 0;
  const bool sg_known = mixed && sg_tiles_known(ctx, *S, &bn1, &bn3);
  // The host halves of the plans are independent given the closed structure
  // and its intermediates, so they are built on host threads: the four
  // contraction plans, the FP64 MPO step's tables and the mixed form's
  // tables.  Device work (uploads, packing) follows on this thread.
  S->prepare_lookup();
  {
    using Fut = std::future<void>;
    std::vector<Fut> jobs;
    auto run = [&](auto fn) { jobs.push_back(std::async(std::launch::async, fn)); };
    run([&] { mv->p1 = plan_contract_axes(L, *S, {2}, {0}, false); });
    run([&] { mv->p2 = plan_contract_cyclic(*s1, W1, 1, 0, 2, false); });
    run([&] { mv->p3 = plan_contract_cyclic(*s2, W2, 4, 0, 2, false); });
    run([&] {
      mv->p4 = plan_contract_into(*s3, R, ca, cb, fa, fb, *S, &mv->missing, false);
    });
    if (real) run([&] { mv->m64 = build_mpo_step64(*fm, *s1, *s3); });
    if (sg_known) run([&] { mv->sg = plan_sg_tables(L, R, *S, *fmx, bn1, bn3); });
    for (Fut &f : jobs) f.wait();
    for (Fut &f : jobs) f.get();  // the first failure, after every job ended
  }
  // the plans chained on the closure's intermediates: the same structures
  UDMRG_REQUIRE(mv->p1->out->keys == s1->keys && mv->p2->out->keys == s2->keys &&
                    mv->p3->out->keys == s3->keys,
                "matvec: intermediate block structures differ from the closure's");
  mv->build_sec[1] = lap();
  for (ContractPlan *cp : {mv->p1.get(), mv->p2.get(), mv->p3.get(), mv->p4.get()})
    gemm_upload(cp->gemm);
  if (mv->m64) upload_mpo_step64(ctx, *mv->m64);
  mv->build_sec[2] = lap();
  mv->sstruct = std::move(S);
  mv->flops = mv->p1->gemm.flops + mv->p2->gemm.flops + mv->p3->gemm.flops + mv->p4->gemm.flops;
  if (mixed) {  // complex data through the real embedding
    if (mv->sg) {
      plan_sg_device(ctx, *mv->sg, L, R);
      mv->sg->tuned = !(ctx.tc_bn1 && ctx.tc_bn3);
    } else {
      mv->sg = plan_sg_matvec_tuned(ctx, L, R, *mv->sstruct, *fmx);
    }
    const double t = lap();
    mv->build_sec[3] = mv->sg->host_sec;
    mv->build_sec[4] = t;
  }
  // the FP64 form is kept in both modes (the mixed solver's final Rayleigh quotient)
  const int es = elem_doubles(psi0.dtype);
  mv->t1 = (double *)ctx.alloc(std::max<int64_t>(mv->p1->out->size(), 1) * es * sizeof(double));
  if (!mv->m64)
    mv->t2 = (double *)ctx.alloc(std::max<int64_t>(mv->p2->out->size(), 1) * es * sizeof(double));
  mv->t3 = (double *)ctx.alloc(std::max<int64_t>(mv->p3->out->size(), 1) * es * sizeof(double));
  tune_gemm_tiles(ctx, *mv);
  mv->build_sec[5] = lap();
  return mv;
}

std::unique_ptr<MatvecPlan> plan_matvec1(Ctx &ctx, const BTensor &L, const BTensor &W,
                                         const BTensor &R, const BTensor &psi0) {
  UDMRG_REQUIRE(psi0.rank() == 3 && L.rank() == 3 && R.rank() == 3 && W.rank() == 4,
                "single-site matvec: expects L(3), W(4), R(3), psi(3)");
  auto mv = std::make_unique<MatvecPlan>();
  mv->ctx = &ctx;
  mv->sites = 1;
  mv->L = &L;
  mv->W1 = &W;
  mv->R = &R;
  TensorPtr S = psi0.clone_struct();
  std::vector<int> ca1, cb1, fa1, fb1, ca2, cb2, fa2, fb2, ca, cb, fa, fb;
  cyclic_axes(3, 3, 2, 0, 1, ca1, cb1, fa1, fb1);  // L(a', w, a) . psi(a, s, b)
  cyclic_axes(4, 4, 1, 0, 2, ca2, cb2, fa2, fb2);
  cyclic_axes(4, 3, 3, 1, 2, ca, cb, fa, fb);
  for (int it = 0; it < 16; ++it) {
    auto s1 = contract_struct(L, *S, ca1, cb1, fa1, fb1);
    auto s2 = contract_struct(*s1, W, ca2, cb2, fa2, fb2);
    auto s4 = contract_struct(*s2, R, ca, cb, fa, fb);
    auto U = struct_union(*S, *s4);
    const bool closed = U->keys == S->keys;
    S = std::move(U);
    if (closed) break;
    UDMRG_REQUIRE(it < 15, "matvec: Krylov block structure did not close");
  }
  mv->p1 = plan_contract_axes(L, *S, {2}, {0});
  mv->p2 = plan_contract_cyclic(*mv->p1->out, W, 1, 0, 2);
  mv->p4 = plan_contract_into(*mv->p2->out, R, ca, cb, fa, fb, *S, &mv->missing);
  mv->sstruct = std::move(S);
  mv->flops = mv->p1->gemm.flops + mv->p2->gemm.flops + mv->p4->gemm.flops;
  const int es = elem_doubles(psi0.dtype);
  mv->t1 = (double *)ctx.alloc(std::max<int64_t>(mv->p1->out->size(), 1) * es * sizeof(double));
  mv->t2 = (double *)ctx.alloc(std::max<int64_t>(mv->p2->out->size(), 1) * es * sizeof(double));
  return mv;
}

void MatvecPlan::apply(const double *in, double *out) {
  if (sg) {
    sg->apply(in, out);
    return;
  }
  apply_fp64(in, out);
}

void MatvecPlan::apply_fp64(const double *in, double *out, bool dw) {
  const DType dt = sstruct->dtype;
  const int es = elem_doubles(dt);
  auto gemm = dw ? run_gemm_dw : run_gemm;
  gemm(*ctx, p1->gemm, dt, L->data, in, t1, 1.0, 0.0);
  if (m64) {
    run_mpo_step64(*ctx, *m64, t1, t3);
  } else {
    gemm(*ctx, p2->gemm, dt, t1, W1->data, t2, 1.0, 0.0);
    if (sites == 2) gemm(*ctx, p3->gemm, dt, t2, W2->data, t3, 1.0, 0.0);
  }
  for (int64_t b : missing)
    UDMRG_CHECK_CUDA(cudaMemsetAsync(out + sstruct->offs[b] * es, 0,
                                     sstruct->block_elems(b) * es * sizeof(double), ctx->stream));
  gemm(*ctx, p4->gemm, dt, sites == 2 ? t3 : t2, R->data, out, 1.0, 0.0);
}

// ---------------------------------------------------------------------------
// Tridiagonal eigenproblems (host, FP64).  Implicit QL iteration with
// Wilkinson-type shifts on a symmetric tridiagonal matrix (the method of
// Bowdler, Martin, Reinsch and Wilkinson, Numer. Math. 11 (1968) 293).
// ---------------------------------------------------------------------------

void tridiag_eig(const std::vector<double> &a, const std::vector<double> &b, int64_t n,
                 std::vector<double> &w, std::vector<double> &z) {
  std::vector<double> d(a.begin(), a.begin() + n), e(n, 0.0);
  for (int64_t i = 0; i + 1 < n; ++i) e[i] = b[i];
  z.assign(n * n, 0.0);
  for (int64_t i = 0; i < n; ++i) z[i * n + i] = 1.0;
  const double eps = 2.220446049250313e-16;
  for (int64_t l = 0; l < n; ++l) {
    int iter = 0;
    while (true) {
      int64_t m = l;
      for (; m + 1 < n; ++m) {
        const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= eps * dd) break;
      }
      if (m == l) break;
      if (++iter > 200) throw Error(kErrNumerics, "tridiagonal eigensolver did not converge");
      // shift from the leading 2x2 block
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + (g >= 0 ? std::fabs(r) : -std::fabs(r)));
      double s = 1.0, c = 1.0, p = 0.0;
      bool deflated = false;
      for (int64_t i = m - 1; i >= l; --i) {
        double f = s * e[i], bb = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {  // underflow: split the matrix here
          d[i + 1] -= p;
          e[m] = 0.0;
          deflated = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * bb;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - bb;
        for (int64_t k = 0; k < n; ++k) {  // accumulate the rotation into z
          const double zk1 = z[k * n + i + 1];
          z[k * n + i + 1] = s * z[k * n + i] + c * zk1;
          z[k * n + i] = c * z[k * n + i] - s * zk1;
        }
      }
      if (deflated) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  // ascending order
  std::vector<int64_t> ord(n);
  for (int64_t i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int64_t x, int64_t y) { return d[x] < d[y]; });
  w.resize(n);
  std::vector<double> zs(n * n);
  for (int64_t j = 0; j < n; ++j) {
    w[j] = d[ord[j]];
    for (int64_t k = 0; k < n; ++k) zs[k * n + j] = z[k * n + ord[j]];
  }
  z.swap(zs);
}

double tridiag_lowest(const std::vector<double> &a, const std::vector<double> &b, int64_t n,
                      std::vector<double> *vec) {
  std::vector<double> w, z;
  tridiag_eig(a, b, n, w, z);
  if (vec) {
    vec->resize(n);
    for (int64_t k = 0; k < n; ++k) (*vec)[k] = z[k * n];
  }
  return w[0];
}

std::vector<double> tridiag_expme1(const std::vector<double> &a, const std::vector<double> &b,
                                   int64_t n, double dt) {
  std::vector<double> w, z;
  tridiag_eig(a, b, n, w, z);
  std::vector<double> out(2 * n, 0.0);
  for (int64_t j = 0; j < n; ++j) {
    const double ph = -dt * w[j];
    const double cr = std::cos(ph) * z[j], ci = std::sin(ph) * z[j];  // e^{-i dt w_j} z[0][j]
    for (int64_t i = 0; i < n; ++i) {
      out[2 * i] += z[i * n + j] * cr;
      out[2 * i + 1] += z[i * n + j] * ci;
    }
  }
  return out;
}

// ---------------------------------------------------------------------------
// Lanczos
// ---------------------------------------------------------------------------

namespace {

struct EventTimer {
  cudaEvent_t a, b;
  EventTimer() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~EventTimer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

struct Bases {
  Ctx &ctx;
  std::vector<double *> v;
  explicit Bases(Ctx &c) : ctx(c) {}
  ~Bases() {
    for (auto p : v) ctx.free(p);
  }
};

// Runs the Krylov steps of one solve.  A step is the fixed launch sequence
// normalise (Y -> v_s, X), matvec (X -> Y), alpha, three-term update, the
// optional Gram-Schmidt passes and publish; every kernel reads the step
// index from the device, so with ctx.krylov_graph the sequence is captured
// once as a CUDA graph and each step is one graph launch.  Direct launches
// and graph replays run the same kernels on the same data (identical
// results).  run() returns after the step's one host synchronisation.
struct KrylovSteps {
  Ctx &ctx;
  KrylovWork &kw;
  MatvecPlan &mv;
  bool reorth;
  bool graph;
  EventTimer ev;
  cudaGraphExec_t exec = nullptr;
  uint64_t graph_kernels = 0;  // kernels one replay launches
  double seconds = 0;          // matvec device time (graph: whole steps)
  bool fp64;  // the plain FP64 matvec even for a mixed-precision plan (direct launches)
  KrylovSteps(Ctx &c, KrylovWork &k, MatvecPlan &m, bool with_reorth, bool fp64_matvec = false)
      : ctx(c), kw(k), mv(m), reorth(with_reorth), graph(c.krylov_graph && !fp64_matvec),
        fp64(fp64_matvec) {}
  ~KrylovSteps() {
    if (exec) cudaGraphExecDestroy(exec);
  }
  void issue(bool timed) {
    krylov_normalise(kw);
    if (timed) cudaEventRecord(ev.a, ctx.stream);
    if (fp64)
      mv.apply_anchor(kw.X, kw.Y);
    else
      mv.apply(kw.X, kw.Y);
    if (timed) cudaEventRecord(ev.b, ctx.stream);
    krylov_alpha(kw);
    krylov_update(kw);
    if (reorth) {
      krylov_project(kw, false);
      krylov_project(kw, true);
    }
    krylov_publish(kw);
  }
  void capture() {
    const uint64_t l0 = ctx.launches;
    UDMRG_CHECK_CUDA(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeRelaxed));
    cudaGraph_t g = nullptr;
    try {
      issue(false);
    } catch (...) {
      cudaStreamEndCapture(ctx.stream, &g);
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      ctx.launches = l0;
      throw;
    }
    UDMRG_CHECK_CUDA(cudaStreamEndCapture(ctx.stream, &g));
    graph_kernels = ctx.launches - l0;
    ctx.launches = l0;  // captured, not launched
    const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    UDMRG_CHECK_CUDA(e);
  }
  void run() {
    if (graph) {
      if (!exec) capture();
      cudaEventRecord(ev.a, ctx.stream);
      UDMRG_CHECK_CUDA(cudaGraphLaunch(exec, ctx.stream));
      cudaEventRecord(ev.b, ctx.stream);
      ctx.launches += graph_kernels;
    } else {
      issue(true);
    }
    ctx.sync();
    float ms = 0;
    cudaEventElapsedTime(&ms, ev.a, ev.b);
    seconds += ms * 1e-3;
  }
};

}  // namespace

LanczosResult lanczos_gs(Ctx &ctx, MatvecPlan &mv, const BTensor &init_state,
                         const LanczosParams &p) {
  const BTensor &S = *mv.sstruct;
  const bool cplx = S.dtype == kC128;
  const int es = elem_doubles(S.dtype);
  const int64_t n = S.size();
  const int64_t nd = n * es;
  const size_t vbytes = std::max<int64_t>(nd, 1) * sizeof(double);
  // eff_ham_eff_dim: element count of the initial state
  const int64_t eff_dim = init_state.size();
  const int64_t maxit = p.max_iterations;
  // the second step already writes a[1] (the reference's loop writes bases[1])
  UDMRG_REQUIRE(maxit >= 2, "Lanczos: max_iterations must be at least 2");
  VecWork w(ctx);
  Bases bases(ctx);
  LanczosResult res;
  const bool mixed = mv.sg != nullptr;
  KrylovWork kw(ctx, n, cplx, maxit);
  KrylovSteps steps(ctx, kw, mv, mixed);
  auto gs = S.clone_struct();
  gs->alloc_data();
  // gs = sum_i vec_i v_i
  auto combine = [&](int64_t m, const std::vector<double> &vec) {
    std::vector<const double *> vs(bases.v.begin(), bases.v.begin() + m);
    std::vector<double> coef;
    for (int64_t i = 0; i < m; ++i) {
      coef.push_back(vec[i]);
      if (cplx) coef.push_back(0.0);
    }
    lincomb(w, gs->data, vs, coef, n, cplx);
  };
  // One Lanczos run from the vector in Y (krylov_begin): step m normalises
  // gamma_{m-1} into v_m, then gamma_m = H v_m - a_m v_m - b_{m-1} v_{m-1};
  // with mixed precision gamma is then projected against every basis vector
  // (FP64 classical Gram-Schmidt, a second pass where the first removed more
  // than half of |gamma|^2), so rounding in the matvec cannot build up ghost
  // Ritz values.  alpha and |gamma| reach the host once per step; the
  // convergence test on the (m+1)-dimensional tridiagonal matrix follows
  // (lanczos_vmps_solver_impl.h:203-235).  first: the steps object of step 0.
  // Returns the Ritz value and leaves the Ritz vector in gs.
  auto run = [&](KrylovSteps &first, bool noise_stop, int64_t &iters) {
    std::vector<double> a(maxit, 0.0), b(maxit, 0.0);
    int64_t m = 0;
    double energy0 = 0.0;
    while (true) {
      if ((int64_t)bases.v.size() <= m) bases.v.push_back((double *)ctx.alloc(vbytes));
      kw.push((int)m, bases.v[m]);
      (m == 0 ? first : steps).run();
      res.matvecs++;
      a[m] = kw.hres[0];
      const double n2 = kw.hres[1];
      if (m == 0) {
        energy0 = a[0];
      } else {
        const double e_new = tridiag_lowest(a, b, m + 1, nullptr);
        // mixed precision also stops once the Ritz value no longer moves above
        // the rounding level of the split-BF16 products
        const bool noise_floor =
            noise_stop && std::fabs(energy0 - e_new) <= 1e-12 * std::fabs(e_new);
        if ((energy0 - e_new) < p.error || noise_floor || m == eff_dim || m == maxit - 1) {
          std::vector<double> vec;
          tridiag_lowest(a, b, m + 1, &vec);
          iters = m + 1;
          combine(m + 1, vec);
          return e_new;
        }
        energy0 = e_new;
      }
      const double norm_gamma = std::sqrt(n2);
      if (norm_gamma == 0.0) {  // invariant subspace
        std::vector<double> vec = {1.0};
        if (m > 0) tridiag_lowest(a, b, m + 1, &vec);
        iters = m + 1;
        combine(m + 1, vec);
        return energy0;
      }
      b[m] = norm_gamma;
      m += 1;
    }
  };
  // Y = init; step 0 normalises it into bases[0] (QuasiNormalize)
  {
    auto v0 = embed(ctx, init_state, S);
    krylov_begin(kw, v0->data);
  }
  int64_t it1 = 0;
  double e = run(steps, mixed, it1);
  res.iters = it1;
  if (mixed) {
    // Refinement.  The mixed-precision Krylov space converges to an
    // eigenvector of the rounded operator; its error (first order in the
    // split-BF16 rounding over the spectral gap) would enter the truncation
    // and the environments.  A second Lanczos run starts from that vector
    // with one FP64 step: alpha_0 = <psi|H psi> and the residual gamma_0 =
    // H psi - alpha_0 psi are exact, so the tridiagonal matrix couples psi
    // to the correction space exactly, and the mixed-precision steps after
    // it only build the correction space (their rounding enters the Ritz
    // vector scaled by the correction's size, the energy by its square).
    // It stops by the same rule; near convergence that is one or two steps.
    res.ritz_eng = e;
    krylov_begin(kw, gs->data);
    KrylovSteps first(ctx, kw, mv, true, /*fp64_matvec=*/true);
    int64_t it2 = 0;
    e = run(first, false, it2);
    steps.seconds += first.seconds;
    res.iters += it2;
    res.fp64_matvecs = 1;
  }
  res.gs_eng = e;
  res.matvec_seconds = steps.seconds;
  if (mv.sg && (tc_check(ctx, mv.sg->g1) | tc_check(ctx, mv.sg->g3)))
    throw Error(kErrTimeout, "tcgen05 GEMM: a bounded device wait ran out");
  res.gs_vec = std::move(gs);
  return res;
}

ExpmvResult lanczos_expmv(Ctx &ctx, MatvecPlan &mv, const BTensor &init_state, double step,
                          const LanczosParams &p) {
  const BTensor &S = *mv.sstruct;
  UDMRG_REQUIRE(S.dtype == kC128, "expmv: complex state required");
  const int64_t n = S.size();
  const int64_t nd = 2 * n;
  const size_t vbytes = std::max<int64_t>(nd, 1) * sizeof(double);
  const int64_t eff_dim = init_state.size();
  const int64_t maxit = p.max_iterations;
  UDMRG_REQUIRE(maxit >= 2, "Lanczos expmv: max_iterations must be at least 2");
  VecWork w(ctx);
  Bases bases(ctx);
  std::vector<double> a(maxit, 0.0), b(maxit, 0.0);
  ExpmvResult res;
  auto combine = [&](int64_t m, const std::vector<double> &coef_il) {
    auto out = S.clone_struct();
    out->alloc_data();
    std::vector<const double *> vs(bases.v.begin(), bases.v.begin() + m);
    lincomb(w, out->data, vs, coef_il, n, true);
    return out;
  };
  const bool mixed = mv.sg != nullptr;
  KrylovWork kw(ctx, n, true, maxit);
  KrylovSteps steps(ctx, kw, mv, mixed);
  {
    auto v0 = embed(ctx, init_state, S);
    krylov_begin(kw, v0->data);
  }
  double initial_norm = 0.0;
  int64_t m = 0;
  std::vector<double> last_coef(2 * maxit, 0.0);
  // step m as in lanczos_gs: one host synchronisation per step
  while (true) {
    double *vm = (double *)ctx.alloc(vbytes);
    bases.v.push_back(vm);
    kw.push((int)m, vm);
    steps.run();
    if (m == 0) initial_norm = std::sqrt(kw.hres[2]);
    a[m] = kw.hres[0];
    const double n2 = kw.hres[1];
    if (m > 0) {
      auto coef = tridiag_expme1(a, b, m + 1, step);
      double dist = 0;
      for (int64_t i = 0; i < m + 1; ++i) {
        const double dr = coef[2 * i] - last_coef[2 * i];
        const double di = coef[2 * i + 1] - last_coef[2 * i + 1];
        dist += dr * dr + di * di;
      }
      dist = std::sqrt(dist);
      if (dist < p.error || m == eff_dim || m == maxit - 1) {
        for (auto &x : coef) x *= initial_norm;
        res.iters = m + 1;
        res.expmv = combine(m + 1, coef);
        return res;
      }
      std::fill(last_coef.begin(), last_coef.end(), 0.0);
      std::copy(coef.begin(), coef.end(), last_coef.begin());
    }
    const double norm_gamma = std::sqrt(n2);
    if (norm_gamma == 0.0) {  // invariant subspace
      res.iters = m + 1;
      if (m == 0) {
        const double ph = -step * a[0];
        res.expmv = combine(1, {initial_norm * std::cos(ph), initial_norm * std::sin(ph)});
      } else {
        auto c = tridiag_expme1(a, b, m + 1, step);
        for (auto &x : c) x *= initial_norm;
        res.expmv = combine(m + 1, c);
      }
      return res;
    }
    b[m] = norm_gamma;
    m += 1;
  }
}

// ---------------------------------------------------------------------------
// Environments
// ---------------------------------------------------------------------------

TensorPtr update_site_lenv(Ctx &ctx, const BTensor &lenv, const BTensor &A, const BTensor &W,
                           bool dw) {
  auto Ad = dag(ctx, A);
  auto t = contract_cyclic(ctx, lenv, A, 2, 0, 1, dw);
  auto t2 = contract_cyclic(ctx, *t, W, 1, 0, 2, dw);
  t.reset();
  return contract_cyclic(ctx, *Ad, *t2, 0, 1, 2, dw);
}

TensorPtr update_site_renv(Ctx &ctx, const BTensor &renv, const BTensor &A, const BTensor &W,
                           bool dw) {
  auto Ad = dag(ctx, A);
  auto t = contract_cyclic(ctx, *Ad, renv, 2, 0, 1, dw);
  auto t2 = contract_cyclic(ctx, *t, W, 1, 2, 2, dw);
  t.reset();
  return contract_cyclic(ctx, *t2, A, 3, 1, 2, dw);
}

static TensorPtr trivial_env(Ctx &ctx, const Index &i0, const Index &iw, DType dt) {
  auto t = std::make_unique<BTensor>();
  t->ctx = &ctx;
  t->dtype = dt;
  t->idx = {i0, iw, i0.inverse()};
  UDMRG_REQUIRE(i0.nsec() == 1 && i0.dims[0] == 1 && iw.nsec() == 1 && iw.dims[0] == 1,
                "trivial env: boundary indexes must be one-dimensional");
  t->set_blocks({0, 0, 0});
  t->alloc_data();
  double one[2] = {1.0, 0.0};
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(t->data, one, elem_doubles(dt) * sizeof(double),
                                   cudaMemcpyHostToDevice, ctx.stream));
  ctx.sync();
  return t;
}

TensorPtr trivial_renv(Ctx &ctx, const BTensor &mps_last, const BTensor &mpo_last) {
  auto t = trivial_env(ctx, mps_last.idx[2], mpo_last.idx[3].inverse(), mps_last.dtype);
  t->nq = mps_last.nq;
  return t;
}

TensorPtr trivial_lenv(Ctx &ctx, const BTensor &mps_first, const BTensor &mpo_first) {
  auto t = trivial_env(ctx, mps_first.idx[0], mpo_first.idx[0].inverse(), mps_first.dtype);
  t->nq = mps_first.nq;
  return t;
}

// ---------------------------------------------------------------------------
// Sweeps
// ---------------------------------------------------------------------------

static double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

static void two_site_update(Ctx &ctx, std::vector<TensorPtr> &mps,
                            std::vector<TensorPtr> &lenvs, std::vector<TensorPtr> &renvs,
                            const std::vector<const BTensor *> &mpo, const SweepParams &p,
                            char dir, int64_t target, std::vector<SiteLog> *log,
                            LearnState *learn, double &e0) {
  const int64_t N = (int64_t)mps.size();
  int64_t l, r, lenv_len, renv_len;
  if (dir == 'r') {
    l = target;
    r = target + 1;
    lenv_len = target;
    renv_len = N - (target + 2);
  } else {
    l = target - 1;
    r = target;
    lenv_len = target - 1;
    renv_len = N - target - 1;
  }
  SiteLog lg{};
  // learned sketch sizes from the spectra this bond had at its previous visit
  SketchHint hint;
  const SketchHint *hp = nullptr;
  BondSpectra now;
  BondSpectra *prev = learn ? &learn->prev[l] : nullptr;
  std::vector<float> feats;
  std::vector<QN> fqn;
  if (prev && !prev->empty()) {
    // dominant sector of the previous spectrum and previous kept counts
    QN top = (*prev)[0].first;
    double best = -1;
    for (auto &kv : *prev)
      if (!kv.second.empty() && kv.second[0] > best) {
        best = kv.second[0];
        top = kv.first;
      }
    const auto &kept_prev = learn->prev_kept[l];
    auto kept_of = [&](const QN &q) {
      for (auto &kk : kept_prev)
        if (kk.first == q) return kk.second;
      return (int64_t)0;
    };
    // the bond's previous cutoff (smallest kept value) and dimension
    double cut = 0.0;
    int64_t dprev = 0;
    for (auto &kv : *prev) {
      const int64_t k = kept_of(kv.first);
      dprev += k;
      if (k > 0 && k <= (int64_t)kv.second.size())
        cut = cut == 0.0 ? kv.second[k - 1] : std::min(cut, kv.second[k - 1]);
    }
    const double growth = std::log2((double)std::max<int64_t>(p.Dmax, 1) /
                                    (double)std::max<int64_t>(dprev, 1));
    for (auto &kv : *prev) {
      feats.resize(feats.size() + kRankIn);
      rank_features(kv.second, kv.first, top, p.trunc_err, kept_of(kv.first), cut, growth,
                    feats.data() + feats.size() - kRankIn);
      fqn.push_back(kv.first);
    }
    if (learn->model && p.svd_mode == kSvdSketchLearned) {
      const int64_t n = (int64_t)fqn.size();
      DeviceScratch s(ctx);
      float *dx = s.get<float>(feats.size()), *dy = s.get<float>(n);
      UDMRG_CHECK_CUDA(cudaMemcpyAsync(dx, feats.data(), feats.size() * sizeof(float),
                                       cudaMemcpyHostToDevice, ctx.stream));
      learn->model->predict(dx, n, dy);
      std::vector<float> y(n);
      UDMRG_CHECK_CUDA(
          cudaMemcpyAsync(y.data(), dy, n * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
      ctx.sync();
      for (int64_t i = 0; i < n; ++i) {
        const double k = std::max(0.0, std::ceil(std::exp2((double)y[i]) - 1.0));
        hint.push_back({fqn[i], (int64_t)k});
      }
      hp = &hint;
    }
  }
  auto res = two_site_update_local(ctx, *lenvs[lenv_len], *renvs[renv_len], *mps[l], *mps[r],
                                   *mpo[l], *mpo[r], p, dir, &lg, hp, learn ? &now : nullptr);
  lg.site = target;
  if (learn) {
    // kept counts of this update per bond QN = the new bond index of mps[l]
    std::vector<std::pair<QN, int64_t>> kept_now;
    const Index &bond = res.mps_l->idx[2];
    for (int q = 0; q < bond.nsec(); ++q) kept_now.push_back({bond.qns[q], bond.dims[q]});
    if (learn->record) {
      for (size_t i = 0; i < fqn.size(); ++i) {
        int64_t k = 0;
        for (auto &kk : kept_now)
          if (kk.first == fqn[i]) k = kk.second;
        learn->x.insert(learn->x.end(), feats.begin() + i * kRankIn,
                        feats.begin() + (i + 1) * kRankIn);
        learn->y.push_back((float)std::log2(1.0 + (double)k));
      }
    }
    learn->prev[l] = std::move(now);
    learn->prev_kept[l] = std::move(kept_now);
  }
  mps[l] = std::move(res.mps_l);
  mps[r] = std::move(res.mps_r);
  if (dir == 'r')
    lenvs[lenv_len + 1] = std::move(res.env);
  else
    renvs[renv_len + 1] = std::move(res.env);
  e0 = lg.e0;
  if (log) log->push_back(lg);
}

LocalUpdate two_site_update_local(Ctx &ctx, const BTensor &lenv, const BTensor &renv,
                                  const BTensor &mps_l, const BTensor &mps_r,
                                  const BTensor &mpo_l, const BTensor &mpo_r,
                                  const SweepParams &p, char dir, SiteLog *log,
                                  const SketchHint *hint, BondSpectra *spectra) {
  UDMRG_REQUIRE(dir == 'r' || dir == 'l', "dir must be 'r' or 'l'");
  const double t0 = now();
  auto init_state = contract_axes(ctx, mps_l, mps_r, {2}, {0});
  auto mv = plan_matvec2(ctx, lenv, mpo_l, mpo_r, renv, *init_state, p.lancz.precision);
  const double tplan = now() - t0;
  auto lres = lanczos_gs(ctx, *mv, *init_state, p.lancz);
  const double t1 = now();
  const double mvflops = mv->flops;
  init_state.reset();
  mv.reset();
  const BTensor &psi = *lres.gs_vec;
  const QN ldiv = mps_l.div();
  const int split = dir == 'r' ? kSvdSplitLeft : kSvdSplitRight;
  SvdResult sres;
  double audit_err = -1.0, audit_sec = 0.0;
  int64_t audit_diff = 0;
  // the mixed form's SVD: Newton-Schulz and factor products in double-word
  // arithmetic (reset on every exit from this scope)
  struct SvdDw {
    Ctx &c;
    SvdDw(Ctx &x, bool on) : c(x) { c.svd_dw = on; }
    ~SvdDw() { c.svd_dw = false; }
  } svd_dw(ctx, p.lancz.precision == kPrecMixed && ctx.anchor_dw);
  if (p.svd_mode == kSvdExact || (p.svd_mode == kSvdSketchLearned && !hint)) {
    sres = svd_trunc(ctx, psi, 2, ldiv, p.trunc_err, p.Dmin, p.Dmax, split,
                     spectra ? kSpectrumFloor : 0);
  } else {
    SketchParams sp;
    sp.oversample = p.svd_oversample;
    sp.max_fraction = p.svd_sketch_max_fraction;
    sp.seed = 0x5EEDull + (uint64_t)mps_l.nblocks();
    if (hint) {
      sp.sketch = *hint;
    } else {  // the bond's current sector dimensions (its state from the last visit)
      const Index &bond = mps_l.idx[2];
      for (int q = 0; q < bond.nsec(); ++q) sp.sketch.push_back({bond.qns[q], bond.dims[q]});
    }
    sres = svd_trunc_sketch(ctx, psi, 2, ldiv, p.trunc_err, p.Dmin, p.Dmax, split, sp);
    if (p.svd_audit) {  // the exact block SVD judges the randomized one
      const double ta = now();
      SvdResult ex = svd_trunc(ctx, psi, 2, ldiv, p.trunc_err, p.Dmin, p.Dmax, split);
      audit_err = std::fabs(ex.trunc_err - sres.trunc_err);
      std::map<QN, int64_t> kx;
      for (size_t q = 0; q < ex.sector_qn.size(); ++q) kx[ex.sector_qn[q]] = ex.sector_kept[q];
      for (size_t q = 0; q < sres.sector_qn.size(); ++q) {
        auto it = kx.find(sres.sector_qn[q]);
        const int64_t k = it == kx.end() ? 0 : it->second;
        audit_diff += std::llabs(k - sres.sector_kept[q]);
        if (it != kx.end()) kx.erase(it);
      }
      for (auto &kv : kx) audit_diff += kv.second;
      audit_sec = now() - ta;
    }
  }
  ctx.svd_dw = false;
  lres.gs_vec.reset();
  if (spectra) {
    spectra->clear();
    for (size_t q = 0; q < sres.sector_qn.size(); ++q)
      spectra->push_back({sres.sector_qn[q], sres.sector_svals[q]});
  }
  LocalUpdate out;
  out.mps_l = std::move(sres.u);
  out.mps_r = std::move(sres.vt);
  ctx.sync();
  const double t2 = now();
  // the mixed form's environments in double-word arithmetic with its anchor
  const bool env_dw = p.lancz.precision == kPrecMixed && ctx.anchor_dw;
  if (dir == 'r')
    out.env = update_site_lenv(ctx, lenv, *out.mps_l, mpo_l, env_dw);
  else
    out.env = update_site_renv(ctx, renv, *out.mps_r, mpo_r, env_dw);
  ctx.sync();
  const double e0 = lres.gs_eng;
  const double t3 = now();
  {
    int64_t sk = 0;
    for (int64_t v : sres.sector_sketch) sk += v;
    if (log)
      *log = {0, e0, sres.trunc_err, sres.D, lres.iters, sres.ee, t1 - t0,
              t2 - t1 - audit_sec, t3 - t2, t3 - t0 - audit_sec, mvflops, sk, sres.grow_rounds,
              audit_err, audit_diff, tplan};
  }
  return out;
}

double two_site_finite_vmps(Ctx &ctx, std::vector<TensorPtr> &mps,
                            const std::vector<const BTensor *> &mpo, const SweepParams &p,
                            std::vector<SiteLog> *log, LearnState *learn) {
  const int64_t N = (int64_t)mps.size();
  UDMRG_REQUIRE(N >= 3 && (int64_t)mpo.size() == N, "vmps: MPS and MPO sizes differ or N < 3");
  // mixed element types: promote real MPO / MPS to complex
  bool cplx = false;
  for (auto &t : mps) cplx |= t->dtype == kC128;
  for (auto *t : mpo) cplx |= t->dtype == kC128;
  std::vector<TensorPtr> mpo_c;
  std::vector<const BTensor *> W = mpo;
  if (cplx) {
    for (auto &t : mps)
      if (t->dtype != kC128) t = to_complex(ctx, *t);
    for (int64_t i = 0; i < N; ++i)
      if (mpo[i]->dtype != kC128) {
        mpo_c.push_back(to_complex(ctx, *mpo[i]));
        W[i] = mpo_c.back().get();
      }
  }
  std::vector<TensorPtr> lenvs(N), renvs(N);
  renvs[0] = trivial_renv(ctx, *mps[N - 1], *W[N - 1]);
  for (int64_t i = 1; i <= N - 2; ++i)
    renvs[i] = update_site_renv(ctx, *renvs[i - 1], *mps[N - i], *W[N - i]);
  lenvs[0] = trivial_lenv(ctx, *mps[0], *W[0]);
  if (learn && (int64_t)learn->prev.size() != N) {  // history is kept across calls
    learn->prev.assign(N, {});
    learn->prev_kept.assign(N, {});
  }
  double e0 = 0.0;
  for (int64_t s = 0; s < p.sweeps; ++s) {
    for (int64_t i = 0; i < N - 2; ++i)
      two_site_update(ctx, mps, lenvs, renvs, W, p, 'r', i, log, learn, e0);
    for (int64_t i = N - 1; i > 1; --i)
      two_site_update(ctx, mps, lenvs, renvs, W, p, 'l', i, log, learn, e0);
  }
  return e0;
}

namespace {

// Two-site forward evolution exp(-i step H_eff) of the pair (l, l+1), truncated
// SVD, MPS split by direction and one environment update
// (TwoSiteFiniteTDVPEvolution, two_site_update_finite_tdvp_impl.h:261-417).
void tdvp_two_site(Ctx &ctx, std::vector<TensorPtr> &mps, std::vector<TensorPtr> &lenvs,
                   std::vector<TensorPtr> &renvs, const std::vector<const BTensor *> &W,
                   const TdvpParams &p, char dir, int64_t target, double step, TdvpLog &lg) {
  const int64_t N = (int64_t)mps.size();
  int64_t l, r, lenv_len, renv_len;
  if (dir == 'r') {
    l = target;
    r = target + 1;
    lenv_len = target;
    renv_len = N - (target + 2);
  } else {
    l = target - 1;
    r = target;
    lenv_len = target - 1;
    renv_len = N - target - 1;
  }
  const double t0 = now();
  auto init = contract_axes(ctx, *mps[l], *mps[r], {2}, {0});
  auto mv = plan_matvec2(ctx, *lenvs[lenv_len], *W[l], *W[r], *renvs[renv_len], *init,
                         p.lancz.precision);
  auto ex = lanczos_expmv(ctx, *mv, *init, step, p.lancz);
  mv.reset();
  init.reset();
  const double t1 = now();
  SvdResult sres = svd_trunc(ctx, *ex.expmv, 2, mps[l]->div(), p.trunc_err, p.Dmin, p.Dmax,
                             dir == 'r' ? kSvdSplitLeft : kSvdSplitRight);
  ex.expmv.reset();
  mps[l] = std::move(sres.u);
  mps[r] = std::move(sres.vt);
  if (dir == 'r')
    lenvs[lenv_len + 1] = update_site_lenv(ctx, *lenvs[lenv_len], *mps[target], *W[target]);
  else
    renvs[renv_len + 1] = update_site_renv(ctx, *renvs[renv_len], *mps[target], *W[target]);
  ctx.sync();
  lg = TdvpLog{0, target, 2, sres.trunc_err, sres.D, ex.iters, sres.ee, t1 - t0, now() - t0};
}

// Single-site backward evolution exp(+i tau/2 H_eff) of the centre tensor at
// `site`, without a split (SingleSiteFiniteTDVPBackwardEvolution with
// dir 'n', two_site_update_finite_tdvp_impl.h:419-531).
void tdvp_one_site(Ctx &ctx, std::vector<TensorPtr> &mps, std::vector<TensorPtr> &lenvs,
                   std::vector<TensorPtr> &renvs, const std::vector<const BTensor *> &W,
                   const TdvpParams &p, int64_t site, double step, TdvpLog &lg) {
  const int64_t N = (int64_t)mps.size();
  const double t0 = now();
  auto mv = plan_matvec1(ctx, *lenvs[site], *W[site], *renvs[N - site - 1], *mps[site]);
  auto ex = lanczos_expmv(ctx, *mv, *mps[site], step, p.lancz);
  mv.reset();
  mps[site] = std::move(ex.expmv);
  ctx.sync();
  const double t1 = now();
  lg = TdvpLog{0, site, 1, 0.0, 0, ex.iters, 0.0, t1 - t0, t1 - t0};
}

}  // namespace

void two_site_finite_tdvp(Ctx &ctx, std::vector<TensorPtr> &mps,
                          const std::vector<const BTensor *> &mpo, const TdvpParams &p,
                          int64_t steps, std::vector<TdvpLog> *log) {
  const int64_t N = (int64_t)mps.size();
  UDMRG_REQUIRE(N >= 3 && (int64_t)mpo.size() == N, "tdvp: MPS and MPO sizes differ or N < 3");
  std::vector<TensorPtr> mpo_c;
  std::vector<const BTensor *> W = mpo;
  for (auto &t : mps)
    if (t->dtype != kC128) t = to_complex(ctx, *t);
  for (int64_t i = 0; i < N; ++i)
    if (mpo[i]->dtype != kC128) {
      mpo_c.push_back(to_complex(ctx, *mpo[i]));
      W[i] = mpo_c.back().get();
    }
  // right-canonical form from the last site down to site 1 (centre at site 0):
  // mps[i] = (U S) V^T, V^T right-isometric, U S absorbed into mps[i - 1]
  for (int64_t i = N - 1; i > 0; --i) {
    SvdResult sr = svd_trunc(ctx, *mps[i], 1, mps[i]->div(), 0.0, 1, INT64_MAX / 4,
                             kSvdSplitRight);
    mps[i] = std::move(sr.vt);
    mps[i - 1] = contract_axes(ctx, *mps[i - 1], *sr.u, {2}, {0});
  }
  std::vector<TensorPtr> lenvs(N), renvs(N);
  renvs[0] = trivial_renv(ctx, *mps[N - 1], *W[N - 1]);
  for (int64_t i = 1; i <= N - 2; ++i)
    renvs[i] = update_site_renv(ctx, *renvs[i - 1], *mps[N - i], *W[N - i]);
  lenvs[0] = trivial_lenv(ctx, *mps[0], *W[0]);
  const double half = p.tau / 2;
  TdvpLog lg{};
  auto put = [&](int64_t st) {
    lg.step = st;
    if (log) log->push_back(lg);
  };
  for (int64_t st = 0; st < steps; ++st) {
    for (int64_t i = 0; i < N - 2; ++i) {
      tdvp_two_site(ctx, mps, lenvs, renvs, W, p, 'r', i, half, lg);
      put(st);
      tdvp_one_site(ctx, mps, lenvs, renvs, W, p, i + 1, -half, lg);
      put(st);
    }
    for (int64_t i = N - 1; i > 1; --i) {
      tdvp_two_site(ctx, mps, lenvs, renvs, W, p, 'l', i, i == N - 1 ? p.tau : half, lg);
      put(st);
      tdvp_one_site(ctx, mps, lenvs, renvs, W, p, i - 1, -half, lg);
      put(st);
    }
    tdvp_two_site(ctx, mps, lenvs, renvs, W, p, 'r', 0, half, lg);
    put(st);
  }
}

}  // namespace udmrg
