// Contraction planner: block matching by quantum numbers -> grouped GEMM.
#include <algorithm>
#include <map>

#include "gemm.hpp"

namespace udmrg {

GemmPlan::~GemmPlan() {
  if (!ctx) return;
  ctx->free(d_segs);
  ctx->free(d_probs);
  for (auto &p : d_tiles) ctx->free(p);
}

template <typename V>
static V *upload_vec(Ctx *ctx, const std::vector<V> &v) {
  if (v.empty()) return nullptr;
  V *d = (V *)ctx->alloc(v.size() * sizeof(V));
  UDMRG_CHECK_CUDA(
      cudaMemcpyAsync(d, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, ctx->stream));
  return d;
}

void GemmPlan::upload() {
  d_segs = upload_vec(ctx, segs);
  d_probs = upload_vec(ctx, probs);
  for (int c = 0; c < kNumCfg; ++c) d_tiles[c] = upload_vec(ctx, tiles[c]);
  // host vectors stay: the descriptors are read before the upload completes
  ctx->sync();
}

static const int kCfgBM[kNumCfg] = {64, 256, 16, 32};
static const int kCfgBN[kNumCfg] = {64, 16, 256, 32};

void cyclic_axes(int ra, int rb, int a_start, int b_start, int n, std::vector<int> &ca,
                 std::vector<int> &cb, std::vector<int> &fa, std::vector<int> &fb) {
  ca.clear();
  cb.clear();
  fa.clear();
  fb.clear();
  for (int i = 0; i < n; ++i) {
    ca.push_back((a_start + i) % ra);
    cb.push_back((b_start + i) % rb);
  }
  for (int i = 0; i < ra - n; ++i) fa.push_back((a_start + n + i) % ra);
  for (int i = 0; i < rb - n; ++i) fb.push_back((b_start + n + i) % rb);
}

namespace {

struct SubDim {
  int64_t ext;
  int64_t sa, sb;  // strides in operand A / B (unused one = 0)
};

// Row-major strides of a block with the given sector ids.
void block_strides(const BTensor &T, int64_t b, std::vector<int64_t> &st) {
  const int r = T.rank();
  st.assign(r, 1);
  for (int i = r - 2; i >= 0; --i) st[i] = st[i + 1] * T.dim_of(b, i + 1);
}

struct Pair {
  int64_t a, b;
};

// Choose the tile configuration with the least padded work and emit the tiles.
void add_tiles(GemmPlan &g, int32_t pid, int64_t M, int64_t N) {
  int best = 0;
  double bestw = 1e300;
  for (int c = 0; c < kNumCfg; ++c) {
    double w = (double)((M + kCfgBM[c] - 1) / kCfgBM[c] * kCfgBM[c]) *
               (double)((N + kCfgBN[c] - 1) / kCfgBN[c] * kCfgBN[c]);
    if (w < bestw * 0.999) {
      bestw = w;
      best = c;
    }
  }
  for (int64_t m0 = 0; m0 < M; m0 += kCfgBM[best])
    for (int64_t n0 = 0; n0 < N; n0 += kCfgBN[best])
      g.tiles[best].push_back({pid, (int32_t)m0, (int32_t)n0, 0});
}

}  // namespace

static std::unique_ptr<ContractPlan> plan_impl(const BTensor &A, const BTensor &B,
                                               const std::vector<int> &ca,
                                               const std::vector<int> &cb,
                                               const std::vector<int> &fa,
                                               const std::vector<int> &fb, const BTensor *dst,
                                               std::vector<int64_t> *missing) {
  UDMRG_REQUIRE(ca.size() == cb.size(), "contract: axis lists differ in length");
  UDMRG_REQUIRE(A.dtype == B.dtype, "contract: operands must have the same element type");
  UDMRG_REQUIRE(fa.size() + ca.size() == (size_t)A.rank(), "contract: bad A axes");
  UDMRG_REQUIRE(fb.size() + cb.size() == (size_t)B.rank(), "contract: bad B axes");
  for (size_t i = 0; i < ca.size(); ++i) {
    const Index &ia = A.idx[ca[i]], &ib = B.idx[cb[i]];
    UDMRG_REQUIRE(ia.same_space(ib) && ia.dir == -ib.dir,
                  "contract: contracted indexes do not match (sectors or directions)");
  }
  auto plan = std::make_unique<ContractPlan>();
  plan->gemm.ctx = A.ctx;
  auto out = std::make_unique<BTensor>();
  out->ctx = A.ctx;
  out->dtype = A.dtype;
  out->nq = A.nq;
  for (int i : fa) out->idx.push_back(A.idx[i]);
  for (int i : fb) out->idx.push_back(B.idx[i]);
  const int ro = out->rank();
  UDMRG_REQUIRE(ro > 0, "contract: full contractions to a scalar are not supported here");

  // B blocks grouped by contracted sector ids
  std::map<std::vector<int32_t>, std::vector<int64_t>> bgroups;
  for (int64_t b = 0; b < B.nblocks(); ++b) {
    std::vector<int32_t> k;
    for (int ax : cb) k.push_back(B.key(b)[ax]);
    bgroups[k].push_back(b);
  }
  // enumerate matching pairs -> output keys
  std::map<std::vector<int32_t>, std::vector<Pair>> outmap;
  for (int64_t a = 0; a < A.nblocks(); ++a) {
    std::vector<int32_t> k;
    for (int ax : ca) k.push_back(A.key(a)[ax]);
    auto it = bgroups.find(k);
    if (it == bgroups.end()) continue;
    for (int64_t b : it->second) {
      std::vector<int32_t> ok;
      ok.reserve(ro);
      for (int ax : fa) ok.push_back(A.key(a)[ax]);
      for (int ax : fb) ok.push_back(B.key(b)[ax]);
      outmap[ok].push_back({a, b});
    }
  }
  std::vector<int32_t> flat;
  flat.reserve(outmap.size() * ro);
  for (auto &kv : outmap) flat.insert(flat.end(), kv.first.begin(), kv.first.end());
  out->set_blocks(flat);  // std::map iteration is already sorted and unique

  const BTensor *C = out.get();
  if (dst) {
    UDMRG_REQUIRE(dst->rank() == ro, "contract-into: rank mismatch");
    for (int i = 0; i < ro; ++i)
      UDMRG_REQUIRE(dst->idx[i] == out->idx[i], "contract-into: index mismatch");
    C = dst;
    if (missing) {
      missing->clear();
      std::vector<char> hit(dst->nblocks(), 0);
      for (auto &kv : outmap) {
        int64_t id = dst->find(kv.first);
        UDMRG_REQUIRE(id >= 0, "contract-into: produced block absent from destination");
        hit[id] = 1;
      }
      for (int64_t i = 0; i < dst->nblocks(); ++i)
        if (!hit[i]) missing->push_back(i);
    }
  }

  GemmPlan &g = plan->gemm;
  std::vector<int64_t> sa, sb;
  const double cplx = A.dtype == kC128 ? 4.0 : 1.0;
  for (auto &kv : outmap) {
    const std::vector<int32_t> &okey = kv.first;
    const std::vector<Pair> &pairs = kv.second;
    GProb p{};
    p.c_off = C->offs[dst ? dst->find(okey) : (int64_t)g.probs.size()];
    // M / N sub-dims (extents are the output block's sector dims)
    std::vector<int64_t> mext, next;
    for (size_t i = 0; i < fa.size(); ++i) mext.push_back(A.idx[fa[i]].dims[okey[i]]);
    for (size_t i = 0; i < fb.size(); ++i) next.push_back(B.idx[fb[i]].dims[okey[fa.size() + i]]);
    // merge decisions valid for all segments
    const int nmi = (int)mext.size(), nni = (int)next.size();
    std::vector<char> mmerge(std::max(nmi - 1, 0), 1), nmerge(std::max(nni - 1, 0), 1);
    for (auto &pr : pairs) {
      block_strides(A, pr.a, sa);
      block_strides(B, pr.b, sb);
      for (int i = 0; i + 1 < nmi; ++i)
        if (sa[fa[i]] != mext[i + 1] * sa[fa[i + 1]]) mmerge[i] = 0;
      for (int i = 0; i + 1 < nni; ++i)
        if (sb[fb[i]] != next[i + 1] * sb[fb[i + 1]]) nmerge[i] = 0;
    }
    // build merged M groups: list of (ext, index of last original dim)
    auto groups = [](const std::vector<int64_t> &ext, const std::vector<char> &mg) {
      std::vector<std::pair<int64_t, int>> gr;
      for (int i = 0; i < (int)ext.size(); ++i) {
        if (i > 0 && mg[i - 1]) {
          gr.back().first *= ext[i];
          gr.back().second = i;
        } else {
          gr.push_back({ext[i], i});
        }
      }
      // drop extent-1 groups
      std::vector<std::pair<int64_t, int>> r;
      for (auto &x : gr)
        if (x.first != 1) r.push_back(x);
      return r;
    };
    auto mg = groups(mext, mmerge);
    auto ng = groups(next, nmerge);
    UDMRG_REQUIRE(mg.size() <= (size_t)kMaxSub && ng.size() <= (size_t)kMaxSub,
                  "contract: too many non-mergeable free axes");
    int64_t M = 1, N = 1;
    for (auto &x : mext) M *= x;
    for (auto &x : next) N *= x;
    UDMRG_REQUIRE(M < (1ll << 31) && N < (1ll << 31), "contract: block too large");
    p.M = (int32_t)M;
    p.N = (int32_t)N;
    p.nm = (int32_t)mg.size();
    p.nn = (int32_t)ng.size();
    for (size_t j = 0; j < mg.size(); ++j) p.m_ext[j] = (int32_t)mg[j].first;
    for (size_t j = 0; j < ng.size(); ++j) p.n_ext[j] = (int32_t)ng[j].first;
    p.seg0 = (int32_t)g.segs.size();
    p.nseg = (int32_t)pairs.size();
    double kflops = 0;
    for (auto &pr : pairs) {
      block_strides(A, pr.a, sa);
      block_strides(B, pr.b, sb);
      GSeg s{};
      s.a_off = A.offs[pr.a];
      s.b_off = B.offs[pr.b];
      for (size_t j = 0; j < mg.size(); ++j) s.a_ms[j] = sa[fa[mg[j].second]];
      for (size_t j = 0; j < ng.size(); ++j) s.b_ns[j] = sb[fb[ng[j].second]];
      // K sub-dims with merging where both operands allow it
      std::vector<SubDim> kd;
      for (size_t i = 0; i < ca.size(); ++i) {
        SubDim d{A.dim_of(pr.a, ca[i]), sa[ca[i]], sb[cb[i]]};
        if (!kd.empty() && kd.back().sa == d.ext * d.sa && kd.back().sb == d.ext * d.sb) {
          kd.back().ext *= d.ext;
          kd.back().sa = d.sa;
          kd.back().sb = d.sb;
        } else if (d.ext != 1) {
          kd.push_back(d);
        }
      }
      // drop unit dims that slipped in through the first slot
      std::vector<SubDim> kd2;
      for (auto &d : kd)
        if (d.ext != 1) kd2.push_back(d);
      UDMRG_REQUIRE(kd2.size() <= (size_t)kMaxSub, "contract: too many contracted sub-dims");
      int64_t K = 1;
      for (auto &d : kd2) K *= d.ext;
      s.nk = (int32_t)kd2.size();
      s.K = (int32_t)K;
      for (size_t j = 0; j < kd2.size(); ++j) {
        s.k_ext[j] = (int32_t)kd2[j].ext;
        s.a_ks[j] = kd2[j].sa;
        s.b_ks[j] = kd2[j].sb;
      }
      kflops += (double)K;
      g.segs.push_back(s);
    }
    g.flops += 2.0 * cplx * (double)M * (double)N * kflops;
    add_tiles(g, (int32_t)g.probs.size(), M, N);
    g.probs.push_back(p);
  }
  gemm_finalize(g);
  plan->out = std::move(out);
  return plan;
}

void gemm_add_simple(GemmPlan &g, int64_t c_off, int64_t M, int64_t N, int64_t K, int64_t a_off,
                     int64_t a_ms, int64_t a_ks, int64_t b_off, int64_t b_ks, int64_t b_ns,
                     bool cplx) {
  if (M == 0 || N == 0) return;
  UDMRG_REQUIRE(M < (1ll << 31) && N < (1ll << 31) && K < (1ll << 31), "gemm: too large");
  GProb p{};
  p.c_off = c_off;
  p.M = (int32_t)M;
  p.N = (int32_t)N;
  p.nm = 1;
  p.nn = 1;
  p.m_ext[0] = (int32_t)M;
  p.n_ext[0] = (int32_t)N;
  p.seg0 = (int32_t)g.segs.size();
  p.nseg = 1;
  GSeg s{};
  s.a_off = a_off;
  s.b_off = b_off;
  s.a_ms[0] = a_ms;
  s.b_ns[0] = b_ns;
  s.nk = K > 0 ? 1 : 0;
  s.K = (int32_t)K;
  s.k_ext[0] = (int32_t)K;
  s.a_ks[0] = a_ks;
  s.b_ks[0] = b_ks;
  g.segs.push_back(s);
  g.flops += 2.0 * (cplx ? 4.0 : 1.0) * (double)M * (double)N * (double)K;
  add_tiles(g, (int32_t)g.probs.size(), M, N);
  g.probs.push_back(p);
}

void gemm_finalize(GemmPlan &g) {
  // largest K first for load balance
  std::vector<int64_t> ktot(g.probs.size(), 0);
  for (size_t i = 0; i < g.probs.size(); ++i)
    for (int s = 0; s < g.probs[i].nseg; ++s) ktot[i] += g.segs[g.probs[i].seg0 + s].K;
  for (int c = 0; c < kNumCfg; ++c)
    std::stable_sort(g.tiles[c].begin(), g.tiles[c].end(), [&](const GTile &x, const GTile &y) {
      return ktot[x.prob] > ktot[y.prob];
    });
  g.upload();
}

std::unique_ptr<ContractPlan> plan_contract(const BTensor &A, const BTensor &B,
                                            const std::vector<int> &ca, const std::vector<int> &cb,
                                            const std::vector<int> &fa,
                                            const std::vector<int> &fb) {
  return plan_impl(A, B, ca, cb, fa, fb, nullptr, nullptr);
}

std::unique_ptr<ContractPlan> plan_contract_into(const BTensor &A, const BTensor &B,
                                                 const std::vector<int> &ca,
                                                 const std::vector<int> &cb,
                                                 const std::vector<int> &fa,
                                                 const std::vector<int> &fb, const BTensor &dst,
                                                 std::vector<int64_t> *missing) {
  return plan_impl(A, B, ca, cb, fa, fb, &dst, missing);
}

std::unique_ptr<ContractPlan> plan_contract_axes(const BTensor &A, const BTensor &B,
                                                 const std::vector<int> &ca,
                                                 const std::vector<int> &cb) {
  std::vector<int> fa, fb;
  for (int i = 0; i < A.rank(); ++i)
    if (std::find(ca.begin(), ca.end(), i) == ca.end()) fa.push_back(i);
  for (int i = 0; i < B.rank(); ++i)
    if (std::find(cb.begin(), cb.end(), i) == cb.end()) fb.push_back(i);
  return plan_contract(A, B, ca, cb, fa, fb);
}

std::unique_ptr<ContractPlan> plan_contract_cyclic(const BTensor &A, const BTensor &B, int a_start,
                                                   int b_start, int n) {
  std::vector<int> ca, cb, fa, fb;
  cyclic_axes(A.rank(), B.rank(), a_start, b_start, n, ca, cb, fa, fb);
  return plan_contract(A, B, ca, cb, fa, fb);
}

TensorPtr run_contract(Ctx &ctx, const ContractPlan &plan, const BTensor &A, const BTensor &B) {
  auto out = plan.out->clone_struct();
  out->alloc_data();
  run_gemm(ctx, plan.gemm, A.dtype, A.data, B.data, out->data, 1.0, 0.0);
  return out;
}

}  // namespace udmrg
