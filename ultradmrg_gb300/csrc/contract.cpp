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

constexpr int kMaxRank = 8;

// Row-major strides of a block with the given sector ids.
void block_strides(const BTensor &T, int64_t b, int64_t *st) {
  const int r = T.rank();
  st[r - 1] = 1;
  for (int i = r - 2; i >= 0; --i) st[i] = st[i + 1] * T.dim_of(b, i + 1);
}

// Sector-id tuples packed 16 bits per axis, first axis in the highest bits,
// so integer order is the lexicographic order of the tuples.
using Key128 = unsigned __int128;

struct Match {
  Key128 okey;
  int64_t a, b;
};

// Choose the tile configuration with the least padded work and emit the tiles.
// Policy 1 charges 32 x 32 tiles (four outputs per thread) twice their padded
// work, so they are taken only where the larger tiles would pad more than
// twice as much.
void add_tiles(GemmPlan &g, int32_t pid, int64_t M, int64_t N, int policy) {
  int best = 0;
  double bestw = 1e300;
  for (int c = 0; c < kNumCfg; ++c) {
    double w = (double)((M + kCfgBM[c] - 1) / kCfgBM[c] * kCfgBM[c]) *
               (double)((N + kCfgBN[c] - 1) / kCfgBN[c] * kCfgBN[c]);
    if (policy == 1 && c == kCfg32x32) w *= 2.0;
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

static void sort_tiles(GemmPlan &g);

static std::unique_ptr<ContractPlan> plan_impl(const BTensor &A, const BTensor &B,
                                               const std::vector<int> &ca,
                                               const std::vector<int> &cb,
                                               const std::vector<int> &fa,
                                               const std::vector<int> &fb, const BTensor *dst,
                                               std::vector<int64_t> *missing, bool upload) {
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

  UDMRG_REQUIRE(A.rank() <= kMaxRank && B.rank() <= kMaxRank && ro <= kMaxRank,
                "contract: tensors of rank above 8 are not supported");
  for (const BTensor *T : {&A, &B})
    for (const Index &ix : T->idx)
      UDMRG_REQUIRE(ix.nsec() < 65536, "contract: more than 65535 sectors on one index");
  // B blocks sorted by their contracted sector ids
  std::vector<std::pair<uint64_t, int64_t>> bk(B.nblocks());
  for (int64_t b = 0; b < B.nblocks(); ++b) {
    uint64_t k = 0;
    for (int ax : cb) k = (k << 16) | (uint64_t)B.key(b)[ax];
    bk[b] = {k, b};
  }
  std::sort(bk.begin(), bk.end());
  // matching pairs with their output keys, sorted by (output key, a, b)
  std::vector<Match> matches;
  for (int64_t a = 0; a < A.nblocks(); ++a) {
    uint64_t k = 0;
    for (int ax : ca) k = (k << 16) | (uint64_t)A.key(a)[ax];
    auto it = std::lower_bound(bk.begin(), bk.end(), std::make_pair(k, (int64_t)-1));
    Key128 ka = 0;
    for (int ax : fa) ka = (ka << 16) | (Key128)A.key(a)[ax];
    for (; it != bk.end() && it->first == k; ++it) {
      Key128 ok = ka;
      for (int ax : fb) ok = (ok << 16) | (Key128)B.key(it->second)[ax];
      matches.push_back({ok, a, it->second});
    }
  }
  std::sort(matches.begin(), matches.end(), [](const Match &x, const Match &y) {
    if (x.okey != y.okey) return x.okey < y.okey;
    if (x.a != y.a) return x.a < y.a;
    return x.b < y.b;
  });
  // output blocks = distinct keys; [mstart[o], mstart[o + 1]) are their matches
  std::vector<int32_t> flat;
  std::vector<size_t> mstart;
  for (size_t i = 0; i < matches.size(); ++i) {
    if (i > 0 && matches[i].okey == matches[i - 1].okey) continue;
    mstart.push_back(i);
    flat.resize(flat.size() + ro);
    Key128 ok = matches[i].okey;
    for (int j = ro - 1; j >= 0; --j) {
      flat[flat.size() - ro + j] = (int32_t)(uint32_t)(ok & 0xFFFF);
      ok >>= 16;
    }
  }
  mstart.push_back(matches.size());
  const size_t nout = mstart.size() - 1;
  out->set_blocks(flat);  // sorted and unique by construction

  const BTensor *C = out.get();
  if (dst) {
    UDMRG_REQUIRE(dst->rank() == ro, "contract-into: rank mismatch");
    for (int i = 0; i < ro; ++i)
      UDMRG_REQUIRE(dst->idx[i] == out->idx[i], "contract-into: index mismatch");
    C = dst;
  }
  // destination block of every output block
  std::vector<int64_t> dest(nout);
  {
    std::vector<int32_t> okey(ro);
    std::vector<char> hit(dst ? dst->nblocks() : 0, 0);
    for (size_t o = 0; o < nout; ++o) {
      if (!dst) {
        dest[o] = (int64_t)o;
        continue;
      }
      std::copy(flat.begin() + o * ro, flat.begin() + (o + 1) * ro, okey.begin());
      const int64_t id = dst->find(okey);
      UDMRG_REQUIRE(id >= 0, "contract-into: produced block absent from destination");
      dest[o] = id;
      hit[id] = 1;
    }
    if (dst && missing) {
      missing->clear();
      for (int64_t i = 0; i < dst->nblocks(); ++i)
        if (!hit[i]) missing->push_back(i);
    }
  }

  GemmPlan &g = plan->gemm;
  int64_t sa[kMaxRank], sb[kMaxRank];
  const double cplx = A.dtype == kC128 ? 4.0 : 1.0;
  const int nmi = (int)fa.size(), nni = (int)fb.size();
  // merged groups of free axes: (extent, index of the last original axis),
  // extent-1 groups dropped
  auto groups = [](const int64_t *ext, int n, const char *mg, int64_t *gext, int *glast) {
    int ng = 0;
    int64_t ce = 1;
    int cl = -1;
    for (int i = 0; i < n; ++i) {
      if (i > 0 && mg[i - 1]) {
        ce *= ext[i];
        cl = i;
      } else {
        if (cl >= 0 && ce != 1) {
          gext[ng] = ce;
          glast[ng++] = cl;
        }
        ce = ext[i];
        cl = i;
      }
    }
    if (cl >= 0 && ce != 1) {
      gext[ng] = ce;
      glast[ng++] = cl;
    }
    return ng;
  };
  for (size_t o = 0; o < nout; ++o) {
    const int32_t *okey = flat.data() + o * ro;
    const size_t m0 = mstart[o], m1 = mstart[o + 1];
    GProb p{};
    p.c_off = C->offs[dest[o]];
    // M / N sub-dims (extents are the output block's sector dims)
    int64_t mext[kMaxRank], next[kMaxRank];
    for (int i = 0; i < nmi; ++i) mext[i] = A.idx[fa[i]].dims[okey[i]];
    for (int i = 0; i < nni; ++i) next[i] = B.idx[fb[i]].dims[okey[nmi + i]];
    // merge decisions valid for all segments
    char mmerge[kMaxRank], nmerge[kMaxRank];
    for (int i = 0; i < kMaxRank; ++i) mmerge[i] = nmerge[i] = 1;
    for (size_t q = m0; q < m1; ++q) {
      block_strides(A, matches[q].a, sa);
      block_strides(B, matches[q].b, sb);
      for (int i = 0; i + 1 < nmi; ++i)
        if (sa[fa[i]] != mext[i + 1] * sa[fa[i + 1]]) mmerge[i] = 0;
      for (int i = 0; i + 1 < nni; ++i)
        if (sb[fb[i]] != next[i + 1] * sb[fb[i + 1]]) nmerge[i] = 0;
    }
    int64_t mgx[kMaxRank], ngx[kMaxRank];
    int mgl[kMaxRank], ngl[kMaxRank];
    const int nmg = groups(mext, nmi, mmerge, mgx, mgl);
    const int nng = groups(next, nni, nmerge, ngx, ngl);
    UDMRG_REQUIRE(nmg <= kMaxSub && nng <= kMaxSub, "contract: too many non-mergeable free axes");
    int64_t M = 1, N = 1;
    for (int i = 0; i < nmi; ++i) M *= mext[i];
    for (int i = 0; i < nni; ++i) N *= next[i];
    UDMRG_REQUIRE(M < (1ll << 31) && N < (1ll << 31), "contract: block too large");
    p.M = (int32_t)M;
    p.N = (int32_t)N;
    p.nm = nmg;
    p.nn = nng;
    for (int j = 0; j < nmg; ++j) p.m_ext[j] = (int32_t)mgx[j];
    for (int j = 0; j < nng; ++j) p.n_ext[j] = (int32_t)ngx[j];
    p.seg0 = (int32_t)g.segs.size();
    p.nseg = (int32_t)(m1 - m0);
    double kflops = 0;
    for (size_t q = m0; q < m1; ++q) {
      const int64_t pa = matches[q].a, pb = matches[q].b;
      block_strides(A, pa, sa);
      block_strides(B, pb, sb);
      GSeg sg{};
      sg.a_off = A.offs[pa];
      sg.b_off = B.offs[pb];
      for (int j = 0; j < nmg; ++j) sg.a_ms[j] = sa[fa[mgl[j]]];
      for (int j = 0; j < nng; ++j) sg.b_ns[j] = sb[fb[ngl[j]]];
      // K sub-dims merged where both operands allow it; unit dims dropped
      SubDim kd[kMaxRank];
      int nk = 0;
      for (size_t i = 0; i < ca.size(); ++i) {
        SubDim d{A.dim_of(pa, ca[i]), sa[ca[i]], sb[cb[i]]};
        if (nk > 0 && kd[nk - 1].sa == d.ext * d.sa && kd[nk - 1].sb == d.ext * d.sb) {
          kd[nk - 1].ext *= d.ext;
          kd[nk - 1].sa = d.sa;
          kd[nk - 1].sb = d.sb;
        } else if (d.ext != 1) {
          kd[nk++] = d;
        }
      }
      int nk2 = 0;
      for (int i = 0; i < nk; ++i)
        if (kd[i].ext != 1) kd[nk2++] = kd[i];
      UDMRG_REQUIRE(nk2 <= kMaxSub, "contract: too many contracted sub-dims");
      int64_t K = 1;
      for (int i = 0; i < nk2; ++i) K *= kd[i].ext;
      sg.nk = nk2;
      sg.K = (int32_t)K;
      for (int j = 0; j < nk2; ++j) {
        sg.k_ext[j] = (int32_t)kd[j].ext;
        sg.a_ks[j] = kd[j].sa;
        sg.b_ks[j] = kd[j].sb;
      }
      kflops += (double)K;
      g.segs.push_back(sg);
    }
    g.flops += 2.0 * cplx * (double)M * (double)N * kflops;
    add_tiles(g, (int32_t)g.probs.size(), M, N, g.policy);
    g.probs.push_back(p);
  }
  if (upload)
    gemm_finalize(g);
  else
    sort_tiles(g);
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
  add_tiles(g, (int32_t)g.probs.size(), M, N, g.policy);
  g.probs.push_back(p);
}

static void sort_tiles(GemmPlan &g) {
  // largest K first for load balance
  std::vector<int64_t> ktot(g.probs.size(), 0);
  for (size_t i = 0; i < g.probs.size(); ++i)
    for (int s = 0; s < g.probs[i].nseg; ++s) ktot[i] += g.segs[g.probs[i].seg0 + s].K;
  for (int c = 0; c < kNumCfg; ++c)
    std::stable_sort(g.tiles[c].begin(), g.tiles[c].end(), [&](const GTile &x, const GTile &y) {
      return ktot[x.prob] > ktot[y.prob];
    });
}

void gemm_finalize(GemmPlan &g) {
  sort_tiles(g);
  g.upload();
}

void gemm_upload(GemmPlan &g) { g.upload(); }

void gemm_keep_upper(GemmPlan &g) {
  for (int c = 0; c < kNumCfg; ++c) {
    auto &t = g.tiles[c];
    t.erase(std::remove_if(t.begin(), t.end(),
                           [&](const GTile &x) { return x.m0 > x.n0 + kCfgBN[c] - 1; }),
            t.end());
    g.ctx->free(g.d_tiles[c]);
    g.d_tiles[c] = upload_vec(g.ctx, t);
  }
  g.ctx->sync();
}

void gemm_retile(GemmPlan &g, int policy) {
  if (policy == g.policy) return;
  g.policy = policy;
  for (auto &t : g.tiles) t.clear();
  for (size_t p = 0; p < g.probs.size(); ++p)
    add_tiles(g, (int32_t)p, g.probs[p].M, g.probs[p].N, policy);
  sort_tiles(g);
  for (int c = 0; c < kNumCfg; ++c) {
    g.ctx->free(g.d_tiles[c]);
    g.d_tiles[c] = upload_vec(g.ctx, g.tiles[c]);
  }
  g.ctx->sync();
}

TensorPtr contract_struct(const BTensor &A, const BTensor &B, const std::vector<int> &ca,
                          const std::vector<int> &cb, const std::vector<int> &fa,
                          const std::vector<int> &fb) {
  UDMRG_REQUIRE(ca.size() == cb.size(), "contract: axis lists differ in length");
  UDMRG_REQUIRE(fa.size() + ca.size() == (size_t)A.rank(), "contract: bad A axes");
  UDMRG_REQUIRE(fb.size() + cb.size() == (size_t)B.rank(), "contract: bad B axes");
  auto out = std::make_unique<BTensor>();
  out->ctx = A.ctx;
  out->dtype = A.dtype;
  out->nq = A.nq;
  for (int i : fa) out->idx.push_back(A.idx[i]);
  for (int i : fb) out->idx.push_back(B.idx[i]);
  const int ro = out->rank();
  UDMRG_REQUIRE(ro > 0 && ro <= kMaxRank, "contract: output rank");
  for (const BTensor *T : {&A, &B})
    for (const Index &ix : T->idx)
      UDMRG_REQUIRE(ix.nsec() < 65536, "contract: more than 65535 sectors on one index");
  // B's distinct (contracted key, free key) pairs, grouped by contracted key
  std::vector<std::pair<uint64_t, Key128>> bk;
  bk.reserve(B.nblocks());
  for (int64_t b = 0; b < B.nblocks(); ++b) {
    uint64_t k = 0;
    for (int ax : cb) k = (k << 16) | (uint64_t)B.key(b)[ax];
    Key128 f = 0;
    for (int ax : fb) f = (f << 16) | (Key128)B.key(b)[ax];
    bk.push_back({k, f});
  }
  std::sort(bk.begin(), bk.end());
  bk.erase(std::unique(bk.begin(), bk.end()), bk.end());
  std::vector<Key128> keys;
  for (int64_t a = 0; a < A.nblocks(); ++a) {
    uint64_t k = 0;
    for (int ax : ca) k = (k << 16) | (uint64_t)A.key(a)[ax];
    Key128 ka = 0;
    for (int ax : fa) ka = (ka << 16) | (Key128)A.key(a)[ax];
    if (!fb.empty()) ka = fa.empty() ? 0 : ka << (16 * fb.size());
    auto it = std::lower_bound(bk.begin(), bk.end(), std::make_pair(k, (Key128)0));
    for (; it != bk.end() && it->first == k; ++it) keys.push_back(ka | it->second);
  }
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  std::vector<int32_t> flat(keys.size() * ro);
  for (size_t o = 0; o < keys.size(); ++o) {
    Key128 ok = keys[o];
    for (int j = ro - 1; j >= 0; --j) {
      flat[o * ro + j] = (int32_t)(uint32_t)(ok & 0xFFFF);
      ok >>= 16;
    }
  }
  out->set_blocks(flat);
  return out;
}

std::unique_ptr<ContractPlan> plan_contract(const BTensor &A, const BTensor &B,
                                            const std::vector<int> &ca, const std::vector<int> &cb,
                                            const std::vector<int> &fa,
                                            const std::vector<int> &fb, bool upload) {
  return plan_impl(A, B, ca, cb, fa, fb, nullptr, nullptr, upload);
}

std::unique_ptr<ContractPlan> plan_contract_into(const BTensor &A, const BTensor &B,
                                                 const std::vector<int> &ca,
                                                 const std::vector<int> &cb,
                                                 const std::vector<int> &fa,
                                                 const std::vector<int> &fb, const BTensor &dst,
                                                 std::vector<int64_t> *missing, bool upload) {
  return plan_impl(A, B, ca, cb, fa, fb, &dst, missing, upload);
}

std::unique_ptr<ContractPlan> plan_contract_axes(const BTensor &A, const BTensor &B,
                                                 const std::vector<int> &ca,
                                                 const std::vector<int> &cb, bool upload) {
  std::vector<int> fa, fb;
  for (int i = 0; i < A.rank(); ++i)
    if (std::find(ca.begin(), ca.end(), i) == ca.end()) fa.push_back(i);
  for (int i = 0; i < B.rank(); ++i)
    if (std::find(cb.begin(), cb.end(), i) == cb.end()) fb.push_back(i);
  return plan_contract(A, B, ca, cb, fa, fb, upload);
}

std::unique_ptr<ContractPlan> plan_contract_cyclic(const BTensor &A, const BTensor &B, int a_start,
                                                   int b_start, int n, bool upload) {
  std::vector<int> ca, cb, fa, fb;
  cyclic_axes(A.rank(), B.rank(), a_start, b_start, n, ca, cb, fa, fb);
  return plan_contract(A, B, ca, cb, fa, fb, upload);
}

TensorPtr run_contract(Ctx &ctx, const ContractPlan &plan, const BTensor &A, const BTensor &B,
                       bool dw) {
  auto out = plan.out->clone_struct();
  out->alloc_data();
  (dw ? run_gemm_dw : run_gemm)(ctx, plan.gemm, A.dtype, A.data, B.data, out->data, 1.0, 0.0);
  return out;
}

}  // namespace udmrg
