#include "sg_matvec.hpp"

#include <algorithm>
#include <array>
#include <chrono>
#include <map>
#include <unordered_map>

namespace udmrg {

SgMatvecPlan::~SgMatvecPlan() {
  if (!ctx) return;
  for (void *p : {(void *)l_img, (void *)psi_img, (void *)t3_img, (void *)r_img, (void *)t1,
                  (void *)d_pairs, (void *)d_outs, (void *)d_rowptr, (void *)d_nz,
                  (void *)d_tasks, (void *)d_gmap, (void *)d_rowinfo, (void *)d_kchunks,
                  (void *)d_tgtref})
    ctx->free(p);
}

namespace {

template <typename V>
V *upload_vec(Ctx &ctx, const std::vector<V> &v) {
  if (v.empty()) return nullptr;
  V *d = (V *)ctx.alloc(v.size() * sizeof(V));
  UDMRG_CHECK_CUDA(
      cudaMemcpyAsync(d, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, ctx.stream));
  return d;
}

using Key = std::array<int32_t, 5>;  // (A', W, S1, S2, B)
struct T1KeyHash {
  size_t operator()(const Key &k) const {
    uint64_t h = 0x9e3779b97f4a7c15ull;
    for (int32_t v : k) h = (h ^ (uint32_t)v) * 0x100000001b3ull + (h >> 29);
    return (size_t)h;
  }
};

struct T1Block {
  int64_t origin;  // element offset of (a'=0, w=0, s1=s2=0, b=0)
  int64_t im;      // offset of the imaginary half (complex data)
  int64_t pitch;
  int32_t dw, ds12;
  int32_t bstride;  // columns per (s1, s2): db rounded up to 8
};

inline int64_t up8(int64_t x) { return (x + 7) & ~(int64_t)7; }

}  // namespace

std::unique_ptr<SgMatvecPlan> plan_sg_tables(const BTensor &L, const BTensor &R, const BTensor &S,
                                             FusedMpo &fm, int bn1, int bn3) {
  UDMRG_REQUIRE((bn1 == 64 || bn1 == 128) && (bn3 == 64 || bn3 == 128),
                "mixed matvec: B tiles of 64 or 128 rows");
  const auto tstart = std::chrono::steady_clock::now();
  // complex L, R, psi: the real embedding [[Re, -Im], [Im, Re]] (the MPO
  // coefficients are real, see FusedMpo)
  const bool cplx = S.dtype == kC128;
  UDMRG_REQUIRE(L.dtype == S.dtype && R.dtype == S.dtype,
                "mixed matvec: L, R and psi must share the element type");
  const int64_t es = cplx ? 2 : 1;  // doubles per element
  auto p = std::make_unique<SgMatvecPlan>();
  p->psi_size = S.size();
  p->cplx = cplx;
  p->bn1 = bn1;
  p->bn3 = bn3;
  p->g1.bn = bn1;
  p->g3.bn = bn3;
  // pack a block (or its real / imaginary part) of a tensor with element
  // offset `off`, row and column strides in elements
  auto add_pack = [&](std::vector<PackOp> &ops, int64_t off, int64_t rs, int64_t cs,
                      int64_t img_off, int64_t rows, int64_t cols, int64_t r0, int64_t k0,
                      int32_t kc, int32_t tr, int part, bool neg) {
    PackOp op{};
    op.src_off = off * es + (part == 1 ? 1 : 0);
    op.src_rs = rs * es;
    op.src_cs = cs * es;
    op.img_off = img_off;
    op.rows = (int32_t)rows;
    op.cols = (int32_t)cols;
    op.r0 = (int32_t)r0;
    op.k0 = (int32_t)k0;
    op.kc = kc;
    op.tr = tr;
    op.neg = neg ? 1 : 0;
    ops.push_back(op);
  };
  auto dim = [](const BTensor &t, int64_t b, int ax) { return t.idx[ax].dims[t.key(b)[ax]]; };

  // ---------------- step 1 groups: one per ket sector A ----------------------
  const int nA = L.idx[2].nsec();
  std::vector<std::vector<int64_t>> lrows(nA), pcols(nA);
  for (int64_t b = 0; b < L.nblocks(); ++b) lrows[L.key(b)[2]].push_back(b);
  for (int64_t b = 0; b < S.nblocks(); ++b) pcols[S.key(b)[0]].push_back(b);
  std::unordered_map<Key, T1Block, T1KeyHash> t1map;  // (A', W, S1, S2, B) -> location in T1
  {
    size_t n = 0;
    for (int A = 0; A < nA; ++A) n += lrows[A].size() * pcols[A].size();
    t1map.reserve(n);
  }
  std::vector<PackOp> &lops = p->l_ops;
  int64_t t1tot = 0, lbytes = 0, pbytes = 0;
  struct G1 {
    int A;
    int64_t M, N, K, t1_off, l_off, p_off;
    int64_t Np;  // T1 row pitch (N, a multiple of 8: 32-byte aligned rows)
    int64_t Kh;  // K rounded up to 8: first K column of the imaginary half
    int64_t Me, Ke;  // embedded GEMM shape (2M x 2Kh for complex data)
  };
  std::vector<G1> g1s;
  for (int A = 0; A < nA; ++A) {
    if (lrows[A].empty() || pcols[A].empty()) continue;
    G1 g{A, 0, 0, L.idx[2].dims[A], t1tot, lbytes, pbytes, 0, 0, 0, 0};
    std::vector<int64_t> rof, cof;
    for (int64_t b : lrows[A]) {
      rof.push_back(g.M);
      g.M += dim(L, b, 0) * dim(L, b, 1);
    }
    for (int64_t b : pcols[A]) {  // columns (s1, s2, b), each b run padded to 8
      cof.push_back(g.N);
      g.N += dim(S, b, 1) * dim(S, b, 2) * up8(dim(S, b, 3));
    }
    UDMRG_REQUIRE(g.M < (1 << 30) && g.N < (1 << 30) && g.K < (1 << 30), "mixed matvec: group too large");
    g.Np = g.N;
    g.Kh = up8(g.K);
    g.Me = es * g.M;
    g.Ke = cplx ? 2 * g.Kh : g.K;
    const int32_t kc = (int32_t)((g.Ke + kTcBK - 1) / kTcBK);
    for (size_t i = 0; i < lrows[A].size(); ++i) {
      const int64_t b = lrows[A][i], nr = dim(L, b, 0) * dim(L, b, 1);
      // real rows [Lr | -Li], imaginary rows [Li | Lr]
      add_pack(lops, L.offs[b], g.K, 1, g.l_off, nr, g.K, rof[i], 0, kc, kTcBM, 0, false);
      if (cplx) {
        add_pack(lops, L.offs[b], g.K, 1, g.l_off, nr, g.K, rof[i], g.Kh, kc, kTcBM, 1, true);
        add_pack(lops, L.offs[b], g.K, 1, g.l_off, nr, g.K, g.M + rof[i], 0, kc, kTcBM, 1,
                 false);
        add_pack(lops, L.offs[b], g.K, 1, g.l_off, nr, g.K, g.M + rof[i], g.Kh, kc, kTcBM, 0,
                 false);
      }
    }
    for (size_t j = 0; j < pcols[A].size(); ++j) {
      const int64_t b = pcols[A][j];
      const int64_t ds12 = dim(S, b, 1) * dim(S, b, 2), db = dim(S, b, 3);
      const int64_t ncol = ds12 * db;
      // one op per (s1, s2): the b run lands at its padded column; K range
      // [psi_r; psi_i]
      for (int64_t q = 0; q < ds12; ++q) {
        add_pack(p->psi_pack.ops, S.offs[b] + q * db, 1, ncol, g.p_off, db, g.K,
                 cof[j] + q * up8(db), 0, kc, bn1, 0, false);
        if (cplx)
          add_pack(p->psi_pack.ops, S.offs[b] + q * db, 1, ncol, g.p_off, db, g.K,
                   cof[j] + q * up8(db), g.Kh, kc, bn1, 1, false);
      }
    }
    // T1 block locations
    for (size_t i = 0; i < lrows[A].size(); ++i) {
      const int64_t lb = lrows[A][i];
      for (size_t j = 0; j < pcols[A].size(); ++j) {
        const int64_t pb = pcols[A][j];
        Key k = {L.key(lb)[0], L.key(lb)[1], S.key(pb)[1], S.key(pb)[2], S.key(pb)[3]};
        T1Block t;
        t.origin = g.t1_off + rof[i] * g.Np + cof[j];
        t.im = cplx ? g.M * g.Np : 0;  // the imaginary half of the group's rows
        t.pitch = g.Np;
        t.dw = (int32_t)dim(L, lb, 1);
        t.ds12 = (int32_t)(dim(S, pb, 1) * dim(S, pb, 2));
        t.bstride = (int32_t)up8(dim(S, pb, 3));
        t1map[k] = t;
      }
    }
    t1tot += g.Me * g.Np;
    lbytes += tc_image_bytes(g.Me, g.Ke, kTcBM);
    pbytes += tc_image_bytes(g.N, g.Ke, bn1);
    g1s.push_back(g);
  }
  p->t1_size = t1tot;
  p->l_bytes = lbytes;
  p->psi_bytes = pbytes;

  // ---------------- step 3 groups: one per bra sector B' of R -----------------
  const int nB = R.idx[0].nsec();
  std::vector<std::vector<int64_t>> rks(nB), orows(nB);
  for (int64_t b = 0; b < R.nblocks(); ++b) rks[R.key(b)[0]].push_back(b);
  for (int64_t b = 0; b < S.nblocks(); ++b) orows[S.key(b)[3]].push_back(b);
  std::vector<PackOp> &rops = p->r_ops;
  int64_t t3bytes = 0, rbytes = 0;
  std::vector<std::pair<int32_t, int32_t>> tgt_key;  // (A', B) of every target
  // fused form: the group (its MpoGroupMap), row block and K block of every target
  struct TgtLoc {
    int32_t g, i, j;
  };
  std::vector<TgtLoc> tgt_loc;
  for (int Bp = 0; Bp < nB; ++Bp) {
    if (orows[Bp].empty()) continue;
    const int64_t dBp = R.idx[0].dims[Bp];
    int64_t M = 0, K = 0;
    std::vector<int64_t> rof, kof;
    for (int64_t b : orows[Bp]) {
      rof.push_back(M);
      M += dim(S, b, 0) * dim(S, b, 1) * dim(S, b, 2);
    }
    for (int64_t b : rks[Bp]) {  // columns (w2, b), each b run padded to 8
      kof.push_back(K);
      K += dim(R, b, 1) * up8(dim(R, b, 2));
    }
    UDMRG_REQUIRE(M < (1 << 30) && K < (1 << 30), "mixed matvec: group too large");
    const int64_t Ke = es * K, Ne = es * dBp;  // embedded shape: M x 2K times (2 dB') x 2K
    const int32_t kc = (int32_t)((Ke + kTcBK - 1) / kTcBK);
    const int64_t t3_off = t3bytes, r_off = rbytes;
    std::vector<int64_t> rows(M);  // output row addresses in doubles
    for (size_t i = 0; i < orows[Bp].size(); ++i) {
      const int64_t b = orows[Bp][i];
      const int64_t nr = dim(S, b, 0) * dim(S, b, 1) * dim(S, b, 2);
      for (int64_t m = 0; m < nr; ++m) rows[rof[i] + m] = (S.offs[b] + m * dBp) * es;
    }
    for (size_t j = 0; j < rks[Bp].size(); ++j) {
      const int64_t b = rks[Bp][j], dw2 = dim(R, b, 1), db = dim(R, b, 2), nc = dw2 * db;
      // B rows: [Rr | -Ri] (real output columns), [Ri | Rr] (imaginary); one
      // op per w2 (the b run at its padded column)
      for (int64_t w2 = 0; w2 < dw2; ++w2) {
        const int64_t off = R.offs[b] + w2 * db, k0 = kof[j] + w2 * up8(db);
        add_pack(rops, off, nc, 1, r_off, dBp, db, 0, k0, kc, bn3, 0, false);
        if (cplx) {
          add_pack(rops, off, nc, 1, r_off, dBp, db, 0, K + k0, kc, bn3, 1, true);
          add_pack(rops, off, nc, 1, r_off, dBp, db, dBp, k0, kc, bn3, 1, false);
          add_pack(rops, off, nc, 1, r_off, dBp, db, dBp, K + k0, kc, bn3, 0, false);
        }
      }
    }
    // fused form: per-row (row block, a', s1's2') and per-K-chunk (K block,
    // w2, b offset, half) tables of the group, in image order
    {
      MpoGroupMap gm{};
      gm.row0 = (int64_t)p->rowinfo.size();
      gm.kch0 = (int64_t)p->kchunks.size();
      gm.tgt0 = (int64_t)p->tgtref.size();
      gm.nrb = (int32_t)orows[Bp].size();
      gm.nkb = (int32_t)rks[Bp].size();
      for (size_t i = 0; i < orows[Bp].size(); ++i) {
        const int64_t b = orows[Bp][i];
        const int32_t da = (int32_t)dim(S, b, 0);
        const int32_t ds12p = (int32_t)(dim(S, b, 1) * dim(S, b, 2));
        for (int32_t a = 0; a < da; ++a)
          for (int32_t q = 0; q < ds12p; ++q) p->rowinfo.push_back({(int32_t)i, a, q, 0});
      }
      for (int32_t half = 0; half < (cplx ? 2 : 1); ++half)
        for (size_t j = 0; j < rks[Bp].size(); ++j) {
          const int64_t b = rks[Bp][j];
          const int32_t dw2 = (int32_t)dim(R, b, 1), dbp = (int32_t)up8(dim(R, b, 2));
          for (int32_t w2 = 0; w2 < dw2; ++w2)
            for (int32_t c8 = 0; c8 < dbp; c8 += 8) p->kchunks.push_back({(int32_t)j, w2, c8, half});
        }
      gm.nkch = (int32_t)(p->kchunks.size() - gm.kch0);
      UDMRG_REQUIRE((int64_t)gm.nkch * 8 == Ke, "mixed matvec: K chunk table");
      p->tgtref.resize(p->tgtref.size() + (size_t)(cplx ? 2 : 1) * gm.nrb * gm.nkb, {-1, 0});
      p->gmap.push_back(gm);
    }
    // MPO-step targets of this group
    for (size_t i = 0; i < orows[Bp].size(); ++i) {
      const int64_t ob = orows[Bp][i];
      const int32_t Ap = S.key(ob)[0], S1p = S.key(ob)[1], S2p = S.key(ob)[2];
      const int32_t da = (int32_t)dim(S, ob, 0);
      const int32_t ds1p = (int32_t)dim(S, ob, 1), ds2p = (int32_t)dim(S, ob, 2);
      for (size_t j = 0; j < rks[Bp].size(); ++j) {
        const int64_t rb = rks[Bp][j];
        const int32_t W2s = R.key(rb)[1], Bs = R.key(rb)[2];
        const int32_t dw2 = (int32_t)dim(R, rb, 1), db = (int32_t)dim(R, rb, 2);
        MpoTarget tg{};
        tg.img_off = t3_off;
        tg.row0 = (int32_t)rof[i];
        tg.k0 = (int32_t)kof[j];
        tg.kc = kc;
        tg.da = da;
        tg.db = db;
        tg.dbp = (int32_t)up8(db);
        tg.ds12p = ds1p * ds2p;
        tg.dw2 = dw2;
        tg.nout = tg.ds12p * dw2;
        tg.kim = (int32_t)K;  // imaginary half of the image columns
        tg.src0 = (int32_t)p->sources.size();
        // sources: T1 blocks (A', W, S1, S2, B) through W1 (W,S1,S1p,Wr) W2 (Wr,S2,S2p,W2s);
        // the fused coefficients depend on the MPO sectors only (cached in fm)
        for (const FusedMpo::Entry &ce : fm.get(S1p, S2p, W2s)) {
          auto tb = t1map.find(Key{Ap, ce.src[0], ce.src[1], ce.src[2], Bs});
          if (tb == t1map.end()) continue;
          MpoSource s{};
          s.t1_off = tb->second.origin;
          s.t1_im = tb->second.im;
          s.row_pitch = tb->second.pitch;
          s.dw = tb->second.dw;
          s.ds12 = tb->second.ds12;
          s.bstride = tb->second.bstride;
          s.coef_off = (int32_t)p->coefs.size();
          for (double v : ce.coef) p->coefs.push_back((float)v);
          p->sources.push_back(s);
        }
        tg.nsrc = (int32_t)p->sources.size() - tg.src0;
        if (tg.nsrc > 0) {
          p->targets.push_back(tg);
          tgt_key.push_back({Ap, Bs});
          tgt_loc.push_back({(int32_t)p->gmap.size() - 1, (int32_t)i, (int32_t)j});
        }
      }
    }
    p->g3.add_group(t3_off, r_off, (int32_t)M, (int32_t)Ne, (int32_t)Ke, rows);
    t3bytes += tc_image_bytes(M, Ke, kTcBM);
    rbytes += tc_image_bytes(Ne, Ke, bn3);
  }
  p->t3_bytes = t3bytes;
  p->r_bytes = rbytes;

  for (auto &g : g1s) {
    std::vector<int64_t> rows(g.Me);
    for (int64_t m = 0; m < g.Me; ++m) rows[m] = g.t1_off + m * g.Np;
    p->g1.add_group(g.l_off, g.p_off, (int32_t)g.Me, (int32_t)g.N, (int32_t)g.Ke, rows);
  }
  // ---------------- MPO step regrouped by (A', B) pair ------------------------
  {
    // targets by (A', B) pair, pairs ascending, targets in plan order
    std::vector<std::pair<std::pair<int32_t, int32_t>, std::vector<int>>> by_pair;
    {
      std::vector<int> ord(p->targets.size());
      for (size_t t = 0; t < ord.size(); ++t) ord[t] = (int)t;
      std::stable_sort(ord.begin(), ord.end(),
                       [&](int x, int y) { return tgt_key[x] < tgt_key[y]; });
      for (int t : ord) {
        if (by_pair.empty() || by_pair.back().first != tgt_key[t])
          by_pair.push_back({tgt_key[t], {}});
        by_pair.back().second.push_back(t);
      }
    }
    // per pair: its input channels' T1 locations (real part), output channels
    // and coefficient nonzeros (o, i, v); the imaginary twin of a complex pair
    // shifts the inputs by the group's real row count and the outputs by the
    // image's real K
    struct PairNz {
      int32_t o, i;
      float v;
    };
    struct Built {
      MpoPair pr;
      std::vector<int64_t> in_im;
      std::vector<int32_t> out_im;
      std::vector<PairNz> nzs;  // sorted by output channel
    };
    std::vector<Built> built;
    // fused form: the (real) pair of every target and its first output channel there
    std::vector<int32_t> tgt_pair(p->targets.size(), -1), tgt_out(p->targets.size(), 0);
    for (auto &kv : by_pair) {
      Built bd{};
      MpoPair &pr = bd.pr;
      pr.in0 = (int32_t)p->ins.size();
      pr.out0 = (int32_t)p->outs.size();
      const MpoTarget &t0 = p->targets[kv.second[0]];
      pr.da = t0.da;
      pr.db = t0.db;
      pr.dbp = t0.dbp;
      // input channels: one per (w, s1 s2) of every distinct source block
      // T1 origin -> first channel (a pair has few source blocks)
      std::vector<std::pair<int64_t, int32_t>> in_first;
      auto first_of = [&](int64_t off) {
        for (const auto &f : in_first)
          if (f.first == off) return f.second;
        return -1;
      };
      for (int t : kv.second) {
        const MpoTarget &tg = p->targets[t];
        for (int s = 0; s < tg.nsrc; ++s) {
          const MpoSource &sr = p->sources[tg.src0 + s];
          if (first_of(sr.t1_off) >= 0) continue;
          in_first.push_back({sr.t1_off, (int32_t)(p->ins.size() - pr.in0)});
          for (int w = 0; w < sr.dw; ++w)
            for (int s12 = 0; s12 < sr.ds12; ++s12) {
              p->ins.push_back({sr.t1_off + (int64_t)w * sr.row_pitch + (int64_t)s12 * sr.bstride,
                                (int64_t)sr.dw * sr.row_pitch});
              bd.in_im.push_back(sr.t1_im);
            }
        }
      }
      pr.nin = (int32_t)p->ins.size() - pr.in0;
      // output channels: one per (s1' s2', w2) of every target block
      std::vector<int32_t> out_first;
      for (int t : kv.second) {
        const MpoTarget &tg = p->targets[t];
        out_first.push_back((int32_t)(p->outs.size() - pr.out0));
        tgt_pair[t] = (int32_t)built.size();
        tgt_out[t] = out_first.back();
        for (int oc = 0; oc < tg.nout; ++oc) {
          p->outs.push_back({tg.img_off, tg.row0 + oc / tg.dw2, tg.ds12p,
                             tg.k0 + (oc % tg.dw2) * tg.dbp, tg.kc});
          bd.out_im.push_back(tg.kim);
        }
      }
      pr.nout = (int32_t)p->outs.size() - pr.out0;
      UDMRG_REQUIRE(pr.nin <= 256 && pr.nout <= 256,
                    "mixed matvec: more than 256 MPO channels in one sector pair");
      std::vector<float> C((size_t)pr.nout * pr.nin, 0.f);
      for (size_t j = 0; j < kv.second.size(); ++j) {
        const MpoTarget &tg = p->targets[kv.second[j]];
        for (int s = 0; s < tg.nsrc; ++s) {
          const MpoSource &sr = p->sources[tg.src0 + s];
          const int i0 = first_of(sr.t1_off);
          const int nin_s = sr.dw * sr.ds12;
          for (int ic = 0; ic < nin_s; ++ic)
            for (int oc = 0; oc < tg.nout; ++oc)
              C[(size_t)(out_first[j] + oc) * pr.nin + i0 + ic] +=
                  p->coefs[sr.coef_off + ic * tg.nout + oc];
        }
      }
      for (int o = 0; o < pr.nout; ++o)
        for (int i = 0; i < pr.nin; ++i) {
          const float v = C[(size_t)o * pr.nin + i];
          if (v != 0.f) bd.nzs.push_back({o, i, v});
        }
      p->max_nin = std::max(p->max_nin, (int)pr.nin);
      p->max_nout = std::max(p->max_nout, (int)pr.nout);
      built.push_back(std::move(bd));
    }
    // emit the pairs (the imaginary twins after all real pairs): CSR rows
    // and nonzero records with their inputs' T1 locations
    if (p->rowptr.empty()) p->rowptr.push_back(0);
    auto emit = [&](const Built &bd, bool imag) {
      MpoPair pr = bd.pr;
      if (imag) {
        const int32_t out0 = (int32_t)p->outs.size();
        for (int o = 0; o < pr.nout; ++o) {
          MpoOut ot = p->outs[pr.out0 + o];
          ot.col0 += bd.out_im[o];
          p->outs.push_back(ot);
        }
        pr.out0 = out0;
      }
      pr.row0 = (int32_t)p->rowptr.size() - 1;
      size_t k = 0;
      for (int o = 0; o < pr.nout; ++o) {
        for (; k < bd.nzs.size() && bd.nzs[k].o == o; ++k) {
          const MpoIn &in = p->ins[pr.in0 + bd.nzs[k].i];
          const int64_t base = in.base + (imag ? bd.in_im[bd.nzs[k].i] : 0);
          UDMRG_REQUIRE(in.astride < (1LL << 31) && base % 8 == 0 && in.astride % 8 == 0,
                        "mixed matvec: MPO-step input not 32-byte aligned");
          p->nz.push_back({base, (int32_t)in.astride, bd.nzs[k].v});
        }
        p->rowptr.push_back((int32_t)p->nz.size());
      }
      for (int o = 0; o < pr.nout; ++o)
        UDMRG_REQUIRE(p->outs[pr.out0 + o].col0 % 8 == 0,
                      "mixed matvec: MPO-step output not 16-byte aligned");
      p->mpo_bytes += (double)pr.da * pr.db * (4.0 * pr.nin + 6.0 * pr.nout);
      p->t1_read_bytes += (double)pr.da * pr.db * 4.0 * pr.nin;
      p->pairs.push_back(pr);
    };
    for (const Built &bd : built) emit(bd, false);
    if (cplx)
      for (const Built &bd : built) emit(bd, true);
    // fused form: the CSR row of output channel 0 of every target (its
    // imaginary twin's for the imaginary half)
    const int32_t nreal = (int32_t)built.size();
    for (size_t t = 0; t < p->targets.size(); ++t) {
      const TgtLoc &lc = tgt_loc[t];
      const MpoGroupMap &gm = p->gmap[lc.g];
      const int32_t q = tgt_pair[t];
      p->tgtref[gm.tgt0 + (int64_t)lc.i * gm.nkb + lc.j] = {p->pairs[q].row0 + tgt_out[t],
                                                             p->targets[t].dw2};
      if (cplx)
        p->tgtref[gm.tgt0 + ((int64_t)gm.nrb + lc.i) * gm.nkb + lc.j] = {
            p->pairs[nreal + q].row0 + tgt_out[t], p->targets[t].dw2};
    }
    // warp tasks: 32 units (a', 8-wide chunk of b) each, the pairs with the
    // most work per unit (nonzeros and output channels) first
    std::vector<int> order(p->pairs.size());
    for (size_t q = 0; q < order.size(); ++q) order[q] = (int)q;
    auto cost = [&](int q) {
      const MpoPair &pr = p->pairs[q];
      return 2 * (p->rowptr[pr.row0 + pr.nout] - p->rowptr[pr.row0]) + 3 * pr.nout;
    };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
    for (int q : order) {
      const MpoPair &pr = p->pairs[q];
      const int64_t units = (int64_t)pr.da * (pr.dbp / 8);
      UDMRG_REQUIRE(units < (1LL << 31), "mixed matvec: sector pair too large");
      for (int64_t u0 = 0; u0 < units; u0 += 32) p->tasks.push_back({q, (int32_t)u0});
    }
  }
  p->host_sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - tstart).count();
  return p;
}

void plan_sg_device(Ctx &ctx, SgMatvecPlan &plan, const BTensor &L, const BTensor &R) {
  const auto tstart = std::chrono::steady_clock::now();
  SgMatvecPlan *p = &plan;
  p->ctx = &ctx;
  p->g1.ctx = &ctx;
  p->g3.ctx = &ctx;
  auto zalloc = [&](int64_t bytes) {
    uint8_t *d = (uint8_t *)ctx.alloc(std::max<int64_t>(bytes, 256));
    UDMRG_CHECK_CUDA(cudaMemsetAsync(d, 0, std::max<int64_t>(bytes, 256), ctx.stream));
    return d;
  };
  p->l_img = zalloc(p->l_bytes);
  p->psi_img = zalloc(p->psi_bytes);
  p->t3_img = zalloc(p->t3_bytes);
  p->r_img = zalloc(p->r_bytes);
  p->t1 = (float *)ctx.alloc(std::max<int64_t>(p->t1_size, 1) * sizeof(float));
  run_pack(ctx, p->l_ops, L.data, true, p->l_img);
  run_pack(ctx, p->r_ops, R.data, true, p->r_img);
  p->psi_pack.upload(ctx);
  p->g1.finalize();
  p->g3.finalize();
  p->d_pairs = upload_vec(ctx, p->pairs);
  p->d_outs = upload_vec(ctx, p->outs);
  p->d_rowptr = upload_vec(ctx, p->rowptr);
  p->d_nz = upload_vec(ctx, p->nz);
  p->d_tasks = upload_vec(ctx, p->tasks);
  p->d_gmap = upload_vec(ctx, p->gmap);
  p->d_rowinfo = upload_vec(ctx, p->rowinfo);
  p->d_kchunks = upload_vec(ctx, p->kchunks);
  p->d_tgtref = upload_vec(ctx, p->tgtref);
  p->mixed_flops = 6.0 * (p->g1.flops + p->g3.flops);
  ctx.sync();
  std::vector<PackOp>().swap(p->l_ops);  // packed; the host copies go
  std::vector<PackOp>().swap(p->r_ops);
  p->dev_sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - tstart).count();
}

std::unique_ptr<SgMatvecPlan> plan_sg_matvec(Ctx &ctx, const BTensor &L, const BTensor &R,
                                             const BTensor &S, FusedMpo &fm, int bn1, int bn3) {
  auto p = plan_sg_tables(L, R, S, fm, bn1, bn3);
  plan_sg_device(ctx, *p, L, R);
  return p;
}

std::array<int64_t, 3> sg_shape_class(const BTensor &S) {
  auto lg2 = [](int64_t x) {
    int64_t k = 0;
    while ((int64_t(1) << k) < x) ++k;
    return k;
  };
  int64_t maxb = 1;
  for (int64_t d : S.idx[3].dims) maxb = std::max(maxb, d);
  return {S.dtype == kC128 ? 1 : 0, lg2(S.size()), lg2(maxb)};
}

bool sg_tiles_known(const Ctx &ctx, const BTensor &S, int *bn1, int *bn3) {
  if (ctx.tc_bn1 && ctx.tc_bn3) {
    *bn1 = ctx.tc_bn1;
    *bn3 = ctx.tc_bn3;
    return true;
  }
  auto it = ctx.tc_tuned.find(sg_shape_class(S));
  if (it == ctx.tc_tuned.end()) return false;
  *bn1 = it->second[0];
  *bn3 = it->second[1];
  return true;
}

std::unique_ptr<SgMatvecPlan> plan_sg_matvec_tuned(Ctx &ctx, const BTensor &L, const BTensor &R,
                                                   const BTensor &S, FusedMpo &fm) {
  if (ctx.tc_bn1 && ctx.tc_bn3) return plan_sg_matvec(ctx, L, R, S, fm, ctx.tc_bn1, ctx.tc_bn3);
  const std::array<int64_t, 3> key = sg_shape_class(S);
  auto it = ctx.tc_tuned.find(key);
  if (it != ctx.tc_tuned.end()) {
    auto p = plan_sg_matvec(ctx, L, R, S, fm, it->second[0], it->second[1]);
    p->tuned = true;
    return p;
  }
  // timed trials: matvecs with each tile choice (input zeros: the kernels'
  // work does not depend on the values), stage by stage
  std::unique_ptr<SgMatvecPlan> cand[2];
  float best[2][4];
  const int64_t nd = S.size() * (S.dtype == kC128 ? 2 : 1);
  DeviceScratch sc(ctx);
  double *x = sc.get<double>(nd), *y = sc.get<double>(nd);
  UDMRG_CHECK_CUDA(cudaMemsetAsync(x, 0, std::max<int64_t>(nd, 1) * sizeof(double), ctx.stream));
  for (int c = 0; c < 2; ++c) cand[c] = plan_sg_matvec(ctx, L, R, S, fm, c == 0 ? 64 : 128,
                                                      c == 0 ? 64 : 128);
  // the two candidates alternate, the best of four per stage (a stage differs
  // between the tiles by a few microseconds, about the spread of one timing)
  for (int rep = 0; rep < 4; ++rep)
    for (int c = 0; c < 2; ++c) {
      float ms[4];
      cand[c]->apply_timed(x, y, ms);
      for (int k = 0; k < 4; ++k) best[c][k] = rep == 0 ? ms[k] : std::min(best[c][k], ms[k]);
    }
  ctx.tc_trials++;
  const int bn1 = best[1][1] < best[0][1] ? 128 : 64;
  const int bn3 = best[1][3] < best[0][3] ? 128 : 64;
  ctx.tc_tuned[key] = {bn1, bn3};
  std::unique_ptr<SgMatvecPlan> p;
  if (bn1 == bn3)
    p = std::move(cand[bn1 == 128 ? 1 : 0]);
  else
    p = plan_sg_matvec(ctx, L, R, S, fm, bn1, bn3);
  p->tuned = true;
  return p;
}

void SgMatvecPlan::apply(const double *psi_in, double *out) {
  run_pack(*ctx, psi_pack, psi_in, true, psi_img);
  run_tc_gemm(*ctx, g1, l_img, psi_img, t1, kTcOutF32, 1.0);
  if (fused) {
    run_tc_mpo_gemm(*ctx, *this, out);
  } else {
    run_mpo_step(*ctx, *this);
    run_tc_gemm(*ctx, g3, t3_img, r_img, out, cplx ? kTcOutC128 : kTcOutF64, 1.0);
  }
}

void SgMatvecPlan::apply_timed(const double *psi_in, double *out, float ms[4]) {
  cudaEvent_t ev[5];
  for (auto &e : ev) UDMRG_CHECK_CUDA(cudaEventCreate(&e));
  cudaEventRecord(ev[0], ctx->stream);
  run_pack(*ctx, psi_pack, psi_in, true, psi_img);
  cudaEventRecord(ev[1], ctx->stream);
  run_tc_gemm(*ctx, g1, l_img, psi_img, t1, kTcOutF32, 1.0);
  cudaEventRecord(ev[2], ctx->stream);
  if (fused) {  // one kernel: its time is stage 3, stage 2 is empty
    cudaEventRecord(ev[3], ctx->stream);
    run_tc_mpo_gemm(*ctx, *this, out);
  } else {
    run_mpo_step(*ctx, *this);
    cudaEventRecord(ev[3], ctx->stream);
    run_tc_gemm(*ctx, g3, t3_img, r_img, out, cplx ? kTcOutC128 : kTcOutF64, 1.0);
  }
  cudaEventRecord(ev[4], ctx->stream);
  UDMRG_CHECK_CUDA(cudaEventSynchronize(ev[4]));
  for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]);
  for (auto &e : ev) cudaEventDestroy(e);
  int st = tc_check(*ctx, g1);
  st |= tc_check(*ctx, g3);
  if (st) throw Error(kErrTimeout, "tcgen05 GEMM: a bounded device wait ran out");
}

}  // namespace udmrg
