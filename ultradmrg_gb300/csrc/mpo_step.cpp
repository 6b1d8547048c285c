#include "mpo_step.hpp"

#include <algorithm>

namespace udmrg {

namespace {

// Host copy of a real tensor, or the real parts of a complex one whose
// imaginary parts are all zero (an MPO made complex by promotion).
std::vector<double> download_data(Ctx &ctx, const BTensor &t) {
  const int es = elem_doubles(t.dtype);
  std::vector<double> h(t.size() * es);
  if (t.size())
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(h.data(), t.data, h.size() * sizeof(double),
                                     cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  if (es == 1) return h;
  std::vector<double> r(t.size());
  for (int64_t i = 0; i < t.size(); ++i) {
    if (h[2 * i + 1] != 0.0)
      throw Error(kErrInvalid,
                  "mixed-precision matvec: MPO with complex coefficients (use the FP64 form)");
    r[i] = h[2 * i];
  }
  return r;
}

template <typename V>
V *upload(Ctx &ctx, const std::vector<V> &v) {
  if (v.empty()) return nullptr;
  V *d = (V *)ctx.alloc(v.size() * sizeof(V));
  UDMRG_CHECK_CUDA(
      cudaMemcpyAsync(d, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, ctx.stream));
  return d;
}

}  // namespace

FusedMpo::FusedMpo(Ctx &ctx, const BTensor &w1, const BTensor &w2) : W1(w1), W2(w2) {
  w1h = download_data(ctx, W1);
  w2h = download_data(ctx, W2);
  for (int64_t b = 0; b < W1.nblocks(); ++b) w1_by_s1o[W1.key(b)[2]].push_back(b);
  for (int64_t b = 0; b < W2.nblocks(); ++b)
    w2_by[{W2.key(b)[0], W2.key(b)[2], W2.key(b)[3]}].push_back(b);
}

const std::vector<FusedMpo::Entry> &FusedMpo::get(int32_t S1p, int32_t S2p, int32_t W2s) {
  const std::array<int32_t, 3> ck = {S1p, S2p, W2s};
  auto cit = cache.find(ck);
  if (cit != cache.end()) return cit->second;
  const int64_t ds1p = W1.idx[2].dims[S1p], ds2p = W2.idx[2].dims[S2p];
  const int64_t dw2 = W2.idx[3].dims[W2s];
  const int64_t nout = ds1p * ds2p * dw2;
  std::map<std::array<int32_t, 3>, std::vector<double>> acc;  // (W, S1, S2) -> coef
  auto it1 = w1_by_s1o.find(S1p);
  if (it1 != w1_by_s1o.end()) {
    for (int64_t b1 : it1->second) {
      const int32_t Ws = W1.key(b1)[0], S1 = W1.key(b1)[1], Wr = W1.key(b1)[3];
      auto it2 = w2_by.find({Wr, S2p, W2s});
      if (it2 == w2_by.end()) continue;
      for (int64_t b2 : it2->second) {
        const int32_t S2 = W2.key(b2)[1];
        const int64_t dw = W1.idx[0].dims[Ws], ds1 = W1.idx[1].dims[S1];
        const int64_t dwr = W1.idx[3].dims[Wr], ds2 = W2.idx[1].dims[S2];
        const int64_t nin = dw * ds1 * ds2;
        auto &c = acc[{Ws, S1, S2}];
        if (c.empty()) c.assign(nin * nout, 0.0);
        // W1(w, s1, s1', wr) W2(wr, s2, s2', w2), blocks row-major
        const double *w1 = w1h.data() + W1.offs[b1];
        const double *w2 = w2h.data() + W2.offs[b2];
        for (int64_t w = 0; w < dw; ++w)
          for (int64_t s1 = 0; s1 < ds1; ++s1)
            for (int64_t s2 = 0; s2 < ds2; ++s2)
              for (int64_t s1o = 0; s1o < ds1p; ++s1o)
                for (int64_t s2o = 0; s2o < ds2p; ++s2o)
                  for (int64_t w2i = 0; w2i < dw2; ++w2i) {
                    double v = 0;
                    for (int64_t wr = 0; wr < dwr; ++wr)
                      v += w1[((w * ds1 + s1) * ds1p + s1o) * dwr + wr] *
                           w2[((wr * ds2 + s2) * ds2p + s2o) * dw2 + w2i];
                    const int64_t ic = (w * ds1 + s1) * ds2 + s2;
                    const int64_t oc = (s1o * ds2p + s2o) * dw2 + w2i;
                    c[ic * nout + oc] += v;
                  }
      }
    }
  }
  std::vector<Entry> entries;
  for (auto &kv : acc) {
    bool nz = false;
    for (double v : kv.second) nz |= (v != 0.0);
    if (nz) entries.push_back({kv.first, std::move(kv.second)});
  }
  return cache.emplace(ck, std::move(entries)).first->second;
}

MpoStep64::~MpoStep64() {
  if (!ctx) return;
  for (void *p : {(void *)d_pairs, (void *)d_ins, (void *)d_outs, (void *)d_rowptr, (void *)d_nz,
                  (void *)d_unit0, (void *)d_unit_pair})
    ctx->free(p);
}

std::unique_ptr<MpoStep64> build_mpo_step64(FusedMpo &fm, const BTensor &T1, const BTensor &T3) {
  UDMRG_REQUIRE(T1.rank() == 5 && T3.rank() == 5, "MPO step: rank-5 intermediates expected");
  auto p = std::make_unique<MpoStep64>();
  // T1 blocks by key (A', W, S1, S2, B)
  std::map<std::array<int32_t, 5>, int64_t> t1blk;
  for (int64_t b = 0; b < T1.nblocks(); ++b) {
    const int32_t *k = T1.key(b);
    t1blk[{k[0], k[1], k[2], k[3], k[4]}] = b;
  }
  // T3 blocks (B, A', S1', S2', W2) grouped by (A', B)
  std::map<std::pair<int32_t, int32_t>, std::vector<int64_t>> by_pair;
  for (int64_t b = 0; b < T3.nblocks(); ++b) by_pair[{T3.key(b)[1], T3.key(b)[0]}].push_back(b);
  p->rowptr.push_back(0);
  p->unit0.push_back(0);
  for (auto &kv : by_pair) {
    const int32_t Ap = kv.first.first, Bs = kv.first.second;
    MpoPair64 pr{};
    pr.in0 = (int32_t)p->ins.size();
    pr.out0 = (int32_t)p->outs.size();
    pr.row0 = (int32_t)(p->rowptr.size() - 1);
    pr.da = (int32_t)T3.idx[1].dims[Ap];
    pr.db = (int32_t)T3.idx[0].dims[Bs];
    std::map<int64_t, int32_t> in_first;  // T1 block -> its first input channel
    struct Src {
      int32_t out_first, in_first, nout, nin;
      const std::vector<double> *coef;
    };
    std::vector<Src> srcs;
    for (int64_t ob : kv.second) {
      const int32_t *k = T3.key(ob);
      const int32_t S1p = k[2], S2p = k[3], W2s = k[4];
      const int64_t ds1p = T3.idx[2].dims[S1p], ds2p = T3.idx[3].dims[S2p];
      const int64_t dw2 = T3.idx[4].dims[W2s];
      const int32_t ofirst = (int32_t)(p->outs.size() - pr.out0);
      const int32_t nout = (int32_t)(ds1p * ds2p * dw2);
      for (int64_t s12 = 0; s12 < ds1p * ds2p; ++s12)
        for (int64_t w2 = 0; w2 < dw2; ++w2)
          p->outs.push_back({T3.offs[ob] + s12 * dw2 + w2, ds1p * ds2p * dw2,
                             (int64_t)pr.da * ds1p * ds2p * dw2});
      for (const FusedMpo::Entry &e : fm.get(S1p, S2p, W2s)) {
        auto tb = t1blk.find({Ap, e.src[0], e.src[1], e.src[2], Bs});
        if (tb == t1blk.end()) continue;
        const int64_t ib = tb->second;
        const int64_t dw = T1.idx[1].dims[e.src[0]], ds1 = T1.idx[2].dims[e.src[1]];
        const int64_t ds2 = T1.idx[3].dims[e.src[2]];
        auto f = in_first.find(ib);
        if (f == in_first.end()) {
          f = in_first.emplace(ib, (int32_t)(p->ins.size() - pr.in0)).first;
          for (int64_t c = 0; c < dw * ds1 * ds2; ++c)
            p->ins.push_back({T1.offs[ib] + c * pr.db, dw * ds1 * ds2 * pr.db});
        }
        srcs.push_back({ofirst, f->second, nout, (int32_t)(dw * ds1 * ds2), &e.coef});
      }
    }
    pr.nin = (int32_t)p->ins.size() - pr.in0;
    pr.nout = (int32_t)p->outs.size() - pr.out0;
    UDMRG_REQUIRE(pr.nin <= 512, "MPO step: more than 512 input channels in one sector pair");
    std::vector<double> C((size_t)pr.nout * std::max(pr.nin, 1), 0.0);
    for (const Src &s : srcs)
      for (int ic = 0; ic < s.nin; ++ic)
        for (int oc = 0; oc < s.nout; ++oc)
          C[(size_t)(s.out_first + oc) * pr.nin + s.in_first + ic] += (*s.coef)[ic * s.nout + oc];
    int64_t nnz = 0;
    for (int o = 0; o < pr.nout; ++o) {
      for (int i = 0; i < pr.nin; ++i) {
        const double v = C[(size_t)o * pr.nin + i];
        if (v != 0.0) p->nz.push_back({v, i, 0});
      }
      nnz += (int64_t)p->nz.size() - p->rowptr.back();
      p->rowptr.push_back((int32_t)p->nz.size());
    }
    p->flops += 2.0 * (double)nnz * pr.da * pr.db;
    p->max_nin = std::max(p->max_nin, (int)pr.nin);
    const int64_t nu = (int64_t)pr.da * ((pr.db + 31) / 32);
    p->unit0.push_back(p->unit0.back() + nu);
    p->unit_pair.insert(p->unit_pair.end(), nu, (int32_t)p->pairs.size());
    p->pairs.push_back(pr);
  }
  return p;
}

void upload_mpo_step64(Ctx &ctx, MpoStep64 &m) {
  MpoStep64 *p = &m;
  p->ctx = &ctx;
  p->d_pairs = upload(ctx, p->pairs);
  p->d_ins = upload(ctx, p->ins);
  p->d_outs = upload(ctx, p->outs);
  p->d_rowptr = upload(ctx, p->rowptr);
  p->d_nz = upload(ctx, p->nz);
  p->d_unit0 = upload(ctx, p->unit0);
  p->d_unit_pair = upload(ctx, p->unit_pair);
  ctx.sync();  // host vectors stay, but the uploads finish before they could move
}

std::unique_ptr<MpoStep64> plan_mpo_step64(Ctx &ctx, FusedMpo &fm, const BTensor &T1,
                                           const BTensor &T3) {
  auto p = build_mpo_step64(fm, T1, T3);
  upload_mpo_step64(ctx, *p);
  return p;
}

}  // namespace udmrg
