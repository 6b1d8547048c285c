// Truncated block SVD on the device.
//
// The tensor is grouped into bond sectors by the QN of the new bond
// (qn_bond = ldiv - sum_{i<ldims} dir_i qn_i, the call convention of
// two_site_update_finite_vmps_impl.h:302-307, where SVD gets Div(mps[l])).
// Each sector is gathered into a dense matrix M_q.  The side that has to come
// out as an isometry is taken from the eigen-decomposition of a Gram matrix
// (M M^T for the left factor, M^T M for the right one; cyclic Jacobi, FP64),
// and the other factor is the exact product with M (U^T M = S V^T or
// M V = U S), so no division by small singular values is needed.
#include "svd.hpp"

#include <algorithm>
#include <cmath>
#include <map>

namespace udmrg {

void select_kept(const std::vector<std::vector<double>> &svals, double trunc_err, int64_t Dmin,
                 int64_t Dmax, std::vector<int64_t> &kept, int64_t &D, double &err,
                 double rtol) {
  struct E {
    double s;
    int q;
    int i;
  };
  std::vector<E> flat;
  for (int q = 0; q < (int)svals.size(); ++q)
    for (int i = 0; i < (int)svals[q].size(); ++i) flat.push_back({svals[q][i], q, i});
  kept.assign(svals.size(), 0);
  const int64_t n = (int64_t)flat.size();
  if (n == 0) {
    D = 0;
    err = 0;
    return;
  }
  double smax = 0;
  for (auto &e : flat) smax = std::max(smax, e.s);
  std::sort(flat.begin(), flat.end(), [](const E &a, const E &b) {
    if (a.s != b.s) return a.s > b.s;
    if (a.q != b.q) return a.q < b.q;
    return a.i < b.i;
  });
  const double tol = rtol * smax;
  std::vector<E> ord;
  ord.reserve(n);
  for (int64_t i = 0; i < n;) {
    int64_t j = i + 1;
    while (j < n && flat[j - 1].s - flat[j].s <= tol) ++j;
    std::vector<E> cl(flat.begin() + i, flat.begin() + j);
    std::sort(cl.begin(), cl.end(), [](const E &a, const E &b) {
      return a.q != b.q ? a.q < b.q : a.i < b.i;
    });
    ord.insert(ord.end(), cl.begin(), cl.end());
    i = j;
  }
  std::vector<double> tail(n + 1, 0.0);
  for (int64_t k = n - 1; k >= 0; --k) tail[k] = tail[k + 1] + ord[k].s * ord[k].s;
  const double total = tail[0];
  const int64_t lo = std::min(Dmin, n), hi = std::min(Dmax, n);
  D = hi;
  for (int64_t k = lo; k <= hi; ++k)
    if (total == 0 || tail[k] / total <= trunc_err) {
      D = k;
      break;
    }
  err = total == 0 ? 0.0 : tail[D] / total;
  for (int64_t k = 0; k < D; ++k) kept[ord[k].q]++;
}

namespace {

struct Sector {
  QN qn;
  std::vector<std::vector<int32_t>> lkeys, rkeys;
  std::vector<int64_t> roff, coff, rsz, csz;
  int64_t rows = 0, cols = 0;
  int64_t m_off = 0;  // dense matrix offset (elements)
};

int64_t prod_dims(const BTensor &T, const std::vector<int32_t> &k, int first) {
  int64_t p = 1;
  for (size_t i = 0; i < k.size(); ++i) p *= T.idx[first + i].dims[k[i]];
  return p;
}

}  // namespace

SvdResult svd_trunc(Ctx &ctx, const BTensor &T, int ldims, const QN &ldiv, double trunc_err,
                    int64_t Dmin, int64_t Dmax, int mode) {
  UDMRG_REQUIRE(ldims > 0 && ldims < T.rank(), "svd: bad ldims");
  UDMRG_REQUIRE(T.dtype == kF64, "svd: complex tensors are not supported by this SVD yet");
  const int r = T.rank();
  // 1. bond sectors
  std::map<QN, std::pair<std::map<std::vector<int32_t>, int>, std::map<std::vector<int32_t>, int>>>
      smap;
  for (int64_t b = 0; b < T.nblocks(); ++b) {
    std::vector<int32_t> lk(T.key(b), T.key(b) + ldims), rk(T.key(b) + ldims, T.key(b) + r);
    QN qrow;
    for (int i = 0; i < ldims; ++i) qrow = qrow + T.idx[i].qns[lk[i]].scaled(T.idx[i].dir);
    auto &sec = smap[ldiv - qrow];
    sec.first[lk] = 0;
    sec.second[rk] = 0;
  }
  std::vector<Sector> secs;
  int64_t mtot = 0;
  for (auto &kv : smap) {
    Sector s;
    s.qn = kv.first;
    for (auto &lk : kv.second.first) {
      s.lkeys.push_back(lk.first);
      s.roff.push_back(s.rows);
      s.rsz.push_back(prod_dims(T, lk.first, 0));
      s.rows += s.rsz.back();
    }
    for (auto &rk : kv.second.second) {
      s.rkeys.push_back(rk.first);
      s.coff.push_back(s.cols);
      s.csz.push_back(prod_dims(T, rk.first, ldims));
      s.cols += s.csz.back();
    }
    s.m_off = mtot;
    mtot += s.rows * s.cols;
    secs.push_back(std::move(s));
  }
  const int nsec = (int)secs.size();
  // 2. gather dense sector matrices
  DeviceScratch scratch(ctx);
  double *Mbuf = scratch.get<double>(std::max<int64_t>(mtot, 1));
  UDMRG_CHECK_CUDA(cudaMemsetAsync(Mbuf, 0, std::max<int64_t>(mtot, 1) * sizeof(double), ctx.stream));
  {
    std::vector<Copy2D> ops;
    std::map<QN, int> qidx;
    for (int q = 0; q < nsec; ++q) qidx[secs[q].qn] = q;
    for (int64_t b = 0; b < T.nblocks(); ++b) {
      std::vector<int32_t> lk(T.key(b), T.key(b) + ldims), rk(T.key(b) + ldims, T.key(b) + r);
      QN qrow;
      for (int i = 0; i < ldims; ++i) qrow = qrow + T.idx[i].qns[lk[i]].scaled(T.idx[i].dir);
      Sector &s = secs[qidx[ldiv - qrow]];
      const int li = (int)(std::lower_bound(s.lkeys.begin(), s.lkeys.end(), lk) - s.lkeys.begin());
      const int ri = (int)(std::lower_bound(s.rkeys.begin(), s.rkeys.end(), rk) - s.rkeys.begin());
      Copy2D c{};
      c.src_off = T.offs[b];
      c.rows = (int32_t)s.rsz[li];
      c.cols = (int32_t)s.csz[ri];
      c.src_ld = c.cols;
      c.src_cs = 1;
      c.dst_off = s.m_off + s.roff[li] * s.cols + s.coff[ri];
      c.dst_ld = s.cols;
      c.dst_cs = 1;
      ops.push_back(c);
    }
    run_copy2d(ctx, ops, T.data, Mbuf, false);
  }
  // 3. Gram matrices on the isometry side
  const bool left = (mode != kSvdSplitRight);
  std::vector<EigJob> jobs(nsec);
  int64_t gtot = 0, ltot = 0;
  for (int q = 0; q < nsec; ++q) {
    const int64_t n = left ? secs[q].rows : secs[q].cols;
    jobs[q].g_off = gtot;
    jobs[q].lam_off = ltot;
    jobs[q].n = (int32_t)n;
    gtot += n * n;
    ltot += n;
  }
  double *G = scratch.get<double>(std::max<int64_t>(gtot, 1));
  double *V = scratch.get<double>(std::max<int64_t>(gtot, 1));
  double *W = scratch.get<double>(std::max<int64_t>(gtot, 1));
  double *lam = scratch.get<double>(std::max<int64_t>(ltot, 1));
  {
    GemmPlan g;
    g.ctx = &ctx;
    for (int q = 0; q < nsec; ++q) {
      const Sector &s = secs[q];
      if (left)  // G = M M^T
        gemm_add_simple(g, jobs[q].g_off, s.rows, s.rows, s.cols, s.m_off, s.cols, 1, s.m_off, 1,
                        s.cols, false);
      else  // G = M^T M
        gemm_add_simple(g, jobs[q].g_off, s.cols, s.cols, s.rows, s.m_off, 1, s.cols, s.m_off,
                        s.cols, 1, false);
    }
    gemm_finalize(g);
    run_gemm(ctx, g, kF64, Mbuf, Mbuf, G, 1.0, 0.0);
  }
  const int st = run_jacobi_eig(ctx, jobs, G, V, W, lam);
  if (st != 0) throw Error(kErrNumerics, "svd: Jacobi eigensolver did not converge");
  // 4. selection on the host
  std::vector<double> hlam(ltot);
  if (ltot)
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(hlam.data(), lam, ltot * sizeof(double),
                                     cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  std::vector<std::vector<double>> sv(nsec);
  for (int q = 0; q < nsec; ++q) {
    const int64_t n = jobs[q].n;
    const int64_t rank_max = std::min(secs[q].rows, secs[q].cols);
    for (int64_t i = 0; i < std::min(n, rank_max); ++i)
      sv[q].push_back(std::sqrt(std::max(hlam[jobs[q].lam_off + i], 0.0)));
  }
  SvdResult res;
  std::vector<int64_t> kept;
  select_kept(sv, trunc_err, Dmin, Dmax, kept, res.D, res.trunc_err);
  // 5. outputs
  Index bond;
  bond.dir = 1;
  std::vector<int> bid(nsec, -1);
  for (int q = 0; q < nsec; ++q)
    if (kept[q] > 0) {
      bid[q] = bond.nsec();
      bond.qns.push_back(secs[q].qn);
      bond.dims.push_back(kept[q]);
    }
  auto u = std::make_unique<BTensor>();
  auto vt = std::make_unique<BTensor>();
  auto s = std::make_unique<BTensor>();
  for (auto *t : {u.get(), vt.get(), s.get()}) {
    t->ctx = &ctx;
    t->dtype = kF64;
    t->nq = T.nq;
  }
  u->idx.assign(T.idx.begin(), T.idx.begin() + ldims);
  u->idx.push_back(bond);
  vt->idx.push_back(bond.inverse());
  vt->idx.insert(vt->idx.end(), T.idx.begin() + ldims, T.idx.end());
  s->idx = {bond.inverse(), bond};
  std::vector<int32_t> ukeys, vkeys, skeys;
  for (int q = 0; q < nsec; ++q) {
    if (bid[q] < 0) continue;
    for (auto &lk : secs[q].lkeys) {
      ukeys.insert(ukeys.end(), lk.begin(), lk.end());
      ukeys.push_back(bid[q]);
    }
    for (auto &rk : secs[q].rkeys) {
      vkeys.push_back(bid[q]);
      vkeys.insert(vkeys.end(), rk.begin(), rk.end());
    }
    skeys.push_back(bid[q]);
    skeys.push_back(bid[q]);
  }
  u->set_blocks(sort_keys(ukeys, u->rank()));
  vt->set_blocks(sort_keys(vkeys, vt->rank()));
  s->set_blocks(sort_keys(skeys, 2));
  u->alloc_data();
  vt->alloc_data();
  s->alloc_data();
  // s: diagonal blocks, filled on the host
  {
    std::vector<double> hs(s->size(), 0.0);
    for (int q = 0; q < nsec; ++q) {
      if (bid[q] < 0) continue;
      const int64_t b = s->find({bid[q], bid[q]});
      const int64_t k = kept[q];
      for (int64_t i = 0; i < k; ++i) {
        hs[s->offs[b] + i * k + i] = sv[q][i];
        res.svals.push_back(sv[q][i]);
        const double p = sv[q][i] * sv[q][i];
        if (p > 0) res.ee += -p * std::log(p);
      }
    }
    if (!hs.empty())
      UDMRG_CHECK_CUDA(cudaMemcpyAsync(s->data, hs.data(), hs.size() * sizeof(double),
                                       cudaMemcpyHostToDevice, ctx.stream));
    ctx.sync();
  }
  // centre factor: C_q = U_q^T M_q (k x cols) on the left side, M_q V_q (rows x k) on the right
  int64_t ctot = 0;
  std::vector<int64_t> coffs(nsec, 0);
  for (int q = 0; q < nsec; ++q) {
    coffs[q] = ctot;
    ctot += kept[q] * (left ? secs[q].cols : secs[q].rows);
  }
  double *Cbuf = scratch.get<double>(std::max<int64_t>(ctot, 1));
  {
    GemmPlan g;
    g.ctx = &ctx;
    for (int q = 0; q < nsec; ++q) {
      if (!kept[q]) continue;
      const Sector &sc = secs[q];
      const int64_t n = jobs[q].n;
      if (left)  // C(i, col) = sum_row V[row, i] M[row, col]
        gemm_add_simple(g, coffs[q], kept[q], sc.cols, sc.rows, jobs[q].g_off, 1, n, sc.m_off,
                        sc.cols, 1, false);
      else  // C(row, i) = sum_col M[row, col] V[col, i]
        gemm_add_simple(g, coffs[q], sc.rows, kept[q], sc.cols, sc.m_off, sc.cols, 1,
                        jobs[q].g_off, n, 1, false);
    }
    gemm_finalize(g);
    if (left)
      run_gemm(ctx, g, kF64, V, Mbuf, Cbuf, 1.0, 0.0);
    else
      run_gemm(ctx, g, kF64, Mbuf, V, Cbuf, 1.0, 0.0);
  }
  if (mode == kSvdFull) {
    // vt = S^{-1} (U^T M): scale row i of each centre block by 1/s_i (0 for s_i == 0)
    std::vector<double> inv;
    std::vector<ScaleJob> sj;
    for (int q = 0; q < nsec; ++q) {
      if (!kept[q]) continue;
      ScaleJob j{};
      j.x_off = coffs[q];
      j.f_off = (int64_t)inv.size();
      j.rows = (int32_t)kept[q];
      j.cols = (int32_t)secs[q].cols;
      j.by_row = 1;
      sj.push_back(j);
      for (int64_t i = 0; i < kept[q]; ++i) inv.push_back(sv[q][i] > 0 ? 1.0 / sv[q][i] : 0.0);
    }
    double *dinv = scratch.get<double>(std::max<size_t>(inv.size(), 1));
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(dinv, inv.data(), inv.size() * sizeof(double),
                                     cudaMemcpyHostToDevice, ctx.stream));
    run_scale(ctx, sj, Cbuf, dinv, false);
  }
  // scatter into u and vt
  std::vector<Copy2D> uops, vops;
  for (int q = 0; q < nsec; ++q) {
    if (!kept[q]) continue;
    const Sector &sc = secs[q];
    const int64_t k = kept[q];
    const int64_t n = jobs[q].n;
    for (size_t li = 0; li < sc.lkeys.size(); ++li) {
      std::vector<int32_t> key = sc.lkeys[li];
      key.push_back(bid[q]);
      const int64_t b = u->find(key);
      Copy2D c{};
      c.dst_off = u->offs[b];
      c.rows = (int32_t)sc.rsz[li];
      c.cols = (int32_t)k;
      c.dst_ld = k;
      c.dst_cs = 1;
      if (left) {  // U rows from the eigenvectors (row-major n x n, columns sorted)
        c.src_off = jobs[q].g_off + sc.roff[li] * n;
        c.src_ld = n;
        c.src_cs = 1;
      } else {  // U S = M V rows from the centre (rows x k)
        c.src_off = coffs[q] + sc.roff[li] * k;
        c.src_ld = k;
        c.src_cs = 1;
      }
      uops.push_back(c);
    }
    for (size_t ri = 0; ri < sc.rkeys.size(); ++ri) {
      std::vector<int32_t> key = {bid[q]};
      key.insert(key.end(), sc.rkeys[ri].begin(), sc.rkeys[ri].end());
      const int64_t b = vt->find(key);
      Copy2D c{};
      c.dst_off = vt->offs[b];
      c.rows = (int32_t)k;
      c.cols = (int32_t)sc.csz[ri];
      c.dst_ld = sc.csz[ri];
      c.dst_cs = 1;
      if (left) {  // (S) V^T columns from the centre (k x cols)
        c.src_off = coffs[q] + sc.coff[ri];
        c.src_ld = sc.cols;
        c.src_cs = 1;
      } else {  // V^T(i, j) = V[coff + j, i]
        c.src_off = jobs[q].g_off + sc.coff[ri] * n;
        c.src_ld = 1;
        c.src_cs = n;
      }
      vops.push_back(c);
    }
  }
  run_copy2d(ctx, uops, left ? V : Cbuf, u->data, false);
  run_copy2d(ctx, vops, left ? Cbuf : V, vt->data, false);
  res.u = std::move(u);
  res.s = std::move(s);
  res.vt = std::move(vt);
  return res;
}

}  // namespace udmrg
