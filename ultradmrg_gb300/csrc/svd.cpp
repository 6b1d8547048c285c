// Truncated block SVD on the device.
//
// The tensor is grouped into bond sectors by the QN of the new bond
// (qn_bond = ldiv - sum_{i<ldims} dir_i qn_i, the call convention of
// two_site_update_finite_vmps_impl.h:302-307, where SVD gets Div(mps[l])).
// Each sector is gathered into a dense matrix M_q.  The factor that has to be
// an isometry (U for a right move / the plain SVD, V for a left move) comes
// from an eigen-decomposition in FP64; the other factor is the exact product
// with M (U^T M = S V^T or M V = U S), so no division by small singular
// values is needed.
//   exact path:      eigenvectors of the full Gram matrix M M^T (or M^T M);
//   randomized path: range of a Gaussian sketch refined by power iterations,
//                    then the eigenvectors of the projected Gram matrix.
#include "svd.hpp"

#include <algorithm>
#include <cmath>
#include <map>

namespace udmrg {

void select_kept(const std::vector<std::vector<double>> &svals, double trunc_err, int64_t Dmin,
                 int64_t Dmax, std::vector<int64_t> &kept, int64_t &D, double &err,
                 double rtol, double extra_mass) {
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
  tail[n] = extra_mass;
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

QN row_qn(const BTensor &T, int64_t b, int ldims) {
  QN q;
  for (int i = 0; i < ldims; ++i) q = q + T.idx[i].qns[T.key(b)[i]].scaled(T.idx[i].dir);
  return q;
}

std::vector<Sector> group_sectors(const BTensor &T, int ldims, const QN &ldiv, int64_t &mtot) {
  const int r = T.rank();
  std::map<QN, std::pair<std::map<std::vector<int32_t>, int>, std::map<std::vector<int32_t>, int>>>
      smap;
  for (int64_t b = 0; b < T.nblocks(); ++b) {
    std::vector<int32_t> lk(T.key(b), T.key(b) + ldims), rk(T.key(b) + ldims, T.key(b) + r);
    auto &sec = smap[ldiv - row_qn(T, b, ldims)];
    sec.first[lk] = 0;
    sec.second[rk] = 0;
  }
  std::vector<Sector> secs;
  mtot = 0;
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
  return secs;
}

void gather(Ctx &ctx, const BTensor &T, int ldims, const QN &ldiv, std::vector<Sector> &secs,
            double *Mbuf, int64_t mtot) {
  const int r = T.rank();
  const bool cplx = T.dtype == kC128;
  UDMRG_CHECK_CUDA(cudaMemsetAsync(Mbuf, 0, std::max<int64_t>(mtot, 1) * (cplx ? 2 : 1) *
                                                sizeof(double), ctx.stream));
  std::vector<Copy2D> ops;
  std::map<QN, int> qidx;
  for (int q = 0; q < (int)secs.size(); ++q) qidx[secs[q].qn] = q;
  for (int64_t b = 0; b < T.nblocks(); ++b) {
    std::vector<int32_t> lk(T.key(b), T.key(b) + ldims), rk(T.key(b) + ldims, T.key(b) + r);
    Sector &s = secs[qidx[ldiv - row_qn(T, b, ldims)]];
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
  run_copy2d(ctx, ops, T.data, Mbuf, cplx);
}

// View of M_q (left side) or M_q^T (right side) as an (xr x xc) matrix.
struct XView {
  int64_t off, xr, xc, sr, sc;  // element (i, j) at off + i*sr + j*sc
};
XView xview(const Sector &s, bool left) {
  if (left) return {s.m_off, s.rows, s.cols, s.cols, 1};
  return {s.m_off, s.cols, s.rows, 1, s.cols};
}

// Build u, s, vt from the isometric factor of every sector: iso(i, j) =
// iso_buf[iso_off[q] + i*iso_ld[q] + j], i over rows (left) or columns (right)
// of M_q, j over the kept states.
// Complex tensors (interleaved storage, offsets in complex elements): the
// isometric factor holds eigenvectors of X X^H; the centre product uses its
// conjugate (U^H M on the left, M conj(W) on the right, W the eigenvectors of
// the transposed view's Gram matrix, whose transpose is V^H).
void build_outputs(Ctx &ctx, DeviceScratch &scratch, const BTensor &T, int ldims,
                   const std::vector<Sector> &secs, const std::vector<int64_t> &kept,
                   const std::vector<std::vector<double>> &sv, int mode, const double *iso_buf,
                   const std::vector<int64_t> &iso_off, const std::vector<int64_t> &iso_ld,
                   const double *Mbuf, SvdResult &res, int64_t iso_total = 0) {
  const int nsec = (int)secs.size();
  const bool left = (mode != kSvdSplitRight);
  const bool cplx = T.dtype == kC128;
  const DType dt = cplx ? kC128 : kF64;
  const int es = cplx ? 2 : 1;
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
  u->dtype = vt->dtype = dt;  // singular values stay real
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
  double *Cbuf = scratch.get<double>(es * std::max<int64_t>(ctot, 1));
  const double *iso_c = iso_buf;  // the operand of the centre product (conjugated if complex)
  if (cplx && iso_total > 0) {
    double *t = scratch.get<double>(2 * iso_total);
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(t, iso_buf, 2 * iso_total * sizeof(double),
                                     cudaMemcpyDeviceToDevice, ctx.stream));
    conj_inplace(ctx, t, iso_total);
    iso_c = t;
  }
  {
    GemmPlan g;
    g.ctx = &ctx;
    for (int q = 0; q < nsec; ++q) {
      if (!kept[q]) continue;
      const Sector &sc = secs[q];
      if (left)  // C(i, col) = sum_row U[row, i] M[row, col]
        gemm_add_simple(g, coffs[q], kept[q], sc.cols, sc.rows, iso_off[q], 1, iso_ld[q], sc.m_off,
                        sc.cols, 1, cplx);
      else  // C(row, i) = sum_col M[row, col] V[col, i]
        gemm_add_simple(g, coffs[q], sc.rows, kept[q], sc.cols, sc.m_off, sc.cols, 1,
                        iso_off[q], iso_ld[q], 1, cplx);
    }
    gemm_finalize(g);
    if (left)
      (ctx.svd_dw ? run_gemm_dw : run_gemm)(ctx, g, dt, iso_c, Mbuf, Cbuf, 1.0, 0.0);
    else
      (ctx.svd_dw ? run_gemm_dw : run_gemm)(ctx, g, dt, Mbuf, iso_c, Cbuf, 1.0, 0.0);
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
    run_scale(ctx, sj, Cbuf, dinv, cplx);
  }
  std::vector<Copy2D> uops, vops;
  for (int q = 0; q < nsec; ++q) {
    if (!kept[q]) continue;
    const Sector &sc = secs[q];
    const int64_t k = kept[q];
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
      if (left) {  // U rows from the isometric factor
        c.src_off = iso_off[q] + sc.roff[li] * iso_ld[q];
        c.src_ld = iso_ld[q];
      } else {  // U S = M V rows from the centre (rows x k)
        c.src_off = coffs[q] + sc.roff[li] * k;
        c.src_ld = k;
      }
      c.src_cs = 1;
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
        c.src_off = iso_off[q] + sc.coff[ri] * iso_ld[q];
        c.src_ld = 1;
        c.src_cs = iso_ld[q];
      }
      vops.push_back(c);
    }
  }
  run_copy2d(ctx, uops, left ? iso_buf : Cbuf, u->data, cplx);
  run_copy2d(ctx, vops, left ? Cbuf : iso_buf, vt->data, cplx);
  res.u = std::move(u);
  res.s = std::move(s);
  res.vt = std::move(vt);
  for (int q = 0; q < nsec; ++q) {
    res.sector_qn.push_back(secs[q].qn);
    res.sector_rows.push_back(secs[q].rows);
    res.sector_cols.push_back(secs[q].cols);
    res.sector_kept.push_back(kept[q]);
    res.sector_svals.push_back(sv[q]);
  }
}

// throws on a failed eigensolve (1: no convergence, 2: non-finite input)
void check_eig_status(int st) {
  if (st == 2) throw Error(kErrNumerics, "svd: non-finite values in the matrix to decompose");
  if (st == 3) throw Error(kErrNumerics, "svd: the multi-CTA reduction timed out");
  if (st != 0) throw Error(kErrNumerics, "svd: eigensolver failed");
}

std::vector<double> download_vec(Ctx &ctx, const double *d, int64_t n) {
  std::vector<double> h(n);
  if (n)
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(h.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost,
                                     ctx.stream));
  ctx.sync();
  return h;
}

}  // namespace

SvdResult svd_trunc(Ctx &ctx, const BTensor &T, int ldims, const QN &ldiv, double trunc_err,
                    int64_t Dmin, int64_t Dmax, int mode, int64_t spectrum_floor) {
  UDMRG_REQUIRE(ldims > 0 && ldims < T.rank(), "svd: bad ldims");
  const bool cplx = T.dtype == kC128;
  const int es = cplx ? 2 : 1;
  int64_t mtot = 0;
  auto secs = group_sectors(T, ldims, ldiv, mtot);
  const int nsec = (int)secs.size();
  DeviceScratch scratch(ctx);
  double *Mbuf = scratch.get<double>(es * std::max<int64_t>(mtot, 1));
  gather(ctx, T, ldims, ldiv, secs, Mbuf, mtot);
  // conjugate copy for the Hermitian Gram matrices X X^H
  const double *Mc = Mbuf;
  if (cplx && mtot > 0) {
    double *t = scratch.get<double>(2 * mtot);
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(t, Mbuf, 2 * mtot * sizeof(double), cudaMemcpyDeviceToDevice,
                                     ctx.stream));
    conj_inplace(ctx, t, mtot);
    Mc = t;
  }
  // Gram matrices on the isometry side
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
  double *G = scratch.get<double>(es * std::max<int64_t>(gtot, 1));
  double *lam = scratch.get<double>(std::max<int64_t>(ltot, 1));
  {
    GemmPlan g;
    g.ctx = &ctx;
    for (int q = 0; q < nsec; ++q) {
      const XView x = xview(secs[q], left);  // G = X X^T (X X^H)
      gemm_add_simple(g, jobs[q].g_off, x.xr, x.xr, x.xc, x.off, x.sr, x.sc, x.off, x.sc, x.sr,
                      cplx);
    }
    gemm_finalize(g);
    gemm_keep_upper(g);  // the eigensolver mirrors the upper triangle
    run_gemm(ctx, g, cplx ? kC128 : kF64, Mbuf, Mc, G, 1.0, 0.0);
  }
  // at most Dmax states are kept: only the leading eigenvalues of the sectors
  // (a margin of 64 below the Dmax-th largest) are computed; the weight of
  // the rest is each Gram matrix's trace minus the computed ones
  SymEigWork wk;
  std::vector<int64_t> rank_cap(nsec);
  for (int q = 0; q < nsec; ++q) rank_cap[q] = std::min(secs[q].rows, secs[q].cols);
  check_eig_status(sym_eig_values(ctx, scratch, jobs, G, lam, wk, cplx,
                                  Dmax > 0 ? std::max(Dmax, Dmin) + 64 : 0,
                                  spectrum_floor, &rank_cap, true));
  const std::vector<double> hlam = download_vec(ctx, lam, ltot);
  std::vector<std::vector<double>> sv(nsec);
  double rest = 0.0;
  for (int q = 0; q < nsec; ++q) {
    const int64_t nc = wk.computed[q];
    const int64_t rank_max = std::min(secs[q].rows, secs[q].cols);
    double listed = 0.0;
    for (int64_t i = 0; i < std::min(nc, rank_max); ++i) {
      const double l = std::max(hlam[jobs[q].lam_off + i], 0.0);
      sv[q].push_back(std::sqrt(l));
      listed += l;
    }
    if (!wk.trace.empty()) rest += std::max(wk.trace[q] - listed, 0.0);
  }
  SvdResult res;
  std::vector<int64_t> kept;
  select_kept(sv, trunc_err, Dmin, Dmax, kept, res.D, res.trunc_err, 1e-12, rest);
  // eigenvectors of the kept states only: the isometric factor (n x kept)
  std::vector<int64_t> iso_off(nsec), iso_ld(nsec);
  int64_t ztot = 0;
  for (int q = 0; q < nsec; ++q) {
    iso_off[q] = ztot;
    iso_ld[q] = std::max<int64_t>(kept[q], 1);
    ztot += (int64_t)jobs[q].n * kept[q];
  }
  double *Z = scratch.get<double>(es * std::max<int64_t>(ztot, 1));
  sym_eig_vectors(ctx, scratch, jobs, G, lam, hlam, kept, iso_off, iso_ld, Z, wk);
  build_outputs(ctx, scratch, T, ldims, secs, kept, sv, mode, Z, iso_off, iso_ld, Mbuf, res,
                ztot);
  res.sector_sketch.assign(nsec, 0);
  return res;
}

SvdResult svd_trunc_sketch(Ctx &ctx, const BTensor &T, int ldims, const QN &ldiv,
                           double trunc_err, int64_t Dmin, int64_t Dmax, int mode,
                           const SketchParams &sp) {
  UDMRG_REQUIRE(ldims > 0 && ldims < T.rank(), "svd: bad ldims");
  UDMRG_REQUIRE(T.dtype == kF64, "svd: complex tensors are not supported by this SVD yet");
  int64_t mtot = 0;
  auto secs = group_sectors(T, ldims, ldiv, mtot);
  const int nsec = (int)secs.size();
  const bool left = (mode != kSvdSplitRight);
  DeviceScratch scratch(ctx);
  double *Mbuf = scratch.get<double>(std::max<int64_t>(mtot, 1));
  gather(ctx, T, ldims, ldiv, secs, Mbuf, mtot);
  // exact squared Frobenius norm of every sector (the residual mass reference)
  std::vector<double> fro(nsec, 0.0);
  {
    VecWork w(ctx);
    for (int q = 0; q < nsec; ++q)
      fro[q] = norm2(w, Mbuf + secs[q].m_off, secs[q].rows * secs[q].cols);
  }
  std::map<QN, int64_t> req;
  for (auto &kv : sp.sketch) req[kv.first] = kv.second;
  std::vector<int64_t> s(nsec), full(nsec);
  for (int q = 0; q < nsec; ++q) {
    full[q] = std::min(secs[q].rows, secs[q].cols);
    auto it = req.find(secs[q].qn);
    const int64_t want = it == req.end() ? full[q] : it->second + sp.oversample;
    s[q] = std::max<int64_t>(1, std::min(full[q], want));
  }
  {
    int64_t ssum = 0, fsum = 0;
    for (int q = 0; q < nsec; ++q) {
      ssum += s[q];
      fsum += full[q];
    }
    if (sp.max_fraction < 1.0 && (double)ssum > sp.max_fraction * (double)fsum)
      return svd_trunc(ctx, T, ldims, ldiv, trunc_err, Dmin, Dmax, mode, kSpectrumFloor);
  }
  // isometric factor of sector q (xr x s_q, row-major) kept at uoff[q] across
  // rounds; a round recomputes only the sectors that missed
  std::vector<int64_t> uoff(nsec);
  int64_t utot = 0;
  for (int q = 0; q < nsec; ++q) {
    uoff[q] = utot;
    utot += xview(secs[q], left).xr * full[q];
  }
  double *Ubuf = scratch.get<double>(std::max<int64_t>(utot, 1));
  std::vector<std::vector<double>> sv(nsec), r2(nsec);
  std::vector<char> need(nsec, 1);

  // One sketch round over the sectors `act`: Gaussian sketch, power iterations
  // with Cholesky-QR, Rayleigh-Ritz (Gram of B = Q^T X, Jacobi), the isometric
  // factor U = Q W into Ubuf, Ritz values into sv and residual norms
  // ||X X^T u_i - theta_i u_i||^2 into r2.
  auto sketch_round = [&](const std::vector<int> &act, int round) {
    const int na = (int)act.size();
    DeviceScratch rs(ctx);
    std::vector<int64_t> yoff(na), zoff(na), soff(na);
    int64_t ytot = 0, ztot = 0, stot = 0, ltot = 0;
    std::vector<EigJob> jobs(na);
    for (int a = 0; a < na; ++a) {
      const int q = act[a];
      const XView x = xview(secs[q], left);
      yoff[a] = ytot;
      zoff[a] = ztot;
      soff[a] = stot;
      ytot += x.xr * s[q];
      ztot += x.xc * s[q];
      stot += s[q] * s[q];
      jobs[a].g_off = soff[a];
      jobs[a].lam_off = ltot;
      jobs[a].n = (int32_t)s[q];
      ltot += s[q];
    }
    double *Y = rs.get<double>(ytot), *Y2 = rs.get<double>(ytot);
    double *Z = rs.get<double>(ztot), *Z2 = rs.get<double>(ztot);
    double *Sg = rs.get<double>(stot), *Ri = rs.get<double>(stot);
    double *Vv = rs.get<double>(stot), *Wk = rs.get<double>(stot);
    double *lam = rs.get<double>(std::max<int64_t>(1, ltot));
    // Z <- Omega (xc x s), Y <- X Z
    fill_normal(ctx, Z, ztot, sp.seed * 0x9E3779B97F4A7C15ull + (uint64_t)round);
    auto mult_xz = [&](const double *zin, double *yout, double beta) {  // Y = X Z (+ beta Y)
      GemmPlan g;
      g.ctx = &ctx;
      for (int a = 0; a < na; ++a) {
        const XView x = xview(secs[act[a]], left);
        const int64_t sq = s[act[a]];
        gemm_add_simple(g, yoff[a], x.xr, sq, x.xc, x.off, x.sr, x.sc, zoff[a], sq, 1, false);
      }
      gemm_finalize(g);
      run_gemm(ctx, g, kF64, Mbuf, zin, yout, 1.0, beta);
    };
    auto mult_xty = [&](const double *yin, double *zout) {  // Z = X^T Y
      GemmPlan g;
      g.ctx = &ctx;
      for (int a = 0; a < na; ++a) {
        const XView x = xview(secs[act[a]], left);
        const int64_t sq = s[act[a]];
        gemm_add_simple(g, zoff[a], x.xc, sq, x.xr, x.off, x.sc, x.sr, yoff[a], sq, 1, false);
      }
      gemm_finalize(g);
      run_gemm(ctx, g, kF64, Mbuf, yin, zout, 1.0, 0.0);
    };
    // small per-sector products: out(rows x s) = in(rows x s) * S(s x s)
    // (S^T when trans: S stored row-major as its transpose)
    auto mult_small = [&](const double *in, const double *S, double *out,
                          const std::vector<int64_t> &off, bool on_y, bool trans = false) {
      GemmPlan h;
      h.ctx = &ctx;
      for (int a = 0; a < na; ++a) {
        const XView x = xview(secs[act[a]], left);
        const int64_t rows = on_y ? x.xr : x.xc, sq = s[act[a]];
        gemm_add_simple(h, off[a], rows, sq, sq, off[a], sq, 1, soff[a], trans ? 1 : sq,
                        trans ? sq : 1, false);
      }
      gemm_finalize(h);
      run_gemm(ctx, h, kF64, in, S, out, 1.0, 0.0);
    };
    // Cholesky-QR of the columns of B (rows x s per sector): out = B R^{-1}
    auto cholqr = [&](const double *bin, double *bout, const std::vector<int64_t> &boff,
                      bool on_y) {
      GemmPlan g;
      g.ctx = &ctx;
      for (int a = 0; a < na; ++a) {
        const XView x = xview(secs[act[a]], left);
        const int64_t rows = on_y ? x.xr : x.xc, sq = s[act[a]];
        gemm_add_simple(g, soff[a], sq, sq, rows, boff[a], 1, sq, boff[a], sq, 1, false);
      }
      gemm_finalize(g);
      run_gemm(ctx, g, kF64, bin, bin, Sg, 1.0, 0.0);
      run_chol_inv(ctx, jobs, Sg, Ri, 1e-28);
      mult_small(bin, Ri, bout, boff, on_y, true);
    };
    mult_xz(Z, Y, 0.0);
    for (int it = 0; it < sp.power_iters; ++it) {
      cholqr(Y, Y2, yoff, true);
      mult_xty(Y2, Z);
      cholqr(Z, Z2, zoff, false);
      mult_xz(Z2, Y, 0.0);
    }
    cholqr(Y, Y2, yoff, true);
    cholqr(Y2, Y, yoff, true);  // second pass: Q = Y (orthonormal to FP64 accuracy)
    // B^T = X^T Q (xc x s) -> G = B B^T = (X^T Q)^T (X^T Q) (s x s)
    mult_xty(Y, Z);
    {
      GemmPlan g;
      g.ctx = &ctx;
      for (int a = 0; a < na; ++a) {
        const XView x = xview(secs[act[a]], left);
        const int64_t sq = s[act[a]];
        gemm_add_simple(g, soff[a], sq, sq, x.xc, zoff[a], 1, sq, zoff[a], sq, 1, false);
      }
      gemm_finalize(g);
      run_gemm(ctx, g, kF64, Z, Z, Sg, 1.0, 0.0);
    }
    {  // Rayleigh-Ritz: all s eigenpairs of G (Vv: row-major s x s eigenvectors)
      SymEigWork wk;
      check_eig_status(sym_eig_values(ctx, rs, jobs, Sg, lam, wk));
      const std::vector<double> hlr = download_vec(ctx, lam, ltot);
      std::vector<int64_t> kk(na), zo(na), zl(na);
      for (int a = 0; a < na; ++a) {
        kk[a] = zl[a] = s[act[a]];
        zo[a] = soff[a];
      }
      sym_eig_vectors(ctx, rs, jobs, Sg, lam, hlr, kk, zo, zl, Vv, wk);
    }
    mult_small(Y, Vv, Y2, yoff, true);   // U = Q W (xr x s)
    mult_small(Z, Vv, Z2, zoff, false);  // P = X^T U = Z W (xc x s)
    // residuals: Y := X P - U Theta (Q in Y is no longer needed), column norms
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(Y, Y2, ytot * sizeof(double), cudaMemcpyDeviceToDevice,
                                     ctx.stream));
    std::vector<ScaleJob> sj(na);
    for (int a = 0; a < na; ++a) {
      const XView x = xview(secs[act[a]], left);
      sj[a] = ScaleJob{yoff[a], jobs[a].lam_off, (int32_t)x.xr, (int32_t)s[act[a]], 0, 0};
    }
    run_scale(ctx, sj, Y, lam, false);
    mult_xz(Z2, Y, -1.0);
    run_col_sumsq(ctx, sj, Y, Wk);  // ||r_i||^2 at lam_off (Wk holds >= ltot doubles)
    // keep U of these sectors
    for (int a = 0; a < na; ++a) {
      const int q = act[a];
      UDMRG_CHECK_CUDA(cudaMemcpyAsync(Ubuf + uoff[q], Y2 + yoff[a],
                                       xview(secs[q], left).xr * s[q] * sizeof(double),
                                       cudaMemcpyDeviceToDevice, ctx.stream));
    }
    const std::vector<double> hr = download_vec(ctx, Wk, ltot);
    const std::vector<double> hl = download_vec(ctx, lam, ltot);
    for (int a = 0; a < na; ++a) {
      const int q = act[a];
      sv[q].assign(s[q], 0.0);
      r2[q].assign(s[q], 0.0);
      for (int64_t i = 0; i < s[q]; ++i) {
        sv[q][i] = std::sqrt(std::max(hl[jobs[a].lam_off + i], 0.0));
        r2[q][i] = std::max(hr[jobs[a].lam_off + i], 0.0);
      }
    }
  };

  SvdResult res;
  for (int round = 0;; ++round) {
    std::vector<int> act;
    for (int q = 0; q < nsec; ++q)
      if (need[q]) act.push_back(q);
    if (!act.empty()) sketch_round(act, round);
    // selection over the Ritz values of all sectors; the weight outside them
    // (exact norms minus Ritz values) counts as discarded
    double resid = 0.0;
    for (int q = 0; q < nsec; ++q) {
      double got = 0.0;
      for (double v : sv[q]) got += v * v;
      resid += std::max(fro[q] - got, 0.0);
    }
    std::vector<int64_t> kept;
    SvdResult trial;
    select_kept(sv, trunc_err, Dmin, Dmax, kept, trial.D, trial.trunc_err, 1e-12, resid);
    // Misses: a sector whose whole sketch is kept, or whose Ritz values are
    // not accurate enough to certify the kept set.  Error of Ritz value i:
    // ||r_i||^2 / (theta_i - theta_last) (the gap to the unresolved part of
    // the spectrum), and ||r_last|| for the last one.  Certified when (a) the
    // kept values of all sectors are accurate to 1e-11 of the total weight and
    // (b) no discarded Ritz value can reach the cutoff c (the smallest kept
    // theta) beyond the tie tolerance of the selection rule.
    double ftot = 0.0, tmax = 0.0, cut = -1.0;
    for (int q = 0; q < nsec; ++q) {
      ftot += fro[q];
      for (int64_t i = 0; i < s[q]; ++i) {
        const double th = sv[q][i] * sv[q][i];
        tmax = std::max(tmax, th);
        if (i < kept[q]) cut = cut < 0 ? th : std::min(cut, th);
      }
    }
    const double tie = 2e-12 * tmax, acc_tol = 1e-11 * ftot / std::max(1, nsec);
    bool grow = false;
    for (int q = 0; q < nsec; ++q) {
      need[q] = 0;
      if (s[q] >= full[q]) continue;
      bool miss = kept[q] == s[q];
      const int64_t last = s[q] - 1;
      const double th_last = sv[q][last] * sv[q][last];
      auto err = [&](int64_t i) {
        if (i == last) return std::sqrt(r2[q][i]);
        const double gap = sv[q][i] * sv[q][i] - th_last;
        return gap > 0 ? r2[q][i] / gap : std::sqrt(r2[q][i]);
      };
      double kerr = 0.0;
      for (int64_t i = 0; i < kept[q] && !miss; ++i) kerr += err(i);
      miss |= kerr > acc_tol;
      for (int64_t j = kept[q]; j < s[q] && !miss && cut >= 0; ++j) {
        const double th = sv[q][j] * sv[q][j];
        miss |= err(j) > std::max(cut - th, tie);
      }
      if (miss) {
        s[q] = std::min(full[q], 2 * s[q] + sp.oversample);
        need[q] = 1;
        grow = true;
      }
    }
    if (grow && round < 8) continue;
    // (after the last round, sectors still marked keep the sketch they have)
    std::vector<int64_t> iso_ld(nsec);
    for (int q = 0; q < nsec; ++q) iso_ld[q] = (int64_t)sv[q].size();
    res.D = trial.D;
    res.trunc_err = trial.trunc_err;
    build_outputs(ctx, scratch, T, ldims, secs, kept, sv, mode, Ubuf, uoff, iso_ld, Mbuf, res);
    res.sector_sketch = iso_ld;
    res.grow_rounds = round;
    ctx.sync();
    return res;
  }
}

}  // namespace udmrg
