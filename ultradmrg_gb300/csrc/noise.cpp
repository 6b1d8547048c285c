// Two-site VMPS with noise (subspace expansion): TwoSiteFiniteVMPSWithNoise
// of algorithm/vmps/two_site_update_noise_finite_vmps_impl.h:81-556 on the
// device kernels of the plain sweep.
//
// * Boundaries (CheckAndUpdateBoundaryMPSTensors, algorithm/vmps/vmps_init.h:
//   135-246): from each end, tensors are canonicalised (SVD keeping every
//   singular value, so a bond keeps min(rows, cols) states per sector, as a
//   QR would); one whose bond can hold the whole block space becomes an index
//   combiner, the rest of it moving into its neighbour; the first site where
//   Dmax binds (or the middle) bounds the sweeps.
// * Noise adaptation (:132-200): before each update the energy expectation of
//   the current two-site state (CalEnergyEptTwoSite, :688-721) against the
//   previous update's energy: a rise of at least alpha times the previous
//   rise lowers the noise by noise_decrease, a smaller rise raises it by
//   noise_increase (capped at max_noise); a fall leaves it.
// * Update (:216-404): Lanczos; unless the noise is below 1e-10 or the
//   quantum-number coverage test (IsQNCovered, :727-765) says the bond is
//   already complete, the expansion term noise * (L psi W1 W2) with the right
//   MPO bond open and fused with psi's right bond (moving right) or
//   noise * (psi R W2 W1) with the left MPO bond fused with the left bond
//   (moving left) is appended to psi's bond sectors (ExpandQNBlocks) and the
//   next-next MPS tensor grows by zeros along that bond (:406-556); then the
//   exact truncated SVD, the MPS update and the environment update.
// The sector conventions of fusion and expansion are those of blockmove.hpp.
#include <chrono>
#include <cmath>
#include <set>

#include "blockmove.hpp"
#include "dmrg.hpp"
#include "vecops.hpp"

namespace udmrg {

namespace {

constexpr int64_t kKeepAll = (int64_t)1 << 40;

double wall() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

void left_canonicalize(Ctx &ctx, std::vector<TensorPtr> &mps, int64_t i) {
  auto r = svd_trunc(ctx, *mps[i], 2, mps[i]->div(), 0.0, kKeepAll, kKeepAll, kSvdSplitLeft);
  mps[i] = std::move(r.u);
  mps[i + 1] = contract_axes(ctx, *r.vt, *mps[i + 1], {1}, {0});
}

void right_canonicalize(Ctx &ctx, std::vector<TensorPtr> &mps, int64_t i) {
  auto r = svd_trunc(ctx, *mps[i], 1, mps[i]->div(), 0.0, kKeepAll, kKeepAll, kSvdSplitRight);
  mps[i] = std::move(r.vt);
  mps[i - 1] = contract_axes(ctx, *mps[i - 1], *r.u, {2}, {0});
}

std::pair<int64_t, int64_t> boundaries(Ctx &ctx, std::vector<TensorPtr> &mps, int64_t Dmax) {
  const int64_t N = (int64_t)mps.size();
  const int64_t lmid = N % 2 == 0 ? N / 2 - 1 : N / 2;
  const int64_t rmid = N / 2;
  int64_t left = 0, right = 0;
  for (int64_t i = 0; i < lmid; ++i) {
    left_canonicalize(ctx, mps, i);
    const BTensor &t = *mps[i];
    const int64_t a = t.idx[0].dim(), s = t.idx[1].dim(), b = t.idx[2].dim();
    if (a * s > Dmax) {
      left = i;
      break;
    }
    if (a * s > b) {
      auto c = combiner(ctx, t.idx[0], t.idx[1], t.idx[2].dir, t.dtype, t.nq);
      auto cd = dag(ctx, *c);
      auto r = contract_axes(ctx, *cd, t, {0, 1}, {0, 1});
      mps[i + 1] = contract_axes(ctx, *r, *mps[i + 1], {1}, {0});
      mps[i] = std::move(c);
    }
    if (i == lmid - 1) left = i;
  }
  for (int64_t i = N - 1; i > rmid; --i) {
    right_canonicalize(ctx, mps, i);
    const BTensor &t = *mps[i];
    const int64_t b = t.idx[0].dim(), s = t.idx[1].dim(), c = t.idx[2].dim();
    if (s * c > Dmax) {
      right = i;
      break;
    }
    if (s * c > b) {
      auto cb = combiner(ctx, t.idx[1], t.idx[2], -1, t.dtype, t.nq);
      cb = permute(ctx, *cb, {2, 0, 1});  // (f, s, c)
      auto cbd = dag(ctx, *cb);
      auto r = contract_axes(ctx, t, *cbd, {1, 2}, {1, 2});
      mps[i - 1] = contract_axes(ctx, *mps[i - 1], *r, {2}, {0});
      mps[i] = std::move(cb);
    }
    if (i == rmid + 1) right = i;
  }
  return {left, right};
}

// The quantum numbers the coverage test reads: a two-state site's outer bond
// sectors, otherwise the sums q_bond + q_phys of the outer bond fused with the
// physical index taken with the same direction.
std::set<QN> side_qns(const BTensor &t, bool left) {
  std::set<QN> out;
  const Index &phys = t.idx[1];
  const Index &bond = t.idx[left ? 0 : 2];
  if (phys.dim() == 2) {
    out.insert(bond.qns.begin(), bond.qns.end());
  } else {
    for (const QN &qb : bond.qns)
      for (const QN &qs : phys.qns) out.insert(qb + qs);
  }
  return out;
}

bool covered(const std::set<QN> &cover, const std::set<QN> &sub) {
  for (const QN &q : sub)
    if (!cover.count(q)) return false;
  return true;
}

// noise * the expansion term, its bond index first.
TensorPtr expansion_term(Ctx &ctx, const BTensor &gs, const BTensor &L, const BTensor &W1,
                         const BTensor &W2, const BTensor &R, char dir, double noise) {
  TensorPtr term;
  if (dir == 'r') {
    auto t1 = contract_axes(ctx, L, gs, {2}, {0});      // (a', w, s1, s2, b)
    auto t2 = contract_cyclic(ctx, *t1, W1, 1, 0, 2);   // (s2, b, a', s1', wr)
    t1.reset();
    auto t3 = contract_cyclic(ctx, *t2, W2, 4, 0, 2);   // (b, a', s1', s2', w2)
    t2.reset();
    term = fuse_axes(ctx, *t3, 0, 4, gs.idx[3].dir);    // (f, a', s1', s2')
  } else {
    auto t1 = contract_axes(ctx, gs, R, {3}, {2});           // (a, s1, s2, b', w2)
    auto t2 = contract_axes(ctx, *t1, W2, {2, 4}, {1, 3});   // (a, s1, b', wl2, s2')
    t1.reset();
    auto t3 = contract_axes(ctx, *t2, W1, {1, 3}, {1, 3});   // (a, b', s2', wl1, s1')
    t2.reset();
    auto t4 = permute(ctx, *t3, {0, 3, 4, 2, 1});            // (a, wl1, s1', s2', b')
    term = fuse_axes(ctx, *t4, 0, 1, gs.idx[0].dir);         // (f, s1', s2', b')
  }
  scale(ctx, term->data, term->size() * elem_doubles(term->dtype), noise);
  return term;
}

struct NoiseState {
  double e0 = 0.0;    // the previous update's energy (this sweep)
  double last = 0.0;  // the previous update's energy expectation
  double noise = 0.0;
};

void noise_update(Ctx &ctx, std::vector<TensorPtr> &mps, std::vector<TensorPtr> &lenvs,
                  std::vector<TensorPtr> &renvs, const std::vector<const BTensor *> &W,
                  const SweepParams &p, const NoiseParams &np, char dir, int64_t target,
                  NoiseState &st, std::vector<SiteLog> *log, std::vector<double> *noise_log) {
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
  const double t0 = wall();
  const BTensor &L = *lenvs[lenv_len], &R = *renvs[renv_len];
  auto init = contract_axes(ctx, *mps[l], *mps[r], {2}, {0});
  auto mv = plan_matvec2(ctx, L, *W[l], *W[r], R, *init, p.lancz.precision);
  // energy expectation of the current state, then the noise for this update
  double actual;
  {
    auto x = embed(ctx, *init, *mv->sstruct);
    auto y = x->clone_struct();
    y->alloc_data();
    mv->apply(x->data, y->data);
    VecWork w(ctx);
    actual = dot(w, x->data, y->data, x->size(), x->dtype == kC128).real();
  }
  if (actual - st.e0 > 0.0) {
    if (actual - st.e0 >= np.alpha * std::fabs(st.last - st.e0))
      st.noise *= np.noise_decrease;
    else
      st.noise = std::min(st.noise * np.noise_increase, np.max_noise);
  }
  auto lres = lanczos_gs(ctx, *mv, *init, p.lancz);
  const double t1 = wall();
  const double mvflops = mv->flops;
  mv.reset();
  init.reset();
  TensorPtr gs = std::move(lres.gs_vec);
  bool expand = std::fabs(st.noise) >= 1e-10;
  if (expand) {
    const auto ql = side_qns(*mps[l], true), qr = side_qns(*mps[r], false);
    if ((dir == 'r' && covered(qr, ql)) || (dir == 'l' && covered(ql, qr))) expand = false;
  }
  if (expand) {
    auto term = expansion_term(ctx, *gs, L, *W[l], *W[r], R, dir, st.noise);
    const Index zeros = term->idx[0].inverse();
    if (dir == 'r') {
      auto g = permute(ctx, *gs, {3, 0, 1, 2});
      auto e = expand_axis(ctx, *g, term.get(), 0, nullptr);
      gs = permute(ctx, *e, {1, 2, 3, 0});
      mps[target + 2] = expand_axis(ctx, *mps[target + 2], nullptr, 0, &zeros);
    } else {
      gs = expand_axis(ctx, *gs, term.get(), 0, nullptr);
      mps[target - 2] = expand_axis(ctx, *mps[target - 2], nullptr, 2, &zeros);
    }
  }
  auto sres = svd_trunc(ctx, *gs, 2, mps[l]->div(), p.trunc_err, p.Dmin, p.Dmax,
                        dir == 'r' ? kSvdSplitLeft : kSvdSplitRight);
  gs.reset();
  mps[l] = std::move(sres.u);
  mps[r] = std::move(sres.vt);
  ctx.sync();
  const double t2 = wall();
  if (dir == 'r')
    lenvs[lenv_len + 1] = update_site_lenv(ctx, L, *mps[target], *W[target]);
  else
    renvs[renv_len + 1] = update_site_renv(ctx, R, *mps[target], *W[target]);
  ctx.sync();
  const double t3 = wall();
  st.e0 = lres.gs_eng;
  st.last = actual;
  if (log)
    log->push_back({target, lres.gs_eng, sres.trunc_err, sres.D, lres.iters, sres.ee, t1 - t0,
                    t2 - t1, t3 - t2, t3 - t0, mvflops, 0, 0, -1.0, 0});
  if (noise_log) noise_log->push_back(expand ? st.noise : 0.0);
}

}  // namespace

double two_site_finite_vmps_noise(Ctx &ctx, std::vector<TensorPtr> &mps,
                                  const std::vector<const BTensor *> &mpo, const SweepParams &p,
                                  const NoiseParams &np, std::vector<SiteLog> *log,
                                  std::vector<double> *noise_log) {
  if (np.noises.empty()) return two_site_finite_vmps(ctx, mps, mpo, p, log, nullptr);
  const int64_t N = (int64_t)mps.size();
  UDMRG_REQUIRE(N >= 4 && (int64_t)mpo.size() == N,
                "noise vmps: MPS and MPO sizes differ or N < 4");
  UDMRG_REQUIRE(p.svd_mode == kSvdExact, "noise vmps: the exact SVD only");
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
  const auto [left, right] = boundaries(ctx, mps, p.Dmax);
  std::vector<TensorPtr> lenvs(N), renvs(N);
  lenvs[0] = trivial_lenv(ctx, *mps[0], *W[0]);
  for (int64_t i = 0; i < left; ++i) lenvs[i + 1] = update_site_lenv(ctx, *lenvs[i], *mps[i], *W[i]);
  renvs[0] = trivial_renv(ctx, *mps[N - 1], *W[N - 1]);
  for (int64_t k = 1; k < N - left - 1; ++k)
    renvs[k] = update_site_renv(ctx, *renvs[k - 1], *mps[N - k], *W[N - k]);
  NoiseState st;
  st.noise = np.noises[0];
  double e0 = 0.0;
  for (int64_t s = 0; s < p.sweeps; ++s) {
    if (s < (int64_t)np.noises.size()) st.noise = np.noises[s];
    st.e0 = 0.0;
    st.last = 0.0;
    for (int64_t i = left; i < right - 1; ++i)
      noise_update(ctx, mps, lenvs, renvs, W, p, np, 'r', i, st, log, noise_log);
    for (int64_t i = right; i > left + 1; --i)
      noise_update(ctx, mps, lenvs, renvs, W, p, np, 'l', i, st, log, noise_log);
    e0 = st.e0;
  }
  return e0;
}

}  // namespace udmrg
