// FiniteDMRG over a matrix-representation MPO (MatReprMPO).
//
// The reference's FiniteDMRG (algorithm/dmrg/dmrg_impl.h:63-502) keeps, per
// site, a sparse matrix of single-site operators (one-site tensors
// {pb_in, pb_out}) and multiplies the two-site state by
// sum_j sum_k (W_r(j,k) (x) R_k) [sum_i (L_i (x) W_l(i,j)) psi]
// (lanczos_dmrg_solver_impl.h:199-283).  That is the two-site matvec with the
// MPO bond split into channels, so the matrix representation is turned into
// MPO tensors W(lvb IN, pb_in IN, pb_out OUT, rvb OUT) — channels with equal
// quantum number grouped into one bond sector, q(column y) = q(row x) -
// Div(op(x, y)) as in MPOGenerator::CalcTgtRvbQN_ (mpogen_impl.h:356-366) —
// and the sweep runs on the same device kernels.
#include <algorithm>
#include <map>

#include "dmrg.hpp"
#include "matrepr.hpp"

namespace udmrg {

namespace {

// dense host copy of a small tensor (row-major over the full index dimensions)
std::vector<double> dense_host(const BTensor &t) {
  const int es = elem_doubles(t.dtype);
  const int r = t.rank();
  std::vector<int64_t> full(r), stride(r);
  int64_t tot = 1;
  for (int i = r - 1; i >= 0; --i) {
    full[i] = t.idx[i].dim();
    stride[i] = tot;
    tot *= full[i];
  }
  std::vector<double> packed(std::max<int64_t>(t.size(), 1) * es);
  if (t.size() > 0) {
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(packed.data(), t.data, t.size() * es * sizeof(double),
                                     cudaMemcpyDeviceToHost, t.ctx->stream));
    t.ctx->sync();
  }
  std::vector<double> out(tot * es, 0.0);
  for (int64_t b = 0; b < t.nblocks(); ++b) {
    const int32_t *k = t.key(b);
    std::vector<int64_t> off(r), dim(r);
    for (int i = 0; i < r; ++i) {
      int64_t o = 0;
      for (int s = 0; s < k[i]; ++s) o += t.idx[i].dims[s];
      off[i] = o;
      dim[i] = t.idx[i].dims[k[i]];
    }
    const int64_t n = t.block_elems(b);
    for (int64_t e = 0; e < n; ++e) {
      int64_t rem = e, pos = 0;
      for (int i = r - 1; i >= 0; --i) {
        pos += (off[i] + rem % dim[i]) * stride[i];
        rem /= dim[i];
      }
      for (int c = 0; c < es; ++c) out[pos * es + c] = packed[(t.offs[b] + e) * es + c];
    }
  }
  return out;
}

// channel -> (sector, offset) for channels grouped by quantum number (sectors
// in ascending QN order, channels in index order inside a sector)
struct Channels {
  Index idx;
  std::vector<int> sec;
  std::vector<int64_t> off;
};
Channels group_channels(const std::vector<QN> &q, int dir) {
  std::map<QN, std::vector<int>> by;
  for (int c = 0; c < (int)q.size(); ++c) by[q[c]].push_back(c);
  Channels ch;
  ch.idx.dir = dir;
  ch.sec.assign(q.size(), 0);
  ch.off.assign(q.size(), 0);
  for (auto &kv : by) {
    const int s = ch.idx.nsec();
    ch.idx.qns.push_back(kv.first);
    ch.idx.dims.push_back((int64_t)kv.second.size());
    for (size_t j = 0; j < kv.second.size(); ++j) {
      ch.sec[kv.second[j]] = s;
      ch.off[kv.second[j]] = (int64_t)j;
    }
  }
  return ch;
}

}  // namespace

// Channels that carry no operator on one side of their bond (unreachable
// finite-state-machine states near the chain ends) are removed, repeatedly,
// together with the operators that touch them; the rest is renumbered.
std::vector<MatReprSite> prune_dead_channels(const std::vector<MatReprSite> &in) {
  const int64_t N = (int64_t)in.size();
  std::vector<MatReprSite> s = in;
  for (int64_t i = 0; i < N; ++i) {
    UDMRG_REQUIRE(s[i].x.size() == s[i].ops.size() && s[i].y.size() == s[i].ops.size(),
                  "mat-repr MPO: coordinate and operator counts differ");
    for (size_t n = 0; n < s[i].ops.size(); ++n)
      UDMRG_REQUIRE(s[i].x[n] >= 0 && s[i].x[n] < s[i].rows && s[i].y[n] >= 0 &&
                        s[i].y[n] < s[i].cols,
                    "mat-repr MPO: coordinate out of range");
    if (i > 0)
      UDMRG_REQUIRE(s[i].rows == s[i - 1].cols,
                    "mat-repr MPO: rows of a site differ from the columns of the previous one");
  }
  for (bool changed = true; changed;) {
    changed = false;
    // alive[b][c]: channel c of bond b (after site b) has operators on both sides
    for (int64_t b = 0; b + 1 < N; ++b) {
      std::vector<char> left(s[b].cols, 0), right(s[b + 1].rows, 0);
      for (size_t n = 0; n < s[b].ops.size(); ++n) left[s[b].y[n]] = 1;
      for (size_t n = 0; n < s[b + 1].ops.size(); ++n) right[s[b + 1].x[n]] = 1;
      std::vector<int64_t> newid(s[b].cols, -1);
      int64_t k = 0;
      for (int64_t c = 0; c < s[b].cols; ++c)
        if (left[c] && right[c]) newid[c] = k++;
      if (k == s[b].cols) continue;
      changed = true;
      auto remap = [&](MatReprSite &st, bool cols) {
        MatReprSite r;
        r.rows = cols ? st.rows : k;
        r.cols = cols ? k : st.cols;
        for (size_t n = 0; n < st.ops.size(); ++n) {
          const int64_t c = cols ? st.y[n] : st.x[n];
          if (newid[c] < 0) continue;
          r.x.push_back(cols ? st.x[n] : newid[c]);
          r.y.push_back(cols ? newid[c] : st.y[n]);
          r.ops.push_back(st.ops[n]);
        }
        st = std::move(r);
      };
      remap(s[b], true);
      remap(s[b + 1], false);
    }
  }
  return s;
}

std::vector<TensorPtr> mat_repr_to_mpo(Ctx &ctx, const std::vector<MatReprSite> &sites_in) {
  const int64_t N = (int64_t)sites_in.size();
  UDMRG_REQUIRE(N >= 1, "mat-repr MPO: no sites");
  const std::vector<MatReprSite> sites = prune_dead_channels(sites_in);
  std::vector<TensorPtr> out;
  std::vector<QN> qrow;
  for (int64_t i = 0; i < N; ++i) {
    const MatReprSite &st = sites[i];
    UDMRG_REQUIRE(!st.ops.empty(), "mat-repr MPO: a site without operators");
    UDMRG_REQUIRE(st.x.size() == st.ops.size() && st.y.size() == st.ops.size(),
                  "mat-repr MPO: coordinate and operator counts differ");
    const BTensor &op0 = *st.ops[0];
    UDMRG_REQUIRE(op0.rank() == 2, "mat-repr MPO: operators must be {pb_in, pb_out}");
    const Index pb_in = op0.idx[0], pb_out = op0.idx[1];
    bool cplx = false;
    for (auto *o : st.ops) {
      UDMRG_REQUIRE(o->rank() == 2 && o->idx[0] == pb_in && o->idx[1] == pb_out,
                    "mat-repr MPO: operators of one site must share their indexes");
      cplx |= o->dtype == kC128;
    }
    if (i == 0) {
      UDMRG_REQUIRE(st.rows == 1, "mat-repr MPO: the first site must have one row");
      qrow.assign(1, QN{});
      for (int k = 0; k < op0.nq; ++k) qrow[0].v[k] = 0;
    }
    UDMRG_REQUIRE((int64_t)qrow.size() == st.rows,
                  "mat-repr MPO: rows of a site differ from the columns of the previous one");
    std::vector<QN> qcol(st.cols);
    std::vector<char> seen(st.cols, 0);
    for (size_t n = 0; n < st.ops.size(); ++n) {
      UDMRG_REQUIRE(st.x[n] >= 0 && st.x[n] < st.rows && st.y[n] >= 0 && st.y[n] < st.cols,
                    "mat-repr MPO: coordinate out of range");
      if (st.ops[n]->nblocks() == 0) continue;
      const QN q = qrow[st.x[n]] - st.ops[n]->div();
      if (seen[st.y[n]])
        UDMRG_REQUIRE(qcol[st.y[n]] == q, "mat-repr MPO: inconsistent column quantum numbers");
      qcol[st.y[n]] = q;
      seen[st.y[n]] = 1;
    }
    for (int64_t y = 0; y < st.cols; ++y)
      UDMRG_REQUIRE(seen[y], "mat-repr MPO: a column without operators");
    const Channels L = group_channels(qrow, -1), R = group_channels(qcol, +1);
    // assemble the blocks of W on the host
    const int es = cplx ? 2 : 1;
    std::map<std::vector<int32_t>, std::vector<double>> blocks;
    const int64_t din = pb_in.dim(), dout = pb_out.dim();
    std::vector<int> sin(din), sout(dout);
    std::vector<int64_t> oin(din), oout(dout);
    for (int s = 0, p = 0; s < pb_in.nsec(); ++s)
      for (int64_t j = 0; j < pb_in.dims[s]; ++j, ++p) sin[p] = s, oin[p] = j;
    for (int s = 0, p = 0; s < pb_out.nsec(); ++s)
      for (int64_t j = 0; j < pb_out.dims[s]; ++j, ++p) sout[p] = s, oout[p] = j;
    for (size_t n = 0; n < st.ops.size(); ++n) {
      const BTensor &op = *st.ops[n];
      const std::vector<double> m = dense_host(op);
      const int oes = elem_doubles(op.dtype);
      const int64_t x = st.x[n], y = st.y[n];
      for (int64_t a = 0; a < din; ++a)
        for (int64_t b = 0; b < dout; ++b) {
          const double re = m[(a * dout + b) * oes], im = oes == 2 ? m[(a * dout + b) * oes + 1] : 0.0;
          if (re == 0.0 && im == 0.0) continue;
          const std::vector<int32_t> key = {L.sec[x], sin[a], sout[b], R.sec[y]};
          auto &blk = blocks[key];
          const int64_t d0 = L.idx.dims[L.sec[x]], d1 = pb_in.dims[sin[a]],
                        d2 = pb_out.dims[sout[b]], d3 = R.idx.dims[R.sec[y]];
          if (blk.empty()) blk.assign(d0 * d1 * d2 * d3 * es, 0.0);
          const int64_t e = ((L.off[x] * d1 + oin[a]) * d2 + oout[b]) * d3 + R.off[y];
          blk[e * es] += re;
          if (es == 2) blk[e * es + 1] += im;
        }
    }
    auto W = std::make_unique<BTensor>();
    W->ctx = &ctx;
    W->dtype = cplx ? kC128 : kF64;
    W->nq = op0.nq;
    W->idx = {L.idx, pb_in, pb_out, R.idx};
    std::vector<int32_t> keys;
    for (auto &kv : blocks) keys.insert(keys.end(), kv.first.begin(), kv.first.end());
    W->set_blocks(sort_keys(keys, 4));
    W->alloc_data();
    std::vector<double> packed(std::max<int64_t>(W->size(), 1) * es, 0.0);
    for (int64_t b = 0; b < W->nblocks(); ++b) {
      const std::vector<int32_t> key(W->key(b), W->key(b) + 4);
      const auto &blk = blocks.at(key);
      std::copy(blk.begin(), blk.end(), packed.begin() + W->offs[b] * es);
    }
    if (W->size() > 0)
      UDMRG_CHECK_CUDA(cudaMemcpyAsync(W->data, packed.data(), W->size() * es * sizeof(double),
                                       cudaMemcpyHostToDevice, ctx.stream));
    ctx.sync();
    out.push_back(std::move(W));
    qrow = qcol;
  }
  return out;
}

}  // namespace udmrg
