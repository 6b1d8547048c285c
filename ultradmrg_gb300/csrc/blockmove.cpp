#include "blockmove.hpp"

#include <algorithm>

namespace udmrg {

namespace {

TensorPtr new_tensor(Ctx &ctx, DType dt, int nq, std::vector<Index> idx,
                     const std::vector<int32_t> &flat_keys) {
  auto t = std::make_unique<BTensor>();
  t->ctx = &ctx;
  t->dtype = dt;
  t->nq = nq;
  t->idx = std::move(idx);
  t->set_blocks(sort_keys(flat_keys, t->rank()));
  t->alloc_data();
  t->zero_data();
  return t;
}

// Row-major strides of block b of T.
std::vector<int64_t> strides_of(const BTensor &T, int64_t b) {
  const int r = T.rank();
  std::vector<int64_t> st(r, 1);
  for (int k = r - 2; k >= 0; --k) st[k] = st[k + 1] * T.dim_of(b, k + 1);
  return st;
}

BlockScatter scatter_op(const BTensor &T, int64_t b) {
  BlockScatter op{};
  UDMRG_REQUIRE(T.rank() <= kMaxScatterRank, "block rearrangement: rank above 6");
  op.rank = T.rank();
  op.src_off = T.offs[b];
  for (int k = 0; k < T.rank(); ++k) op.dims[k] = T.dim_of(b, k);
  return op;
}

}  // namespace

FusedIndex fuse_index(const Index &i1, const Index &i2, int out_dir) {
  FusedIndex f;
  f.idx.dir = out_dir;
  for (int s1 = 0; s1 < i1.nsec(); ++s1)
    for (int s2 = 0; s2 < i2.nsec(); ++s2) {
      const QN q = (i1.qns[s1].scaled(i1.dir) + i2.qns[s2].scaled(i2.dir)).scaled(out_dir);
      int fs = f.idx.find(q);
      if (fs < 0) {
        fs = f.idx.nsec();
        f.idx.qns.push_back(q);
        f.idx.dims.push_back(0);
      }
      f.where[{s1, s2}] = {fs, f.idx.dims[fs]};
      f.idx.dims[fs] += i1.dims[s1] * i2.dims[s2];
    }
  return f;
}

ExpandedIndex expanded_index(const Index &a, const Index &b) {
  UDMRG_REQUIRE(a.dir == b.dir, "expand: the appended index has the other direction");
  ExpandedIndex e;
  e.idx = a;
  for (int s = 0; s < b.nsec(); ++s) {
    int t = e.idx.find(b.qns[s]);
    if (t < 0) {
      t = e.idx.nsec();
      e.idx.qns.push_back(b.qns[s]);
      e.idx.dims.push_back(0);
    }
    e.bmap.push_back({t, e.idx.dims[t]});
    e.idx.dims[t] += b.dims[s];
  }
  return e;
}

TensorPtr permute(Ctx &ctx, const BTensor &T, const std::vector<int> &perm) {
  const int r = T.rank();
  UDMRG_REQUIRE((int)perm.size() == r, "permute: permutation length");
  std::vector<Index> idx(r);
  for (int k = 0; k < r; ++k) idx[k] = T.idx[perm[k]];
  std::vector<int32_t> flat;
  for (int64_t b = 0; b < T.nblocks(); ++b)
    for (int k = 0; k < r; ++k) flat.push_back(T.key(b)[perm[k]]);
  auto out = new_tensor(ctx, T.dtype, T.nq, idx, flat);
  std::vector<BlockScatter> ops;
  for (int64_t b = 0; b < T.nblocks(); ++b) {
    std::vector<int32_t> k(r);
    for (int j = 0; j < r; ++j) k[j] = T.key(b)[perm[j]];
    const int64_t ob = out->find(k);
    const auto st = strides_of(*out, ob);
    BlockScatter op = scatter_op(T, b);
    op.dst_off = out->offs[ob];
    for (int j = 0; j < r; ++j) op.dst_st[perm[j]] = st[j];
    ops.push_back(op);
  }
  run_block_scatter(ctx, ops, T.data, out->data, T.dtype == kC128);
  return out;
}

TensorPtr fuse_axes(Ctx &ctx, const BTensor &T, int ax1, int ax2, int out_dir) {
  const int r = T.rank();
  UDMRG_REQUIRE(ax1 != ax2 && ax1 >= 0 && ax2 >= 0 && ax1 < r && ax2 < r, "fuse: axes");
  const FusedIndex f = fuse_index(T.idx[ax1], T.idx[ax2], out_dir);
  std::vector<int> rest;
  for (int k = 0; k < r; ++k)
    if (k != ax1 && k != ax2) rest.push_back(k);
  std::vector<Index> idx = {f.idx};
  for (int k : rest) idx.push_back(T.idx[k]);
  std::vector<int32_t> flat;
  std::vector<std::vector<int32_t>> okeys;
  for (int64_t b = 0; b < T.nblocks(); ++b) {
    std::vector<int32_t> k = {f.where.at({T.key(b)[ax1], T.key(b)[ax2]}).first};
    for (int j : rest) k.push_back(T.key(b)[j]);
    flat.insert(flat.end(), k.begin(), k.end());
    okeys.push_back(k);
  }
  auto out = new_tensor(ctx, T.dtype, T.nq, idx, flat);
  std::vector<BlockScatter> ops;
  for (int64_t b = 0; b < T.nblocks(); ++b) {
    const int64_t ob = out->find(okeys[b]);
    const auto st = strides_of(*out, ob);  // st[0]: the fused axis
    const int64_t off = f.where.at({T.key(b)[ax1], T.key(b)[ax2]}).second;
    BlockScatter op = scatter_op(T, b);
    op.dst_off = out->offs[ob] + off * st[0];
    op.dst_st[ax1] = T.dim_of(b, ax2) * st[0];
    op.dst_st[ax2] = st[0];
    for (size_t j = 0; j < rest.size(); ++j) op.dst_st[rest[j]] = st[j + 1];
    ops.push_back(op);
  }
  run_block_scatter(ctx, ops, T.data, out->data, T.dtype == kC128);
  return out;
}

TensorPtr expand_axis(Ctx &ctx, const BTensor &T, const BTensor *P, int axis,
                      const Index *extra) {
  const int r = T.rank();
  UDMRG_REQUIRE(axis >= 0 && axis < r, "expand: axis");
  UDMRG_REQUIRE(P || extra, "expand: nothing to append");
  if (P) {
    UDMRG_REQUIRE(P->rank() == r && P->dtype == T.dtype, "expand: tensors differ");
    for (int k = 0; k < r; ++k)
      UDMRG_REQUIRE(k == axis || P->idx[k] == T.idx[k], "expand: indexes differ off the axis");
  }
  const ExpandedIndex e = expanded_index(T.idx[axis], P ? P->idx[axis] : *extra);
  std::vector<Index> idx = T.idx;
  idx[axis] = e.idx;
  std::vector<int32_t> flat(T.keys);
  if (P) flat.insert(flat.end(), P->keys.begin(), P->keys.end());
  if (P)
    for (int64_t b = 0; b < P->nblocks(); ++b)
      flat[T.keys.size() + b * r + axis] = e.bmap[P->key(b)[axis]].first;
  auto out = new_tensor(ctx, T.dtype, T.nq, idx, flat);
  auto place = [&](const BTensor &S, int64_t b, int sec, int64_t off,
                   std::vector<BlockScatter> &ops) {
    std::vector<int32_t> k(S.key(b), S.key(b) + r);
    k[axis] = sec;
    const int64_t ob = out->find(k);
    const auto st = strides_of(*out, ob);
    BlockScatter op = scatter_op(S, b);
    op.dst_off = out->offs[ob] + off * st[axis];
    for (int j = 0; j < r; ++j) op.dst_st[j] = st[j];
    ops.push_back(op);
  };
  std::vector<BlockScatter> ops;
  for (int64_t b = 0; b < T.nblocks(); ++b) place(T, b, T.key(b)[axis], 0, ops);
  run_block_scatter(ctx, ops, T.data, out->data, T.dtype == kC128);
  if (P) {
    ops.clear();
    for (int64_t b = 0; b < P->nblocks(); ++b) {
      const auto &m = e.bmap[P->key(b)[axis]];
      place(*P, b, m.first, m.second, ops);
    }
    run_block_scatter(ctx, ops, P->data, out->data, T.dtype == kC128);
  }
  return out;
}

TensorPtr combiner(Ctx &ctx, const Index &i1, const Index &i2, int out_dir, DType dt, int nq) {
  FusedIndex F = fuse_index(i1, i2, -out_dir);
  const Index f = F.idx.inverse();
  std::vector<int32_t> flat;
  for (auto &kv : F.where) {
    flat.push_back(kv.first.first);
    flat.push_back(kv.first.second);
    flat.push_back(kv.second.first);
  }
  auto out = new_tensor(ctx, dt, nq, {i1, i2, f}, flat);
  std::vector<double> h((size_t)out->size() * elem_doubles(dt), 0.0);
  const int es = elem_doubles(dt);
  for (auto &kv : F.where) {
    const int s1 = kv.first.first, s2 = kv.first.second;
    const int fs = kv.second.first;
    const int64_t off = kv.second.second;
    const int64_t ob = out->find({s1, s2, fs});
    const int64_t d1 = i1.dims[s1], d2 = i2.dims[s2], df = f.dims[fs];
    for (int64_t x = 0; x < d1; ++x)
      for (int64_t y = 0; y < d2; ++y)
        h[(size_t)(out->offs[ob] + (x * d2 + y) * df + off + x * d2 + y) * es] = 1.0;
  }
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(out->data, h.data(), h.size() * sizeof(double),
                                   cudaMemcpyHostToDevice, ctx.stream));
  ctx.sync();
  return out;
}

}  // namespace udmrg
