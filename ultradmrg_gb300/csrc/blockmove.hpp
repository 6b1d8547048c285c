// Index-level rearrangements of block tensors: transpose, fusing two indexes
// into one (FuseIndex), appending blocks along an index (ExpandQNBlocks) and
// index combiners (IndexCombine).  The noise (subspace-expansion) update
// needs them; the tensor library that defines them in the reference
// (TensorToolkit) is not available, so their sector conventions are fixed
// here:
//  * a fused index has one sector per quantum number, in order of first
//    appearance with the first index's sectors running slowest; inside a
//    sector the (first, second) sector pairs come in that order, each pair's
//    elements row-major (first index slowest); dir_f q_f = dir_1 q_1 +
//    dir_2 q_2;
//  * an expanded index keeps the original sectors in order, each followed by
//    the appended part of the same quantum number; new quantum numbers come
//    after, in the appended index's order.
#pragma once

#include <map>

#include "btensor.hpp"

namespace udmrg {

constexpr int kMaxScatterRank = 6;

// Scatter of one source block (row-major over dims) into the destination:
// element x goes to dst_off + sum_k x_k dst_st[k] (element units).
struct BlockScatter {
  int64_t src_off, dst_off;
  int64_t dims[kMaxScatterRank];
  int64_t dst_st[kMaxScatterRank];
  int32_t rank, pad;
};

void run_block_scatter(Ctx &ctx, const std::vector<BlockScatter> &ops, const double *src,
                       double *dst, bool cplx);

struct FusedIndex {
  Index idx;
  std::map<std::pair<int, int>, std::pair<int, int64_t>> where;  // (s1, s2) -> (sector, offset)
};
FusedIndex fuse_index(const Index &i1, const Index &i2, int out_dir);

struct ExpandedIndex {
  Index idx;
  std::vector<std::pair<int, int64_t>> bmap;  // appended sector -> (sector, offset)
};
ExpandedIndex expanded_index(const Index &a, const Index &b);

// Axes permuted: output axis k is input axis perm[k].
TensorPtr permute(Ctx &ctx, const BTensor &T, const std::vector<int> &perm);
// Axes ax1, ax2 fused into a new first index (direction out_dir); the other
// axes follow in order.
TensorPtr fuse_axes(Ctx &ctx, const BTensor &T, int ax1, int ax2, int out_dir);
// T with P's blocks appended along `axis` (P's other indexes equal T's); with
// P == nullptr, zeros whose index along `axis` is `extra`.
TensorPtr expand_axis(Ctx &ctx, const BTensor &T, const BTensor *P, int axis,
                      const Index *extra);
// (i1, i2, f): ones where (x1, x2) meets its place in f; f has direction
// out_dir and dir_f q_f = -(dir_1 q_1 + dir_2 q_2) (divergence zero).
TensorPtr combiner(Ctx &ctx, const Index &i1, const Index &i2, int out_dir, DType dt, int nq);

}  // namespace udmrg
