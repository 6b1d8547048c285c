// Matrix-representation MPO (MatReprMPO, one_dim_tn/mpo/mat_repr_mpo.h:21):
// per site a sparse rows x cols matrix whose elements are one-site operators.
#pragma once

#include "btensor.hpp"

namespace udmrg {

struct MatReprSite {
  int64_t rows = 0, cols = 0;
  std::vector<int64_t> x, y;          // coordinates of the non-null elements
  std::vector<const BTensor *> ops;   // operator tensors {pb_in, pb_out}
};

// Without channels that carry no operator on one side of their bond.
std::vector<MatReprSite> prune_dead_channels(const std::vector<MatReprSite> &sites);
// MPO tensors W(lvb IN, pb_in IN, pb_out OUT, rvb OUT) of the same Hamiltonian
// (dead channels pruned first).
std::vector<TensorPtr> mat_repr_to_mpo(Ctx &ctx, const std::vector<MatReprSite> &sites);

}  // namespace udmrg
