// The MPO step of the two-site matvec, T3 = (W1 W2) T1, as a sparse channel
// map on CUDA cores.
//
// In the four-step contraction of eff_ham_mul_two_site_state
// (lanczos_vmps_solver_impl.h:268-272) the two middle steps contract T1 with
// the MPO tensors, whose sector dimensions are a few elements: as GEMMs their
// K and N are tiny and the tiles are mostly padding.  Here the two MPO
// tensors are first contracted over their shared bond (FusedMpo, per target
// sector triple), then every (A', B) sector pair of T1/T3 becomes one small
// dense channel map: out[o](a', b) = sum_i C[o][i] in[i](a', b), applied per
// (a', 32 b) work unit by one warp.
#pragma once

#include <array>
#include <map>

#include "btensor.hpp"

namespace udmrg {

// W1 (w, s1, s1', wr) and W2 (wr, s2, s2', w2) contracted over wr, by the
// output sector triple (S1', S2', W2): the contributing input sectors
// (W, S1, S2) with their dense coefficient matrices coef[ic * nout + oc],
// ic = (w ds1 + s1) ds2 + s2, oc = (s1' ds2' + s2') dw2 + w2.  Host side;
// zero matrices are dropped.  Complex MPO tensors are accepted when every
// imaginary part is zero (an MPO promoted to complex with its state).
struct FusedMpo {
  struct Entry {
    std::array<int32_t, 3> src;  // (W, S1, S2)
    std::vector<double> coef;
  };
  const BTensor &W1, &W2;
  std::vector<double> w1h, w2h;
  std::map<int32_t, std::vector<int64_t>> w1_by_s1o;
  std::map<std::array<int32_t, 3>, std::vector<int64_t>> w2_by;  // (wr, s2', w2)
  std::map<std::array<int32_t, 3>, std::vector<Entry>> cache;
  FusedMpo(Ctx &ctx, const BTensor &W1, const BTensor &W2);
  const std::vector<Entry> &get(int32_t S1p, int32_t S2p, int32_t W2s);
};

// FP64 form.  T1 blocks (A', W, S1, S2, B) and T3 blocks (B, A', S1', S2', W2)
// row-major in their tensors' buffers (the layouts of the grouped-GEMM plans
// of the first and last steps).
struct MpoIn64 {
  int64_t base;     // element offset of channel (w, s1, s2) at (a' = 0, b = 0)
  int64_t astride;  // elements between consecutive a' (b is contiguous)
};
struct MpoOut64 {
  int64_t base;     // element offset of channel (s1', s2', w2) at (a' = 0, b = 0)
  int64_t astride, bstride;
};
struct MpoPair64 {
  int32_t in0, nin, out0, nout;
  int32_t row0, da, db, pad;  // row0: first CSR row of the pair
};
struct MpoNz64 {
  double v;
  int32_t i, pad;
};

struct MpoStep64 {
  Ctx *ctx = nullptr;
  std::vector<MpoPair64> pairs;
  std::vector<MpoIn64> ins;
  std::vector<MpoOut64> outs;
  std::vector<int32_t> rowptr;
  std::vector<MpoNz64> nz;
  std::vector<int64_t> unit0;      // first work unit of each pair (+ total)
  std::vector<int32_t> unit_pair;  // pair of every work unit
  MpoPair64 *d_pairs = nullptr;
  MpoIn64 *d_ins = nullptr;
  MpoOut64 *d_outs = nullptr;
  int32_t *d_rowptr = nullptr;
  MpoNz64 *d_nz = nullptr;
  int64_t *d_unit0 = nullptr;
  int32_t *d_unit_pair = nullptr;
  int max_nin = 0;
  double flops = 0;  // 2 per nonzero coupling and (a', b) entry
  ~MpoStep64();
};

// T1, T3: the block structures of the two outer steps' intermediate tensors.
// Every T3 entry is written (zero where no coupling reaches it).
std::unique_ptr<MpoStep64> plan_mpo_step64(Ctx &ctx, FusedMpo &fm, const BTensor &T1,
                                           const BTensor &T3);
// The same in two parts: the host tables (no device call; safe on a host
// thread with its own FusedMpo), then their upload.
std::unique_ptr<MpoStep64> build_mpo_step64(FusedMpo &fm, const BTensor &T1, const BTensor &T3);
void upload_mpo_step64(Ctx &ctx, MpoStep64 &p);
void run_mpo_step64(Ctx &ctx, const MpoStep64 &p, const double *t1, double *t3);

}  // namespace udmrg
