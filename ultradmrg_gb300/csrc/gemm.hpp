// Grouped block-GEMM: descriptors shared by the planner and the kernels.
//
// One "problem" is one output block C (row-major M x N, contiguous) that
// accumulates over a list of "segments"; a segment is one (A block, B block)
// pair whose product contributes to C.  M, N and K are each a product of up to
// kMaxSub sub-dimensions (tensor axes), so a block contraction over any axes
// is a GEMM without materialised permutations:
//   A(m, k) = A[a_off + sum_j m_j a_ms[j] + sum_j k_j a_ks[j]]
//   B(k, n) = B[b_off + sum_j k_j b_ks[j] + sum_j n_j b_ns[j]]
// with m, n, k decomposed row-major over their sub-dimension extents.
#pragma once

#include "btensor.hpp"

namespace udmrg {

constexpr int kMaxSub = 4;

struct GSeg {
  int64_t a_off, b_off;
  int64_t a_ms[kMaxSub];
  int64_t b_ns[kMaxSub];
  int64_t a_ks[kMaxSub];
  int64_t b_ks[kMaxSub];
  int32_t k_ext[kMaxSub];
  int32_t nk, K;
};

struct GProb {
  int64_t c_off;
  int32_t M, N;
  int32_t m_ext[kMaxSub];
  int32_t n_ext[kMaxSub];
  int32_t nm, nn;
  int32_t seg0, nseg;
};

struct GTile {
  int32_t prob, m0, n0, pad;
};

// Tile configurations of the FP64 kernel (BM x BN output tile).
enum TileCfg : int { kCfg64x64 = 0, kCfg256x16 = 1, kCfg16x256 = 2, kCfg32x32 = 3, kNumCfg = 4 };

struct GemmPlan {
  Ctx *ctx = nullptr;
  std::vector<GSeg> segs;
  std::vector<GProb> probs;
  std::vector<GTile> tiles[kNumCfg];
  double flops = 0;  // algorithmic: sum 2*M*N*K (x4 for complex data)
  int policy = 0;    // tile policy (add_tiles): 0 least padded work, 1 fewer 32 x 32 tiles
  // device copies
  GSeg *d_segs = nullptr;
  GProb *d_probs = nullptr;
  GTile *d_tiles[kNumCfg] = {nullptr, nullptr, nullptr, nullptr};

  GemmPlan() = default;
  GemmPlan(const GemmPlan &) = delete;
  GemmPlan &operator=(const GemmPlan &) = delete;
  ~GemmPlan();
  void upload();
  int64_t ntiles() const {
    int64_t s = 0;
    for (auto &t : tiles) s += (int64_t)t.size();
    return s;
  }
};

// Add a plain strided GEMM problem (one segment, single sub-dims):
//   C[c_off + m*N + n] = sum_k A[a_off + m*a_ms + k*a_ks] * B[b_off + k*b_ks + n*b_ns]
void gemm_add_simple(GemmPlan &g, int64_t c_off, int64_t M, int64_t N, int64_t K, int64_t a_off,
                     int64_t a_ms, int64_t a_ks, int64_t b_off, int64_t b_ks, int64_t b_ns,
                     bool cplx);
// Sort tiles (largest K first) and upload the descriptors.
void gemm_finalize(GemmPlan &g);
// the descriptors of a plan made with upload = false onto the device
void gemm_upload(GemmPlan &g);
// The same problems tiled under another policy (results are bit-identical:
// every output element sums its segments and K in the same order).
void gemm_retile(GemmPlan &g, int policy);
// Square problems whose result is symmetric (Hermitian): drop the tiles
// entirely below the diagonal (the caller mirrors the upper triangle).
void gemm_keep_upper(GemmPlan &g);

// Run C = alpha * A*B (+ beta * C) for every problem of the plan.
void run_gemm(Ctx &ctx, const GemmPlan &plan, DType dt, const double *a, const double *b,
              double *c, double alpha, double beta);
// The same GEMMs of real data in double-word FP32 arithmetic (48-bit
// operands, FP64 in and out; about 2^-48 relative per product); complex data
// on the FP64 pipe.
void run_gemm_dw(Ctx &ctx, const GemmPlan &plan, DType dt, const double *a, const double *b,
                 double *c, double alpha, double beta);

// Contraction of two block tensors.  Output axes: A's free axes in
// a_free_order, then B's free axes in b_free_order.
struct ContractPlan {
  TensorPtr out;  // structure of the result (no data)
  GemmPlan gemm;
};

// upload = false: the GEMM descriptors stay on the host (no device call;
// safe on a host thread) until gemm_upload.
std::unique_ptr<ContractPlan> plan_contract(const BTensor &A, const BTensor &B,
                                            const std::vector<int> &ca, const std::vector<int> &cb,
                                            const std::vector<int> &a_free_order,
                                            const std::vector<int> &b_free_order,
                                            bool upload = true);

// Plan whose output is written into an existing structure `dst` (every block
// the contraction produces must exist in dst).  Blocks of dst that receive no
// contribution are listed in `missing` (block ids) and must be zeroed by the
// caller.
std::unique_ptr<ContractPlan> plan_contract_into(const BTensor &A, const BTensor &B,
                                                 const std::vector<int> &ca,
                                                 const std::vector<int> &cb,
                                                 const std::vector<int> &a_free_order,
                                                 const std::vector<int> &b_free_order,
                                                 const BTensor &dst,
                                                 std::vector<int64_t> *missing,
                                                 bool upload = true);

// Plain-axes contraction (qlten's Contract(A, B, {axes_a, axes_b}, C)).
std::unique_ptr<ContractPlan> plan_contract_axes(const BTensor &A, const BTensor &B,
                                                 const std::vector<int> &ca,
                                                 const std::vector<int> &cb, bool upload = true);
// Cyclic contraction (qlten's Contract<T, Q, a_tail, b_head>(A, B, a_start, b_start, n, C)).
std::unique_ptr<ContractPlan> plan_contract_cyclic(const BTensor &A, const BTensor &B, int a_start,
                                                   int b_start, int n, bool upload = true);
void cyclic_axes(int ra, int rb, int a_start, int b_start, int n, std::vector<int> &ca,
                 std::vector<int> &cb, std::vector<int> &fa, std::vector<int> &fb);

// Block structure (indexes and blocks, no data, no GEMM plan) of a
// contraction's output: the same as the plan's `out`, at a fraction of the
// cost (no segments, tiles or uploads).
TensorPtr contract_struct(const BTensor &A, const BTensor &B, const std::vector<int> &ca,
                          const std::vector<int> &cb, const std::vector<int> &fa,
                          const std::vector<int> &fb);

// Execute a plan: allocates the output data.
// dw: the GEMMs of real data in double-word FP32 arithmetic (run_gemm_dw).
TensorPtr run_contract(Ctx &ctx, const ContractPlan &plan, const BTensor &A, const BTensor &B,
                       bool dw = false);

}  // namespace udmrg
