// Block-sparse tensor runtime: host metadata, device data.
//
// Storage model (the QLTensor model of QuantumLiquids/TensorToolkit as used
// by qlmps): an Index is an ordered list of QN sectors (qn, dim) plus a
// direction (OUT = +1, IN = -1).  A tensor holds dense blocks keyed by one
// sector id per index; a block may exist only if sum_i dir_i * qn_i == div.
// Blocks are kept sorted lexicographically by their sector-id tuples and
// packed back to back in one device buffer, each block row-major over the
// tensor's axes.
#pragma once

#include <array>
#include <map>
#include <memory>
#include <unordered_map>

#include "common.hpp"

namespace udmrg {

struct Index {
  std::vector<QN> qns;
  std::vector<int64_t> dims;
  int dir = 1;  // +1 OUT, -1 IN
  int nsec() const { return (int)qns.size(); }
  int64_t dim() const {
    int64_t s = 0;
    for (auto d : dims) s += d;
    return s;
  }
  Index inverse() const {
    Index r = *this;
    r.dir = -dir;
    return r;
  }
  bool same_space(const Index &o) const { return qns == o.qns && dims == o.dims; }
  bool operator==(const Index &o) const { return same_space(o) && dir == o.dir; }
  int find(const QN &q) const {
    for (int i = 0; i < nsec(); ++i)
      if (qns[i] == q) return i;
    return -1;
  }
};

// Device context: one GPU, one stream, stream-ordered allocations.
struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // second stream for work that overlaps the main one
  int num_sms = 0;
  // pinned host scratch for small device->host reads
  double *pinned = nullptr;
  size_t pinned_cap = 0;
  // counts of kernels launched by this library through this context
  uint64_t launches = 0;
  // Krylov solvers replay each step as one CUDA graph (captured once per solve)
  bool krylov_graph = true;
  // The mixed solver's FP64-accurate anchor matvec: its two block-GEMM stages
  // in double-word FP32 arithmetic (true) or on the FP64 pipe (false)
  bool anchor_dw = true;
  // Host buffers of udmrg_matvec_plan_apply_host that are page-locked and
  // mapped into the device's address space (cudaMallocHost / cudaHostAlloc /
  // cudaHostRegister) are used in place by the mixed matvec: 0 never (one
  // copy each way through device buffers), 1 the input (the psi pack reads
  // it over the host link), 2 input and output (the .R GEMM's epilogue also
  // writes the result there).  Other host memory is always copied.
  int host_mapped = 0;
  // Set while a mixed-precision update runs its SVD with anchor_dw: the SVD's
  // Newton-Schulz and factor products in double-word arithmetic (its Gram
  // products stay on the FP64 pipe)
  bool svd_dw = false;
  // Mixed matvec: B-tile rows of the tcgen05 GEMMs L.psi (tc_bn1) and .R
  // (tc_bn3), 64 or 128; 0: chosen per plan by timed trials, cached per
  // shape class in tc_tuned (class -> {bn1, bn3}); tc_trials counts them
  int tc_bn1 = 0, tc_bn3 = 0;
  std::map<std::array<int64_t, 3>, std::array<int, 2>> tc_tuned;
  int64_t tc_trials = 0;
  // Grouped FP64 / double-word GEMMs of a two-site matvec's FP64-accurate
  // product: tile policy 0 or 1 (gemm.hpp), or -1: chosen per plan by timed
  // trials, cached per shape class in gemm_tuned; gemm_trials counts them
  int gemm_policy = -1;
  std::map<std::array<int64_t, 4>, int> gemm_tuned;
  int64_t gemm_trials = 0;
  // C-ABI lifetime: live tensor / plan handles on this context; a context
  // whose destroy was requested is deleted when the last handle goes
  int64_t live_handles = 0;
  bool closing = false;
  void *owner = nullptr;  // the C-ABI object that holds this context

  explicit Ctx(int dev);
  ~Ctx();
  void *alloc(size_t bytes);
  void free(void *p);
  void sync();
  double *host_scratch(size_t ndoubles);
};

struct KeyHash {
  size_t operator()(const std::vector<int32_t> &k) const {
    uint64_t h = 1469598103934665603ull;
    for (auto v : k) {
      h ^= (uint64_t)(uint32_t)v;
      h *= 1099511628211ull;
    }
    return (size_t)h;
  }
};

struct BTensor {
  Ctx *ctx = nullptr;
  DType dtype = kF64;
  int nq = 1;
  std::vector<Index> idx;
  std::vector<int32_t> keys;  // nblocks * rank, sorted lexicographically
  std::vector<int64_t> offs;  // element offset of each block (nblocks + 1)
  double *data = nullptr;     // device buffer, offs.back() elements
  bool owns = true;

  BTensor() = default;
  BTensor(const BTensor &) = delete;
  BTensor &operator=(const BTensor &) = delete;
  ~BTensor();

  int rank() const { return (int)idx.size(); }
  int64_t nblocks() const { return rank() ? (int64_t)keys.size() / rank() : 0; }
  int64_t size() const { return offs.empty() ? 0 : offs.back(); }
  const int32_t *key(int64_t b) const { return keys.data() + b * rank(); }
  int64_t block_elems(int64_t b) const { return offs[b + 1] - offs[b]; }
  int64_t dim_of(int64_t b, int axis) const { return idx[axis].dims[key(b)[axis]]; }
  QN block_div(const int32_t *k) const;
  QN div() const;  // divergence of the first block (all blocks agree)

  // block lookup by sector-id tuple (built on demand)
  int64_t find(const std::vector<int32_t> &k) const;
  // builds find's lookup now (find from several host threads at once is safe
  // after this)
  void prepare_lookup() const {
    if (!lookup_built_) build_lookup();
  }
  void build_lookup() const;

  // Set the block list (must be sorted and unique), compute offsets.
  void set_blocks(std::vector<int32_t> sorted_keys);
  void alloc_data();   // allocate (uninitialised) device data for size()
  void zero_data();    // memset device data to 0 (stream ordered)
  size_t bytes() const { return (size_t)size() * elem_doubles(dtype) * sizeof(double); }

  // structure copy without data
  std::unique_ptr<BTensor> clone_struct() const;
  std::unique_ptr<BTensor> clone() const;  // with data (device copy)

 private:
  mutable std::unordered_map<std::vector<int32_t>, int64_t, KeyHash> lookup_;
  mutable bool lookup_built_ = false;
};

using TensorPtr = std::unique_ptr<BTensor>;

// Scope-bound device allocations (freed on every exit path, exceptions included).
struct DeviceScratch {
  Ctx &ctx;
  std::vector<void *> ptrs;
  explicit DeviceScratch(Ctx &c) : ctx(c) {}
  ~DeviceScratch() {
    for (void *p : ptrs) ctx.free(p);
  }
  template <typename T>
  T *get(size_t count) {
    void *p = ctx.alloc(std::max<size_t>(count, 1) * sizeof(T));
    ptrs.push_back(p);
    return (T *)p;
  }
};

// Sort + deduplicate a flat key list (rank-sized tuples).
std::vector<int32_t> sort_keys(const std::vector<int32_t> &flat, int rank);

}  // namespace udmrg
