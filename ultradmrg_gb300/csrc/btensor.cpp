#include "btensor.hpp"

#include <algorithm>
#include <cstring>
#include <numeric>

namespace udmrg {

Ctx::Ctx(int dev) : device(dev) {
  UDMRG_CHECK_CUDA(cudaSetDevice(dev));
  UDMRG_CHECK_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  UDMRG_CHECK_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  UDMRG_CHECK_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
  // keep freed blocks in the pool instead of returning them to the driver
  cudaMemPool_t pool;
  UDMRG_CHECK_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
  uint64_t thr = UINT64_MAX;
  UDMRG_CHECK_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  host_scratch(1024);
}

Ctx::~Ctx() {
  if (stream) {
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
  }
  if (side) {
    cudaStreamSynchronize(side);
    cudaStreamDestroy(side);
  }
  if (pinned) cudaFreeHost(pinned);
}

void *Ctx::alloc(size_t bytes) {
  if (bytes == 0) return nullptr;
  void *p = nullptr;
  UDMRG_CHECK_CUDA(cudaMallocAsync(&p, bytes, stream));
  return p;
}

void Ctx::free(void *p) {
  if (p) cudaFreeAsync(p, stream);
}

void Ctx::sync() { UDMRG_CHECK_CUDA(cudaStreamSynchronize(stream)); }

double *Ctx::host_scratch(size_t n) {
  if (n > pinned_cap) {
    if (pinned) {
      UDMRG_CHECK_CUDA(cudaStreamSynchronize(stream));
      cudaFreeHost(pinned);
    }
    size_t cap = std::max<size_t>(n, 2 * pinned_cap);
    UDMRG_CHECK_CUDA(cudaMallocHost(&pinned, cap * sizeof(double)));
    pinned_cap = cap;
  }
  return pinned;
}

BTensor::~BTensor() {
  if (owns && data && ctx) ctx->free(data);
}

QN BTensor::block_div(const int32_t *k) const {
  QN q;
  for (int i = 0; i < rank(); ++i) q = q + idx[i].qns[k[i]].scaled(idx[i].dir);
  return q;
}

QN BTensor::div() const {
  if (nblocks() == 0) return QN();
  return block_div(key(0));
}

void BTensor::build_lookup() const {
  lookup_.clear();
  lookup_.reserve((size_t)nblocks() * 2);
  const int r = rank();
  for (int64_t b = 0; b < nblocks(); ++b)
    lookup_.emplace(std::vector<int32_t>(key(b), key(b) + r), b);
  lookup_built_ = true;
}

int64_t BTensor::find(const std::vector<int32_t> &k) const {
  if (!lookup_built_) build_lookup();
  auto it = lookup_.find(k);
  return it == lookup_.end() ? -1 : it->second;
}

std::vector<int32_t> sort_keys(const std::vector<int32_t> &flat, int rank) {
  const int64_t n = rank ? (int64_t)flat.size() / rank : 0;
  std::vector<int64_t> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  auto less = [&](int64_t a, int64_t b) {
    return std::lexicographical_compare(flat.begin() + a * rank, flat.begin() + (a + 1) * rank,
                                        flat.begin() + b * rank, flat.begin() + (b + 1) * rank);
  };
  std::sort(ord.begin(), ord.end(), less);
  std::vector<int32_t> out;
  out.reserve(flat.size());
  for (int64_t i = 0; i < n; ++i) {
    if (i > 0 && !less(ord[i - 1], ord[i])) continue;  // duplicate
    out.insert(out.end(), flat.begin() + ord[i] * rank, flat.begin() + (ord[i] + 1) * rank);
  }
  return out;
}

void BTensor::set_blocks(std::vector<int32_t> sorted) {
  keys = std::move(sorted);
  const int r = rank();
  const int64_t nb = nblocks();
  offs.assign(nb + 1, 0);
  for (int64_t b = 0; b < nb; ++b) {
    int64_t e = 1;
    for (int i = 0; i < r; ++i) {
      int32_t s = keys[b * r + i];
      UDMRG_REQUIRE(s >= 0 && s < idx[i].nsec(), "block sector id out of range");
      e *= idx[i].dims[s];
    }
    offs[b + 1] = offs[b] + e;
  }
  lookup_built_ = false;
}

void BTensor::alloc_data() {
  if (data && owns) ctx->free(data);
  data = (double *)ctx->alloc(bytes());
  owns = true;
}

void BTensor::zero_data() {
  if (data && size()) UDMRG_CHECK_CUDA(cudaMemsetAsync(data, 0, bytes(), ctx->stream));
}

std::unique_ptr<BTensor> BTensor::clone_struct() const {
  auto t = std::make_unique<BTensor>();
  t->ctx = ctx;
  t->dtype = dtype;
  t->nq = nq;
  t->idx = idx;
  t->keys = keys;
  t->offs = offs;
  return t;
}

std::unique_ptr<BTensor> BTensor::clone() const {
  auto t = clone_struct();
  t->alloc_data();
  if (size())
    UDMRG_CHECK_CUDA(cudaMemcpyAsync(t->data, data, bytes(), cudaMemcpyDeviceToDevice, ctx->stream));
  return t;
}

}  // namespace udmrg
