// 2-norm of a device vector without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need a norm:
// hosts whose device memory is owned by another allocator or fully reserved,
// and latency-critical loops that must not touch the allocator.  For them this file offers udmrg_norm_noalloc, a variant of the
// library's two-stage reduction (the one behind udmrg_tensor_norm) whose
// per-block partial sums live in a fixed, file-scope device array instead of
// a buffer taken from the stream-ordered pool.
//
// Limits and behaviour:
//  * at most kNoAllocMaxDoubles = 16,777,216 doubles per call (4096 blocks of
//    4096 elements); larger inputs are rejected with status 1;
//  * the scratch array (32 KB) is reserved on every GPU that loads the library
//    until the process exits;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it, so make
//    that first call before any stream capture; the cache assumes that the
//    device's primary context lives until the process exits (after
//    cudaDeviceReset the cached address is stale);
//  * devices 0..63 only;
//  * a CUDA error left pending by an earlier call of the caller is reported
//    (status 2) and left in place, not cleared;
//  * all calls share the one array: calls whose kernels overlap on the GPU
//    (different streams without ordering between them) race.
#include <mutex>

#include "../../include/ultradmrg_gb300.h"
#include "common.hpp"

namespace udmrg {
const char *set_last_error_noalloc(const char *msg);
}

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerThread = 16;
constexpr int64_t kNoAllocChunk = (int64_t)kNoAllocThreads * kNoAllocPerThread;  // 4096
constexpr int kNoAllocMaxBlocks = 4096;
constexpr int64_t kNoAllocMaxDoubles = kNoAllocChunk * kNoAllocMaxBlocks;  // 16,777,216
constexpr int kMaxDevices = 64;

// One partial sum per block of the first stage.
static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxBlocks];

std::mutex g_setup_mutex;
double *g_partials_addr[kMaxDevices] = {nullptr};

__global__ void noalloc_sumsq_kernel(const double *__restrict__ x, int64_t n,
                                     double *__restrict__ partials) {
  const int64_t base = (int64_t)blockIdx.x * kNoAllocChunk;
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < kNoAllocPerThread; ++i) {
    const int64_t k = base + (int64_t)i * kNoAllocThreads + threadIdx.x;
    if (k < n) s = fma(x[k], x[k], s);
  }
  __shared__ double sh[kNoAllocThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kNoAllocThreads / 32; ++w) t += sh[w];
    partials[blockIdx.x] = t;
  }
}

__global__ void noalloc_finish_kernel(const double *__restrict__ partials, int nb,
                                      double *__restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partials[i];
  __shared__ double sh[kNoAllocThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kNoAllocThreads / 32; ++w) t += sh[w];
    out[0] = sqrt(t);
  }
}

// Device address of the scratch array for the current device (set up once).
// On failure *msg names the cause.
int partials_for_current_device(double **p, const char **msg) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    *msg = "udmrg_norm_noalloc: cudaGetDevice failed";
    return udmrg::kErrCuda;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    *msg = "udmrg_norm_noalloc: device number above 63 (the address table holds 64 devices)";
    return udmrg::kErrInvalid;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_partials_addr[dev]) {
    double *addr = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress((void **)&addr, g_noalloc_partials);
    if (rc != cudaSuccess || addr == nullptr) {
      *msg = "udmrg_norm_noalloc: cudaGetSymbolAddress of the scratch array failed";
      return udmrg::kErrCuda;
    }
    g_partials_addr[dev] = addr;
  }
  *p = g_partials_addr[dev];
  return udmrg::kOk;
}

}  // namespace

extern "C" int udmrg_norm_noalloc(const double *d_x, int64_t n_doubles, double *d_norm,
                                  void *stream) {
  if (d_norm == nullptr || (n_doubles > 0 && d_x == nullptr) || n_doubles < 0) {
    udmrg::set_last_error_noalloc("udmrg_norm_noalloc: null pointer or negative length");
    return udmrg::kErrInvalid;
  }
  if (n_doubles > kNoAllocMaxDoubles) {
    udmrg::set_last_error_noalloc(
        "udmrg_norm_noalloc: input longer than the 16,777,216-double maximum of the "
        "static scratch");
    return udmrg::kErrInvalid;
  }
  // an error of the caller's own earlier launches is theirs to read: report
  // it without clearing it, so that the launch check below sees only ours
  if (cudaPeekAtLastError() != cudaSuccess) {
    udmrg::set_last_error_noalloc(
        "udmrg_norm_noalloc: a CUDA error from an earlier call is pending (not cleared)");
    return udmrg::kErrCuda;
  }
  double *partials = nullptr;
  const char *msg = nullptr;
  const int st = partials_for_current_device(&partials, &msg);
  if (st != udmrg::kOk) {
    udmrg::set_last_error_noalloc(msg);
    return st;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = (int)((n_doubles + kNoAllocChunk - 1) / kNoAllocChunk);
  if (nb > 0) noalloc_sumsq_kernel<<<nb, kNoAllocThreads, 0, s>>>(d_x, n_doubles, partials);
  noalloc_finish_kernel<<<1, kNoAllocThreads, 0, s>>>(partials, nb, d_norm);
  if (cudaGetLastError() != cudaSuccess) {
    udmrg::set_last_error_noalloc("udmrg_norm_noalloc: kernel launch failed");
    return udmrg::kErrCuda;
  }
  return udmrg::kOk;
}
