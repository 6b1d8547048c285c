// Common definitions for the GB300 two-site DMRG runtime.
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace udmrg {

// Element types of block data.  Complex is stored interleaved (re, im).
enum DType : int { kF64 = 0, kC128 = 1 };

inline int elem_doubles(DType t) { return t == kC128 ? 2 : 1; }

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// Status codes returned through the C ABI.
enum Status : int {
  kOk = 0,
  kErrInvalid = 1,     // bad argument / inconsistent tensors
  kErrCuda = 2,        // a CUDA runtime call failed
  kErrNumerics = 3,    // LAPACK-like failure (eigensolver did not converge)
  kErrTimeout = 4,     // a bounded device wait ran out
  kErrInternal = 5,
};

#define UDMRG_CHECK_CUDA(expr)                                                   \
  do {                                                                           \
    cudaError_t _e = (expr);                                                     \
    if (_e != cudaSuccess)                                                       \
      throw ::udmrg::Error(::udmrg::kErrCuda, std::string(#expr) + ": " +        \
                                                  cudaGetErrorString(_e));       \
  } while (0)

#define UDMRG_REQUIRE(cond, msg)                                                 \
  do {                                                                           \
    if (!(cond)) throw ::udmrg::Error(::udmrg::kErrInvalid, (msg));              \
  } while (0)

// Quantum number: up to four U(1) charges (U(1): nq=1, U(1)xU(1): nq=2).
constexpr int kMaxQ = 4;
struct QN {
  int32_t v[kMaxQ] = {0, 0, 0, 0};
  bool operator==(const QN &o) const {
    for (int i = 0; i < kMaxQ; ++i)
      if (v[i] != o.v[i]) return false;
    return true;
  }
  bool operator!=(const QN &o) const { return !(*this == o); }
  bool operator<(const QN &o) const {
    for (int i = 0; i < kMaxQ; ++i)
      if (v[i] != o.v[i]) return v[i] < o.v[i];
    return false;
  }
  QN operator+(const QN &o) const {
    QN r;
    for (int i = 0; i < kMaxQ; ++i) r.v[i] = v[i] + o.v[i];
    return r;
  }
  QN operator-(const QN &o) const {
    QN r;
    for (int i = 0; i < kMaxQ; ++i) r.v[i] = v[i] - o.v[i];
    return r;
  }
  QN scaled(int s) const {
    QN r;
    for (int i = 0; i < kMaxQ; ++i) r.v[i] = s * v[i];
    return r;
  }
};

struct QNHash {
  size_t operator()(const QN &q) const {
    uint64_t h = 1469598103934665603ull;
    for (int i = 0; i < kMaxQ; ++i) {
      h ^= (uint64_t)(uint32_t)q.v[i];
      h *= 1099511628211ull;
    }
    return (size_t)h;
  }
};

}  // namespace udmrg
