// Grouped block-GEMM kernels, FP64 and complex128 (the plain FP64 form), and
// the same GEMMs in double-word FP32 arithmetic (FP64 data in and out).
//
// A persistent grid walks a list of output tiles (BM x BN); each tile loops
// over the K-segments of its problem and over K in BK chunks, stages A and B
// chunks in shared memory (any strides, see gemm.hpp) and accumulates in
// registers (TM x TN per thread).  The epilogue writes C = alpha*acc (+beta*C)
// once, so no output element is touched by two CTAs and results do not depend
// on scheduling.
//
// Double-word form: this GPU issues about two FP64 FMAs per clock per SM but
// 128 FP32 operations.  Each FP64 operand is staged as an unevaluated sum
// hi + lo of two floats (hi = x rounded to 24 bits, lo = the remainder rounded
// to 24 bits: 48 significant bits), split with integer instructions only.  A
// multiply-add takes the exact product of the high parts (a multiply and an
// FMA), the two cross terms, and adds the product into the accumulator's
// high part with the error-free TwoSum (Knuth), all low-order terms going
// into the accumulator's low part; the pair is renormalised (Fast2Sum,
// Dekker) after every K chunk, so the low part stays below an ulp of the high
// part.  Relative error of a dot product about (1 + sqrt(K / BK)) 2^-48, far
// below what the mixed solver's FP64 anchor needs.  Operands below 2^-102 in
// magnitude keep only their high part, below 2^-126 they count as zero.
#include "gemm.hpp"

namespace udmrg {

namespace {

struct Cplx {
  double x, y;
};

// double-word: value hi + lo with |lo| <= ulp(hi) / 2 after renormalisation
struct DW {
  float hi, lo;
};

__device__ __forceinline__ void fma_acc(double &acc, double a, double b) { acc = fma(a, b, acc); }
__device__ __forceinline__ void fma_acc(Cplx &acc, Cplx a, Cplx b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
// acc += a * b in double-word arithmetic (explicitly rounded operations: no
// contraction into FMAs that would break the error-free transformations)
__device__ __forceinline__ void fma_acc(DW &acc, DW a, DW b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float pe = __fmaf_rn(a.hi, b.hi, -p);                      // a.hi b.hi - p, exact
  const float cross = __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi));
  const float s = __fadd_rn(acc.hi, p);                             // TwoSum(acc.hi, p)
  const float bb = __fsub_rn(s, acc.hi);
  const float err = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(err, __fadd_rn(pe, cross)));
}
__device__ __forceinline__ void renorm(double &) {}
__device__ __forceinline__ void renorm(Cplx &) {}
__device__ __forceinline__ void renorm(DW &a) {  // Fast2Sum(hi, lo)
  const float s = __fadd_rn(a.hi, a.lo);
  a.lo = __fsub_rn(a.lo, __fsub_rn(s, a.hi));
  a.hi = s;
}
__device__ __forceinline__ double zero_of(double) { return 0.0; }
__device__ __forceinline__ Cplx zero_of(Cplx) { return Cplx{0.0, 0.0}; }
__device__ __forceinline__ DW zero_of(DW) { return DW{0.f, 0.f}; }

// FP64 -> double-word with integer instructions (the FP64 <-> FP32
// conversions would run on the FP64 pipe).  x = (H 2^29 + R) 2^(e - 1075) with
// H the significand's leading 24 bits rounded to nearest even and R the
// signed remainder (|R| <= 2^28): hi = H 2^(e - 1046), lo = R 2^(e - 1075).
__device__ __forceinline__ DW df_split(double x) {
  const uint64_t d = (uint64_t)__double_as_longlong(x);
  const uint32_t sign = (uint32_t)(d >> 63) << 31;
  const int e = (int)((d >> 52) & 0x7FF);
  if (e == 0) return DW{__uint_as_float(sign), 0.f};  // zero, FP64 subnormal
  if (e == 0x7FF) return DW{__uint_as_float(sign | 0x7F800000u), 0.f};
  const uint64_t S = (d & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  uint32_t H = (uint32_t)(S >> 29);
  int32_t R = (int32_t)(S & 0x1FFFFFFFull);
  if (R > 0x10000000 || (R == 0x10000000 && (H & 1u))) {
    H += 1u;
    R -= 0x20000000;
  }
  int fe = e - 1023 + 127;  // exponent field of hi
  if (H == 0x1000000u) {
    H = 0x800000u;
    fe += 1;
  }
  if (fe >= 255) return DW{__uint_as_float(sign | 0x7F800000u), 0.f};
  if (fe <= 0) return DW{__uint_as_float(sign), 0.f};
  const float hi = __uint_as_float(sign | ((uint32_t)fe << 23) | (H & 0x7FFFFFu));
  float lo = 0.f;
  if (R != 0) {
    const float r = __int2float_rn(R);  // |R| < 2^29: one rounding to 24 bits
    const int re = (int)((__float_as_uint(r) >> 23) & 0xFFu) + (e - 1075);
    if (re > 0)
      lo = __uint_as_float((uint32_t)((int32_t)__float_as_uint(r) + (e - 1075) * 8388608));
    if (sign) lo = -lo;
  }
  return DW{hi, lo};
}
__device__ __forceinline__ double widen(float v) {  // FP32 -> FP64, integer instructions
  const uint32_t u = __float_as_uint(v);
  const uint64_t sg = (uint64_t)(u >> 31) << 63;
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint64_t m = (uint64_t)(u & 0x7FFFFFu) << 29;
  if (e == 0) {  // FP32 subnormal: exact via the FP64 pipe (rare)
    return (double)v;
  }
  if (e == 0xFFu) return __longlong_as_double((long long)(sg | (0x7FFull << 52) | m));
  return __longlong_as_double((long long)(sg | ((uint64_t)(e + 896u) << 52) | m));
}

// staging: global element -> shared-memory operand
__device__ __forceinline__ double stage(double x, double) { return x; }
__device__ __forceinline__ Cplx stage(Cplx x, Cplx) { return x; }
__device__ __forceinline__ DW stage(double x, DW) { return df_split(x); }
__device__ __forceinline__ double result(double a) { return a; }
__device__ __forceinline__ Cplx result(Cplx a) { return a; }
__device__ __forceinline__ double result(DW a) { return widen(a.hi) + widen(a.lo); }
__device__ __forceinline__ double scale_add(double acc, double alpha, double beta, double c) {
  return beta == 0.0 ? alpha * acc : alpha * acc + beta * c;
}
__device__ __forceinline__ Cplx scale_add(Cplx acc, double alpha, double beta, Cplx c) {
  if (beta == 0.0) return Cplx{alpha * acc.x, alpha * acc.y};
  return Cplx{alpha * acc.x + beta * c.x, alpha * acc.y + beta * c.y};
}

// Offset of a row-major multi-index over n sub-dims.
__device__ __forceinline__ int64_t sub_off(int64_t i, const int32_t *ext, const int64_t *str,
                                           int n) {
  if (n == 1) return i * str[0];
  int64_t off = 0;
  for (int j = n - 1; j >= 0; --j) {
    const int64_t e = ext[j];
    const int64_t q = i / e;
    off += (i - q * e) * str[j];
    i = q;
  }
  return off;
}

// T: the arithmetic (double, Cplx, DW); In: the element type in global memory
template <typename T, typename In, int BM, int BN, int TM, int TN, int BK>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    grouped_gemm_kernel(const GTile *__restrict__ tiles, int ntiles,
                        const GProb *__restrict__ probs, const GSeg *__restrict__ segs,
                        const In *__restrict__ A, const In *__restrict__ B, In *__restrict__ C,
                        double alpha, double beta) {
  constexpr int NT = (BM / TM) * (BN / TN);
  // rows padded by one element: the staging stores of a warp walk K (the
  // rows) when K is the operand's contiguous direction, and unpadded rows of
  // 8-byte elements would all start in the same shared-memory bank
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % (BN / TN);  // column group
  const int ty = tid / (BN / TN);  // row group

  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const GTile tile = tiles[t];
    const GProb p = probs[tile.prob];
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = zero_of(T());

    for (int si = 0; si < p.nseg; ++si) {
      const GSeg s = segs[p.seg0 + si];
      // load mapping: pick the fast index so that global loads are coalesced
      const bool a_kfast = (s.nk > 0 && s.a_ks[s.nk - 1] == 1);
      const bool b_kfast = (s.nk > 0 && s.b_ks[s.nk - 1] == 1);
      for (int k0 = 0; k0 < s.K; k0 += BK) {
        for (int e = tid; e < BM * BK; e += NT) {
          int mm, kk;
          if (a_kfast) {
            kk = e % BK;
            mm = e / BK;
          } else {
            mm = e % BM;
            kk = e / BM;
          }
          const int m = tile.m0 + mm, k = k0 + kk;
          T v = zero_of(T());
          if (m < p.M && k < s.K)
            v = stage(A[s.a_off + sub_off(m, p.m_ext, s.a_ms, p.nm) +
                        sub_off(k, s.k_ext, s.a_ks, s.nk)],
                      T());
          As[kk][mm] = v;
        }
        for (int e = tid; e < BN * BK; e += NT) {
          int nn, kk;
          if (b_kfast) {
            kk = e % BK;
            nn = e / BK;
          } else {
            nn = e % BN;
            kk = e / BN;
          }
          const int n = tile.n0 + nn, k = k0 + kk;
          T v = zero_of(T());
          if (n < p.N && k < s.K)
            v = stage(B[s.b_off + sub_off(k, s.k_ext, s.b_ks, s.nk) +
                        sub_off(n, p.n_ext, s.b_ns, p.nn)],
                      T());
          Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
          T a[TM], b[TN];
#pragma unroll
          for (int i = 0; i < TM; ++i) a[i] = As[kk][ty * TM + i];
#pragma unroll
          for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx * TN + j];
#pragma unroll
          for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) fma_acc(acc[i][j], a[i], b[j]);
        }
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) renorm(acc[i][j]);
        __syncthreads();
      }
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int m = tile.m0 + ty * TM + i;
      if (m >= p.M) continue;
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int n = tile.n0 + tx * TN + j;
        if (n >= p.N) continue;
        In *cp = C + p.c_off + (int64_t)m * p.N + n;
        *cp = scale_add(result(acc[i][j]), alpha, beta, beta == 0.0 ? zero_of(In()) : *cp);
      }
    }
  }
}

template <typename T, typename In, int BM, int BN, int TM, int TN, int BK>
void launch_cfg(Ctx &ctx, const GemmPlan &plan, int cfg, const In *a, const In *b, In *c,
                double alpha, double beta) {
  const int ntiles = (int)plan.tiles[cfg].size();
  if (ntiles == 0) return;
  constexpr int NT = (BM / TM) * (BN / TN);
  int per_sm = 0;
  UDMRG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, grouped_gemm_kernel<T, In, BM, BN, TM, TN, BK>, NT, 0));
  const int grid = std::min(ntiles, std::max(1, per_sm) * ctx.num_sms);
  grouped_gemm_kernel<T, In, BM, BN, TM, TN, BK><<<grid, NT, 0, ctx.stream>>>(
      plan.d_tiles[cfg], ntiles, plan.d_probs, plan.d_segs, a, b, c, alpha, beta);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

template <typename T, typename In>
void run_typed(Ctx &ctx, const GemmPlan &plan, const In *a, const In *b, In *c, double alpha,
               double beta) {
  // K chunk: 16 for 8-byte operands, 8 for complex (keeps static shared memory < 48 KB)
  constexpr int BK = sizeof(T) == 8 ? 16 : 8;
  launch_cfg<T, In, 64, 64, 4, 4, BK>(ctx, plan, kCfg64x64, a, b, c, alpha, beta);
  launch_cfg<T, In, 256, 16, 4, 4, BK>(ctx, plan, kCfg256x16, a, b, c, alpha, beta);
  launch_cfg<T, In, 16, 256, 4, 4, BK>(ctx, plan, kCfg16x256, a, b, c, alpha, beta);
  launch_cfg<T, In, 32, 32, 2, 2, BK>(ctx, plan, kCfg32x32, a, b, c, alpha, beta);
}

}  // namespace

void run_gemm(Ctx &ctx, const GemmPlan &plan, DType dt, const double *a, const double *b,
              double *c, double alpha, double beta) {
  if (dt == kF64)
    run_typed<double, double>(ctx, plan, a, b, c, alpha, beta);
  else
    run_typed<Cplx, Cplx>(ctx, plan, (const Cplx *)a, (const Cplx *)b, (Cplx *)c, alpha, beta);
}

void run_gemm_dw(Ctx &ctx, const GemmPlan &plan, DType dt, const double *a, const double *b,
                 double *c, double alpha, double beta) {
  if (dt == kF64)
    run_typed<DW, double>(ctx, plan, a, b, c, alpha, beta);
  else  // complex data: the FP64 pipe
    run_typed<Cplx, Cplx>(ctx, plan, (const Cplx *)a, (const Cplx *)b, (Cplx *)c, alpha, beta);
}

}  // namespace udmrg
