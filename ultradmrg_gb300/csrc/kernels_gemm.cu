// Grouped block-GEMM kernels, FP64 and complex128 (the plain FP64 form).
//
// A persistent grid walks a list of output tiles (BM x BN); each tile loops
// over the K-segments of its problem and over K in BK chunks, stages A and B
// chunks in shared memory (any strides, see gemm.hpp) and accumulates in
// registers (TM x TN per thread).  The epilogue writes C = alpha*acc (+beta*C)
// once, so no output element is touched by two CTAs and results do not depend
// on scheduling.
#include "gemm.hpp"

namespace udmrg {

namespace {

struct Cplx {
  double x, y;
};

__device__ __forceinline__ void fma_acc(double &acc, double a, double b) { acc = fma(a, b, acc); }
__device__ __forceinline__ void fma_acc(Cplx &acc, Cplx a, Cplx b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ double zero_of(double) { return 0.0; }
__device__ __forceinline__ Cplx zero_of(Cplx) { return Cplx{0.0, 0.0}; }
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

template <typename T, int BM, int BN, int TM, int TN, int BK>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    grouped_gemm_kernel(const GTile *__restrict__ tiles, int ntiles,
                        const GProb *__restrict__ probs, const GSeg *__restrict__ segs,
                        const T *__restrict__ A, const T *__restrict__ B, T *__restrict__ C,
                        double alpha, double beta) {
  constexpr int NT = (BM / TM) * (BN / TN);
  __shared__ T As[BK][BM];
  __shared__ T Bs[BK][BN];
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
            v = A[s.a_off + sub_off(m, p.m_ext, s.a_ms, p.nm) + sub_off(k, s.k_ext, s.a_ks, s.nk)];
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
            v = B[s.b_off + sub_off(k, s.k_ext, s.b_ks, s.nk) + sub_off(n, p.n_ext, s.b_ns, p.nn)];
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
        T *cp = C + p.c_off + (int64_t)m * p.N + n;
        *cp = scale_add(acc[i][j], alpha, beta, beta == 0.0 ? zero_of(T()) : *cp);
      }
    }
  }
}

template <typename T, int BM, int BN, int TM, int TN, int BK>
void launch_cfg(Ctx &ctx, const GemmPlan &plan, int cfg, const T *a, const T *b, T *c,
                double alpha, double beta) {
  const int ntiles = (int)plan.tiles[cfg].size();
  if (ntiles == 0) return;
  constexpr int NT = (BM / TM) * (BN / TN);
  int per_sm = 0;
  UDMRG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, grouped_gemm_kernel<T, BM, BN, TM, TN, BK>, NT, 0));
  const int grid = std::min(ntiles, std::max(1, per_sm) * ctx.num_sms);
  grouped_gemm_kernel<T, BM, BN, TM, TN, BK><<<grid, NT, 0, ctx.stream>>>(
      plan.d_tiles[cfg], ntiles, plan.d_probs, plan.d_segs, a, b, c, alpha, beta);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

template <typename T>
void run_typed(Ctx &ctx, const GemmPlan &plan, const T *a, const T *b, T *c, double alpha,
               double beta) {
  // K chunk: 16 for real data, 8 for complex (keeps static shared memory < 48 KB)
  constexpr int BK = sizeof(T) == 8 ? 16 : 8;
  launch_cfg<T, 64, 64, 4, 4, BK>(ctx, plan, kCfg64x64, a, b, c, alpha, beta);
  launch_cfg<T, 256, 16, 4, 4, BK>(ctx, plan, kCfg256x16, a, b, c, alpha, beta);
  launch_cfg<T, 16, 256, 4, 4, BK>(ctx, plan, kCfg16x256, a, b, c, alpha, beta);
  launch_cfg<T, 32, 32, 2, 2, BK>(ctx, plan, kCfg32x32, a, b, c, alpha, beta);
}

}  // namespace

void run_gemm(Ctx &ctx, const GemmPlan &plan, DType dt, const double *a, const double *b,
              double *c, double alpha, double beta) {
  if (dt == kF64)
    run_typed<double>(ctx, plan, a, b, c, alpha, beta);
  else
    run_typed<Cplx>(ctx, plan, (const Cplx *)a, (const Cplx *)b, (Cplx *)c, alpha, beta);
}

}  // namespace udmrg
