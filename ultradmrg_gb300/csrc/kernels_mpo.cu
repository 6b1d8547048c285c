// MPO step of the mixed-precision matvec: T3 = (W1 W2) T1 on CUDA cores,
// grouped by (A', B) sector pair.  One CTA takes a pair and a chunk of a'
// rows; for every 32-wide tile of the contiguous b index it stages all input
// channels of the pair in shared memory (each T1 entry is read once), then
// each warp produces output channels (lanes over b) as FP32 dot products with
// the pair's coefficient matrix, split into three BF16 planes and written into
// the step-3 tile images.  HBM bound: T1 read once (FP32), T3 written once
// (3 x BF16).
#include <cuda_bf16.h>

#include "sg_matvec.hpp"

namespace udmrg {

namespace {

constexpr int kAChunk = 8;  // a' rows per work unit (matches the planner)
constexpr int kThreads = 256;

__device__ __forceinline__ int canon(int r, int k, int tr) {
  return (((k >> 3) * (tr >> 3) + (r >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1);
}

__global__ void __launch_bounds__(kThreads)
    mpo_pair_kernel(const int32_t *__restrict__ units, int nunits,
                    const MpoPair *__restrict__ pairs, const MpoIn *__restrict__ ins,
                    const MpoOut *__restrict__ outs, const int32_t *__restrict__ rowptr,
                    const MpoNz *__restrict__ nz, const float *__restrict__ t1,
                    uint8_t *__restrict__ img) {
  extern __shared__ float sm[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int nwarps = kThreads / 32;
  const int64_t plane = (int64_t)kTcBM * kTcBK * 2;
  for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
    const MpoPair pr = pairs[units[2 * u]];
    const int a0 = units[2 * u + 1];
    float *X = sm;
    const int a1 = min(a0 + kAChunk, pr.da);
    for (int a = a0; a < a1; ++a) {
      for (int b0 = 0; b0 < pr.db; b0 += 32) {
        __syncthreads();  // C loaded / previous tile consumed
        for (int e = tid; e < pr.nin * 32; e += kThreads) {
          const int i = e >> 5, b = b0 + (e & 31);
          const MpoIn in = ins[pr.in0 + i];
          X[e] = b < pr.db ? t1[in.base + (int64_t)a * in.astride + b] : 0.f;
        }
        __syncthreads();
        const int b = b0 + lane;
        for (int o = warp; o < pr.nout; o += nwarps) {
          const int k0 = __ldg(rowptr + pr.row0 + o), k1 = __ldg(rowptr + pr.row0 + o + 1);
          float acc = 0.f;
          for (int k = k0; k < k1; ++k) {
            const MpoNz e = nz[k];
            acc = fmaf(e.v, X[(e.i << 5) + lane], acc);
          }
          if (b < pr.db) {
            const MpoOut ot = outs[pr.out0 + o];
            const int row = ot.row0 + a * ot.rstride;
            const int col = ot.col0 + b;
            const int64_t off = ot.img_off +
                                ((int64_t)(row / kTcBM) * ot.kc + col / kTcBK) * 3 * plane +
                                canon(row % kTcBM, col % kTcBK, kTcBM);
            const __nv_bfloat16 h = __float2bfloat16_rn(acc);
            const float r1 = acc - __bfloat162float(h);
            const __nv_bfloat16 m = __float2bfloat16_rn(r1);
            const __nv_bfloat16 l = __float2bfloat16_rn(r1 - __bfloat162float(m));
            *(__nv_bfloat16 *)(img + off) = h;
            *(__nv_bfloat16 *)(img + off + plane) = m;
            *(__nv_bfloat16 *)(img + off + 2 * plane) = l;
          }
        }
      }
    }
  }
}

}  // namespace

void run_mpo_step(Ctx &ctx, const SgMatvecPlan &p) {
  const int nunits = (int)p.units.size() / 2;
  if (nunits == 0) return;
  const size_t smem = (size_t)p.max_nin * 32 * sizeof(float);
  UDMRG_REQUIRE(smem <= 200 * 1024, "mixed matvec: too many MPO input channels in a sector pair");
  static size_t attr = 0;
  if (smem > 48 * 1024 && smem > attr) {
    UDMRG_CHECK_CUDA(cudaFuncSetAttribute(mpo_pair_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = smem;
  }
  const int grid = std::min(nunits, 16 * ctx.num_sms);
  mpo_pair_kernel<<<grid, kThreads, smem, ctx.stream>>>(p.d_units, nunits, p.d_pairs, p.d_ins,
                                                         p.d_outs, p.d_rowptr, p.d_nz, p.t1,
                                                         p.t3_img);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

}  // namespace udmrg
