// MPO step of the mixed-precision matvec: T3 = (W1 W2) T1 on CUDA cores
// (HBM bound: FP32 reads of T1, split-BF16 writes of the step-3 operand
// images).  One CTA per target block; each thread owns (a', b) positions and
// accumulates all output channels of that position in registers.
#include <cuda_bf16.h>

#include "sg_matvec.hpp"

namespace udmrg {

namespace {

constexpr int kMaxOut = 32;

__device__ __forceinline__ int canon(int r, int k, int tr) {
  return (((k >> 3) * (tr >> 3) + (r >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1);
}

template <int NOUT>
__device__ void target_body(const MpoTarget &tg, const MpoSource *__restrict__ src,
                            const float *__restrict__ coefs, const float *__restrict__ t1,
                            uint8_t *__restrict__ img) {
  const int64_t plane = (int64_t)kTcBM * kTcBK * 2;
  const int npos = tg.da * tg.db;
  for (int e = threadIdx.x; e < npos; e += blockDim.x) {
    const int a = e / tg.db, b = e - a * tg.db;
    float acc[NOUT];
#pragma unroll
    for (int o = 0; o < NOUT; ++o) acc[o] = 0.f;
    for (int s = 0; s < tg.nsrc; ++s) {
      const MpoSource sr = src[tg.src0 + s];
      const float *c = coefs + sr.coef_off;
      const int nin = sr.dw * sr.ds12;
      for (int ic = 0; ic < nin; ++ic) {
        const int w = ic / sr.ds12, s12 = ic - w * sr.ds12;
        const float x =
            t1[sr.t1_off + ((int64_t)a * sr.dw + w) * sr.row_pitch + (int64_t)s12 * tg.db + b];
#pragma unroll
        for (int o = 0; o < NOUT; ++o)
          if (o < tg.nout) acc[o] = fmaf(__ldg(c + ic * tg.nout + o), x, acc[o]);
      }
    }
#pragma unroll
    for (int o = 0; o < NOUT; ++o) {
      if (o >= tg.nout) break;
      const int row = tg.row0 + a * tg.ds12p + o / tg.dw2;
      const int col = tg.k0 + (o % tg.dw2) * tg.db + b;
      const int64_t off = tg.img_off +
                          ((int64_t)(row / kTcBM) * tg.kc + col / kTcBK) * 3 * plane +
                          canon(row % kTcBM, col % kTcBK, kTcBM);
      const float v = acc[o];
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      const float r1 = v - __bfloat162float(h);
      const __nv_bfloat16 m = __float2bfloat16_rn(r1);
      const __nv_bfloat16 l = __float2bfloat16_rn(r1 - __bfloat162float(m));
      *(__nv_bfloat16 *)(img + off) = h;
      *(__nv_bfloat16 *)(img + off + plane) = m;
      *(__nv_bfloat16 *)(img + off + 2 * plane) = l;
    }
  }
}

__global__ void mpo_step_kernel(const MpoTarget *__restrict__ targets, int ntargets,
                                const MpoSource *__restrict__ src,
                                const float *__restrict__ coefs, const float *__restrict__ t1,
                                uint8_t *__restrict__ img) {
  for (int t = blockIdx.x; t < ntargets; t += gridDim.x) {
    const MpoTarget tg = targets[t];
    if (tg.nout <= 4)
      target_body<4>(tg, src, coefs, t1, img);
    else if (tg.nout <= 8)
      target_body<8>(tg, src, coefs, t1, img);
    else if (tg.nout <= 16)
      target_body<16>(tg, src, coefs, t1, img);
    else
      target_body<kMaxOut>(tg, src, coefs, t1, img);
  }
}

}  // namespace

void run_mpo_step(Ctx &ctx, const SgMatvecPlan &p) {
  const int n = (int)p.targets.size();
  if (n == 0) return;
  const int grid = std::min(n, 32 * ctx.num_sms);
  mpo_step_kernel<<<grid, 128, 0, ctx.stream>>>(p.d_targets, n, p.d_sources, p.d_coefs, p.t1,
                                                p.t3_img);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

}  // namespace udmrg
