// MPO step of the mixed-precision matvec: T3 = (W1 W2) T1 on CUDA cores,
// grouped by (A', B) sector pair.  The work unit of one warp is (pair, a',
// 32-wide tile of the contiguous b index): the warp stages the pair's input
// channels for its 32 columns in a warp-private slice of shared memory (each
// T1 entry read once, coalesced), then produces every output channel as an
// FP32 dot product with the pair's CSR coefficient row (lanes over b), splits
// it into three BF16 planes and writes them into the step-3 tile images.
// Units are independent: no block-wide barrier.  HBM bound: T1 read once
// (FP32), T3 written once (3 x BF16).
#include <cuda_bf16.h>

#include "mpo_step.hpp"
#include "sg_matvec.hpp"

namespace udmrg {

namespace {

__device__ __forceinline__ int canon(int r, int k, int tr) {
  return (((k >> 3) * (tr >> 3) + (r >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1);
}

__global__ void mpo_unit_kernel(const int64_t *__restrict__ unit0,
                                const int32_t *__restrict__ unit_pair, int64_t nunits,
                                const MpoPair *__restrict__ pairs, const MpoIn *__restrict__ ins,
                                const MpoOut *__restrict__ outs,
                                const int32_t *__restrict__ rowptr, const MpoNz *__restrict__ nz,
                                const float *__restrict__ t1, uint8_t *__restrict__ img,
                                int slice) {
  extern __shared__ float sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarp = blockDim.x >> 5;
  float *X = sm + (int64_t)warp * slice;  // slice = max input channels x 32
  const int64_t plane = (int64_t)kTcBM * kTcBK * 2;
  for (int64_t u = (int64_t)blockIdx.x * nwarp + warp; u < nunits;
       u += (int64_t)gridDim.x * nwarp) {
    const int lo = __ldg(unit_pair + u);
    const MpoPair pr = pairs[lo];
    const int nbt = (pr.db + 31) >> 5;
    const int64_t local = u - __ldg(unit0 + lo);
    const int a = (int)(local / nbt);
    const int b = (int)(local - (int64_t)a * nbt) * 32 + lane;
    const bool col = b < pr.db;
    for (int i = 0; i < pr.nin; ++i) {
      const MpoIn in = ins[pr.in0 + i];
      X[(i << 5) + lane] = col ? __ldg(t1 + in.base + (int64_t)a * in.astride + b) : 0.f;
    }
    __syncwarp();
    for (int ob = 0; ob < pr.nout; ob += 32) {
      // row pointers of outputs ob .. ob + oc - 1 (lane oo holds output oo's
      // start) and the end pointer of the last one
      const int oc = min(32, pr.nout - ob);
      const int rp = __ldg(rowptr + pr.row0 + ob + min(lane, oc));
      const int rend = __ldg(rowptr + pr.row0 + ob + oc);
      for (int oo = 0; oo < oc; ++oo) {
        const int o = ob + oo;
        const int k0 = __shfl_sync(0xffffffffu, rp, oo);
        const int k1n = __shfl_sync(0xffffffffu, rp, (oo + 1) & 31);
        const int k1 = oo + 1 < oc ? k1n : rend;
        float acc = 0.f;
        // 32 nonzeros per coalesced load, broadcast lane by lane
        for (int kb = k0; kb < k1; kb += 32) {
          const int k = kb + lane;
          int ei = 0;
          float ev = 0.f;
          if (k < k1) {
            const MpoNz e = nz[k];
            ei = e.i;
            ev = e.v;
          }
          const int cnt = min(32, k1 - kb);
#pragma unroll 4
          for (int t = 0; t < cnt; ++t) {
            const int i = __shfl_sync(0xffffffffu, ei, t);
            const float v = __shfl_sync(0xffffffffu, ev, t);
            acc = fmaf(v, X[(i << 5) + lane], acc);
          }
        }
        if (col) {
          const MpoOut ot = outs[pr.out0 + o];
          const int row = ot.row0 + a * ot.rstride;
          const int c = ot.col0 + b;
          const int64_t off = ot.img_off +
                              ((int64_t)(row / kTcBM) * ot.kc + c / kTcBK) * 3 * plane +
                              canon(row % kTcBM, c % kTcBK, kTcBM);
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
    __syncwarp();  // X is rewritten by the next unit
  }
}

// FP64 form: the same work units; inputs from T1 and outputs to T3 in their
// block layouts (b contiguous in T1, strided in T3), FP64 accumulation.
__global__ void mpo_unit64_kernel(const int64_t *__restrict__ unit0,
                                  const int32_t *__restrict__ unit_pair, int64_t nunits,
                                  const MpoPair64 *__restrict__ pairs,
                                  const MpoIn64 *__restrict__ ins,
                                  const MpoOut64 *__restrict__ outs,
                                  const int32_t *__restrict__ rowptr,
                                  const MpoNz64 *__restrict__ nz,
                                  const double *__restrict__ t1, double *__restrict__ t3,
                                  int slice) {
  extern __shared__ double sm64[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarp = blockDim.x >> 5;
  double *X = sm64 + (int64_t)warp * slice;  // slice = max input channels x 32
  for (int64_t u = (int64_t)blockIdx.x * nwarp + warp; u < nunits;
       u += (int64_t)gridDim.x * nwarp) {
    const int lo = __ldg(unit_pair + u);
    const MpoPair64 pr = pairs[lo];
    const int nbt = (pr.db + 31) >> 5;
    const int64_t local = u - __ldg(unit0 + lo);
    const int a = (int)(local / nbt);
    const int b = (int)(local - (int64_t)a * nbt) * 32 + lane;
    const bool col = b < pr.db;
    for (int i = 0; i < pr.nin; ++i) {
      const MpoIn64 in = ins[pr.in0 + i];
      X[(i << 5) + lane] = col ? __ldg(t1 + in.base + (int64_t)a * in.astride + b) : 0.0;
    }
    __syncwarp();
    for (int o = 0; o < pr.nout; ++o) {
      const int k0 = __ldg(rowptr + pr.row0 + o), k1 = __ldg(rowptr + pr.row0 + o + 1);
      double acc = 0.0;
      for (int k = k0; k < k1; ++k) {
        const MpoNz64 e = nz[k];
        acc = fma(e.v, X[(e.i << 5) + lane], acc);
      }
      if (col) {
        const MpoOut64 ot = outs[pr.out0 + o];
        t3[ot.base + (int64_t)a * ot.astride + (int64_t)b * ot.bstride] = acc;
      }
    }
    __syncwarp();  // X is rewritten by the next unit
  }
}

}  // namespace

void run_mpo_step64(Ctx &ctx, const MpoStep64 &p, const double *t1, double *t3) {
  if (p.pairs.empty()) return;
  const int64_t nunits = p.unit0.back();
  if (nunits == 0) return;
  const int slice = std::max(1, p.max_nin) * 32;
  const size_t per_warp = (size_t)slice * sizeof(double);
  UDMRG_REQUIRE(per_warp <= 200 * 1024, "MPO step: too many input channels in a pair");
  const int warps = (int)std::max<size_t>(1, std::min<size_t>(8, (96 * 1024) / per_warp));
  const size_t smem = per_warp * warps;
  static size_t attr = 0;
  if (smem > 48 * 1024 && smem > attr) {
    UDMRG_CHECK_CUDA(cudaFuncSetAttribute(mpo_unit64_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = smem;
  }
  const int64_t blocks = (nunits + warps - 1) / warps;
  const int grid = (int)std::min<int64_t>(blocks, 16 * (int64_t)ctx.num_sms);
  mpo_unit64_kernel<<<grid, 32 * warps, smem, ctx.stream>>>(
      p.d_unit0, p.d_unit_pair, nunits, p.d_pairs, p.d_ins, p.d_outs, p.d_rowptr, p.d_nz, t1, t3,
      slice);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

void run_mpo_step(Ctx &ctx, const SgMatvecPlan &p) {
  const int npairs = (int)p.pairs.size();
  if (npairs == 0) return;
  const int64_t nunits = p.unit0.back();
  if (nunits == 0) return;
  const int slice = std::max(1, p.max_nin) * 32;
  const size_t per_warp = (size_t)slice * sizeof(float);
  UDMRG_REQUIRE(per_warp <= 200 * 1024, "mixed matvec: too many MPO input channels in a pair");
  const int warps = (int)std::max<size_t>(1, std::min<size_t>(8, (96 * 1024) / per_warp));
  const size_t smem = per_warp * warps;
  static size_t attr = 0;
  if (smem > 48 * 1024 && smem > attr) {
    UDMRG_CHECK_CUDA(cudaFuncSetAttribute(mpo_unit_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = smem;
  }
  const int64_t blocks = (nunits + warps - 1) / warps;
  const int grid = (int)std::min<int64_t>(blocks, 16 * (int64_t)ctx.num_sms);
  mpo_unit_kernel<<<grid, 32 * warps, smem, ctx.stream>>>(p.d_unit0, p.d_unit_pair, nunits,
                                                          p.d_pairs,
                                                          p.d_ins, p.d_outs, p.d_rowptr, p.d_nz,
                                                          p.t1, p.t3_img, slice);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

}  // namespace udmrg
