// MPO step of the mixed-precision matvec: T3 = (W1 W2) T1 on CUDA cores,
// grouped by (A', B) sector pair.  A thread owns one unit (pair, a', 8-wide
// chunk of b): for each output channel of the pair it accumulates the
// coefficient-weighted input chunks (two 16-byte loads of FP32 T1 per
// nonzero, read straight from global memory: an input channel serves ~1.25
// outputs, the second use hits L1), splits the eight sums into three BF16
// planes and writes each plane with one 16-byte store into the step-3 tile
// image.  A warp takes 32 consecutive units of one pair, so the CSR walk over
// the pair's nonzeros is warp-uniform (broadcast metadata loads, no
// divergence).  The pair's nonzero records, channel ends and image targets
// are loaded 32 at a time, one per lane, and shuffled out; nonzeros are
// processed four at a time with their eight loads in flight.  Padded b columns (up to a multiple of 8) read and
// write zeros.  HBM bound: T1 read once (FP32), T3 written once (3 x BF16).
#include <cuda_bf16.h>

#include <climits>

#include "mpo_step.hpp"
#include "sg_matvec.hpp"
#include "tc_roles.cuh"

namespace udmrg {

namespace {

__device__ __forceinline__ int canon(int r, int k, int tr) {
  return (((k >> 3) * (tr >> 3) + (r >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1);
}

constexpr int kMpoWarps = 8;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kNzBatch = 4;  // nonzeros whose loads are in flight together

__global__ void __launch_bounds__(32 * kMpoWarps, 2)
    mpo_chunk_kernel(const MpoTask *__restrict__ tasks, int ntasks,
                     const MpoPair *__restrict__ pairs, const MpoOut *__restrict__ outs,
                     const int32_t *__restrict__ rowptr, const MpoNzRec *__restrict__ nzr,
                     const float *__restrict__ t1, uint8_t *__restrict__ img) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int64_t plane = (int64_t)kTcBM * kTcBK * 2;
  tc::pdl_wait();  // T1 from the L.psi GEMM
  for (int t = blockIdx.x * kMpoWarps + warp; t < ntasks; t += gridDim.x * kMpoWarps) {
    const MpoTask tk = tasks[t];
    const MpoPair pr = pairs[tk.pair];
    const int nch = pr.dbp >> 3;
    const int u = tk.u0 + lane;
    const bool valid = u < pr.da * nch;
    const int a = valid ? u / nch : 0;
    const int c8 = valid ? (u - a * nch) * 8 : 0;
    const int kbeg = __ldg(rowptr + pr.row0), kend = __ldg(rowptr + pr.row0 + pr.nout);
    // Output channels [ob, ob + 32): lane l holds channel ob + l's end in the
    // nonzero list and its image target (loaded together, read by shuffles).
    int ob = 0;
    const bool has = lane < pr.nout;
    int endv = has ? __ldg(rowptr + pr.row0 + 1 + lane) : INT_MAX;
    MpoOut outv = has ? outs[pr.out0 + lane] : MpoOut{0, 0, 0, 0, 0};
    int o = 0;
    int next = __shfl_sync(kFull, endv, 0);  // end of output channel o's nonzeros
    float acc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = 0.f;
    // write channel o's sums, then move to channel o + 1 (warp-uniform)
    auto finish = [&]() {
      const int sl = o - ob;
      const long long off0 = __shfl_sync(kFull, (long long)outv.img_off, sl);
      const int row0 = __shfl_sync(kFull, outv.row0, sl);
      const int rstride = __shfl_sync(kFull, outv.rstride, sl);
      const int col0 = __shfl_sync(kFull, outv.col0, sl);
      const int kc = __shfl_sync(kFull, outv.kc, sl);
      if (valid) {
        const int row = row0 + a * rstride;
        const int col = col0 + c8;
        const int64_t off = off0 + ((int64_t)(row >> 7) * kc + (col >> 6)) * 3 * plane +
                            canon(row & 127, col & 63, kTcBM);
        uint4 h, m, l;
        split8(acc, h, m, l);
        *(uint4 *)(img + off) = h;
        *(uint4 *)(img + off + plane) = m;
        *(uint4 *)(img + off + 2 * plane) = l;
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[j] = 0.f;
      if (++o - ob == 32) {
        ob += 32;
        const bool h2 = ob + lane < pr.nout;
        endv = h2 ? __ldg(rowptr + pr.row0 + 1 + ob + lane) : INT_MAX;
        outv = h2 ? outs[pr.out0 + ob + lane] : MpoOut{0, 0, 0, 0, 0};
      }
      next = __shfl_sync(kFull, endv, o - ob);
    };
    // Nonzeros 32 at a time, one record per lane (shuffled out), eight
    // nonzeros' sixteen 16-byte loads in flight together.
    for (int kb = kbeg; kb < kend; kb += 32) {
      const int nb = min(32, kend - kb);
      MpoNzRec mine{0, 0, 0.f};
      if (lane < nb) mine = nzr[kb + lane];
      for (int q0 = 0; q0 < nb; q0 += kNzBatch) {
        float4 x[kNzBatch][2];
        float v[kNzBatch];
#pragma unroll
        for (int q = 0; q < kNzBatch; ++q) {
          const int sl = q0 + q;
          const long long base = __shfl_sync(kFull, (long long)mine.base, sl);
          const int astride = __shfl_sync(kFull, mine.astride, sl);
          v[q] = __shfl_sync(kFull, mine.v, sl);
          x[q][0] = x[q][1] = make_float4(0.f, 0.f, 0.f, 0.f);
          if (sl < nb && valid) {
            const float4 *src = (const float4 *)(t1 + base + (int64_t)a * astride + c8);
            x[q][0] = __ldg(src);
            x[q][1] = __ldg(src + 1);
          }
        }
#pragma unroll
        for (int q = 0; q < kNzBatch; ++q) {
          if (q0 + q >= nb) break;
          while (kb + q0 + q >= next) finish();  // output channel o is complete
          acc[0] = fmaf(v[q], x[q][0].x, acc[0]);
          acc[1] = fmaf(v[q], x[q][0].y, acc[1]);
          acc[2] = fmaf(v[q], x[q][0].z, acc[2]);
          acc[3] = fmaf(v[q], x[q][0].w, acc[3]);
          acc[4] = fmaf(v[q], x[q][1].x, acc[4]);
          acc[5] = fmaf(v[q], x[q][1].y, acc[5]);
          acc[6] = fmaf(v[q], x[q][1].z, acc[6]);
          acc[7] = fmaf(v[q], x[q][1].w, acc[7]);
        }
      }
    }
    while (o < pr.nout) finish();  // the last channel and channels without nonzeros
  }
  tc::pdl_launch_dependents();
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
  const int ntasks = (int)p.tasks.size();
  if (ntasks == 0) return;
  const int blocks = (ntasks + kMpoWarps - 1) / kMpoWarps;
  const int grid = std::min(blocks, 16 * ctx.num_sms);
  UDMRG_CHECK_CUDA(tc::launch_pdl(mpo_chunk_kernel, dim3(grid), dim3(32 * kMpoWarps), 0,
                                  ctx.stream, p.d_tasks, ntasks, p.d_pairs, p.d_outs, p.d_rowptr,
                                  p.d_nz, p.t1, p.t3_img));
  ctx.launches++;
}

}  // namespace udmrg
