// The MPO step fused into the producers of the .R GEMM of the mixed matvec.
//
// res_B'[(a', s1', s2') x b'] = T3_B'[(a', s1', s2') x (w2, b)] . R_B'[b' x (w2, b)]^T,
// T3 = (W1 W2) T1.  Instead of writing T3 as a split-BF16 image and reading
// it back, eight producer warps build each 128-row x 64-K tile of T3 in
// shared memory: thread (row r, half h) computes the four 8-wide K chunks
// 4h .. 4h + 3 of row r, each the CSR walk of the unfused MPO step
// (kernels_mpo.cu) for one output channel and one 8-wide b chunk: two 16-byte
// FP32 loads of T1 per nonzero, FP32 accumulation in the same order, the same
// three-way BF16 split (so the MMA operands, and the result, are bit-identical
// to the unfused kernels), three 16-byte shared-memory stores in the
// canonical K-major layout.  Thread 0 also stages the B tile (R image) by a
// bulk copy.  Warp 8 issues the MMAs, warps 9-12 drain the accumulators
// (tc_roles.cuh).  A stage is complete after all 256 producer arrivals (each
// after a proxy fence: the MMA reads shared memory through the async proxy)
// and the B tile's transaction bytes.
#include <algorithm>

#include "sg_matvec.hpp"
#include "tc_roles.cuh"

namespace udmrg {

namespace {

constexpr int kProducers = 256;  // warps 0-7
constexpr int kMmaWarp = 8;
constexpr int kFusedThreads = kProducers + 32 + 128;  // + MMA warp + four epilogue warps

struct ChunkWork {
  int k0, k1;    // the output channel's nonzeros [k0, k1) (empty: zero chunk)
  int c8;        // first b of the chunk
};

template <int BN>
__global__ void __launch_bounds__(kFusedThreads, 1)
    tc_mpo_gemm_kernel(const TcTile *__restrict__ tiles, int ntiles,
                       const TcGroup *__restrict__ groups, const MpoGroupMap *__restrict__ gmap,
                       const MpoRowInfo *__restrict__ rowinfo,
                       const MpoKChunk *__restrict__ kchunks, const MpoTgtRef *__restrict__ tgtref,
                       const int32_t *__restrict__ rowptr, const MpoNzRec *__restrict__ nzr,
                       const float *__restrict__ t1, const uint8_t *__restrict__ bimg,
                       const int64_t *__restrict__ rowaddr, void *__restrict__ out, int out_kind,
                       double alpha, int *__restrict__ err) {
  using S = TcShape<BN>;
  extern __shared__ __align__(1024) uint8_t smem[];
  const TcBars b = tc_bars<BN>(smem);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // full barrier: every producer thread, plus the expect-tx arrival of thread 0
  const uint32_t tmem = tc_setup<BN>(b, kProducers + 1, kMmaWarp);
  if (tid < kProducers) {
    const int r = tid & (kTcBM - 1), h = tid >> 7;
    constexpr int64_t planeA = (int64_t)kTcBM * kTcBK * 2;
    uint32_t G = 0;
    bool ok = true;
    for (int t = blockIdx.x; ok && t < ntiles && !*b.abort_flag; t += gridDim.x) {
      const TcTile tile = tiles[t];
      const TcGroup g = groups[tile.group];
      const MpoGroupMap gm = gmap[tile.group];
      const int64_t grow = (int64_t)tile.mtile * kTcBM + r;
      const bool rv = grow < g.M;
      const MpoRowInfo ri = rv ? rowinfo[gm.row0 + grow] : MpoRowInfo{0, 0, 0, 0};
      const uint8_t *bbase = bimg + g.b_img + (int64_t)tile.ntile * g.kc * S::kUnitB;
      for (int c = 0; c < g.kc; ++c, ++G) {
        const uint32_t s = G % S::kStages;
        if (G >= S::kStages && !wait_phase(&b.empty[s], ((G / S::kStages) - 1) & 1)) {
          tc_fail(b, err, 1);
          ok = false;
          break;
        }
        uint8_t *st = smem + s * S::kStageBytes;
        if (tid == 0) {
          tc::mbar_expect_tx(&b.full[s], (uint32_t)S::kUnitB);
          tc::bulk_g2s(st + kTcUnitA, bbase + (int64_t)c * S::kUnitB, (uint32_t)S::kUnitB,
                       &b.full[s]);
        }
        // the four chunks' output channels, then their first nonzeros' loads
        // together (eight 16-byte loads in flight), then the rest
        ChunkWork cw[4];
#pragma unroll
        for (int qq = 0; qq < 4; ++qq) {
          const int kq = c * 8 + h * 4 + qq;
          cw[qq] = {0, 0, 0};
          if (rv && kq < gm.nkch) {
            const MpoKChunk kc = kchunks[gm.kch0 + kq];
            const MpoTgtRef tr =
                tgtref[gm.tgt0 + ((int64_t)kc.half * gm.nrb + ri.rb) * gm.nkb + kc.kb];
            if (tr.csr0 >= 0) {
              const int crow = tr.csr0 + ri.s12p * tr.dw2 + kc.w2;
              cw[qq] = {__ldg(rowptr + crow), __ldg(rowptr + crow + 1), kc.c8};
            }
          }
        }
        float4 x[4][2];
        float v[4];
#pragma unroll
        for (int qq = 0; qq < 4; ++qq) {
          x[qq][0] = x[qq][1] = make_float4(0.f, 0.f, 0.f, 0.f);
          v[qq] = 0.f;
          if (cw[qq].k0 < cw[qq].k1) {
            const MpoNzRec e = nzr[cw[qq].k0];
            const float4 *src =
                (const float4 *)(t1 + e.base + (int64_t)ri.a * e.astride + cw[qq].c8);
            x[qq][0] = __ldg(src);
            x[qq][1] = __ldg(src + 1);
            v[qq] = e.v;
          }
        }
#pragma unroll
        for (int qq = 0; qq < 4; ++qq) {
          float acc[8];
          acc[0] = fmaf(v[qq], x[qq][0].x, 0.f);
          acc[1] = fmaf(v[qq], x[qq][0].y, 0.f);
          acc[2] = fmaf(v[qq], x[qq][0].z, 0.f);
          acc[3] = fmaf(v[qq], x[qq][0].w, 0.f);
          acc[4] = fmaf(v[qq], x[qq][1].x, 0.f);
          acc[5] = fmaf(v[qq], x[qq][1].y, 0.f);
          acc[6] = fmaf(v[qq], x[qq][1].z, 0.f);
          acc[7] = fmaf(v[qq], x[qq][1].w, 0.f);
          for (int k = cw[qq].k0 + 1; k < cw[qq].k1; ++k) {
            const MpoNzRec e = nzr[k];
            const float4 *src =
                (const float4 *)(t1 + e.base + (int64_t)ri.a * e.astride + cw[qq].c8);
            const float4 y0 = __ldg(src), y1 = __ldg(src + 1);
            acc[0] = fmaf(e.v, y0.x, acc[0]);
            acc[1] = fmaf(e.v, y0.y, acc[1]);
            acc[2] = fmaf(e.v, y0.z, acc[2]);
            acc[3] = fmaf(e.v, y0.w, acc[3]);
            acc[4] = fmaf(e.v, y1.x, acc[4]);
            acc[5] = fmaf(e.v, y1.y, acc[5]);
            acc[6] = fmaf(e.v, y1.z, acc[6]);
            acc[7] = fmaf(e.v, y1.w, acc[7]);
          }
          uint4 hi, mi, lo;
          split8(acc, hi, mi, lo);
          const int off = canon_off(r, (h * 4 + qq) * 8, kTcBM);
          *(uint4 *)(st + off) = hi;
          *(uint4 *)(st + planeA + off) = mi;
          *(uint4 *)(st + 2 * planeA + off) = lo;
        }
        // generic-proxy stores -> the MMA's async-proxy reads
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc::mbar_arrive(&b.full[s]);
      }
    }
  } else if (warp == kMmaWarp) {
    if (lane == 0) tc_mma_role<BN>(tiles, ntiles, groups, smem, b, tmem, err);
  } else {  // epilogue: warps 9-12, TMEM lane quarters 1, 2, 3, 0
    tc_epilogue_role<BN>(warp & 3, lane, tiles, ntiles, groups, rowaddr, out, out_kind, alpha,
                         b, tmem, err);
  }
  tc_teardown<BN>(tmem, kMmaWarp);
}

}  // namespace

template <int BN>
static void launch_tc_mpo_gemm(Ctx &ctx, const SgMatvecPlan &p, double *out) {
  const TcPlan &plan = p.g3;
  const int ntiles = (int)plan.tiles.size();
  static bool attr_set = false;
  if (!attr_set) {
    UDMRG_CHECK_CUDA(cudaFuncSetAttribute(tc_mpo_gemm_kernel<BN>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          TcShape<BN>::kSmemBytes));
    attr_set = true;
  }
  const int grid = std::min(ntiles, ctx.num_sms);
  tc_mpo_gemm_kernel<BN><<<grid, kFusedThreads, TcShape<BN>::kSmemBytes, ctx.stream>>>(
      plan.d_tiles, ntiles, plan.d_groups, p.d_gmap, p.d_rowinfo, p.d_kchunks, p.d_tgtref,
      p.d_rowptr, p.d_nz, p.t1, p.r_img, plan.d_rowaddr, out,
      p.cplx ? kTcOutC128 : kTcOutF64, 1.0, plan.d_err);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

void run_tc_mpo_gemm(Ctx &ctx, const SgMatvecPlan &p, double *out) {
  if (p.g3.tiles.empty()) return;
  if (p.g3.bn == 128)
    launch_tc_mpo_gemm<128>(ctx, p, out);
  else
    launch_tc_mpo_gemm<64>(ctx, p, out);
}

}  // namespace udmrg
