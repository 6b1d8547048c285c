// Roles shared by the warp-specialised tcgen05 split-BF16 GEMM kernels (the
// image GEMM of tc_gemm.cu and the GEMM with the MPO step fused into its
// producers, tc_mpo_gemm.cu): shared-memory layout and barriers, the MMA
// issue role (one thread: six split products per 16-deep K step into an FP32
// TMEM accumulator) and the epilogue role (four warps drain the accumulator
// into FP32, FP64 or interleaved complex rows).  Every wait is bounded; a
// timeout sets the error flag and the abort flag, and every role leaves its
// loop.
#pragma once

#include "tc_common.cuh"
#include "tc_gemm.hpp"

namespace udmrg {

namespace {

constexpr int kAcc = 2;  // TMEM accumulators (epilogue of tile i overlaps tile i+1)
// Headroom after the stage buffers: no descriptor read can leave the
// allocation even if a stride field were misread.
constexpr int kPadBytes = 8 * 1024;
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s: a wait this long means a fault

// Shared-memory and TMEM layout for B tiles of BN rows (UMMA N): stages of
// one A unit (128 x 64, three planes) and one B unit (BN x 64, three planes).
template <int BN>
struct TcShape {
  static_assert(BN == 64 || BN == 128, "tcgen05 GEMM: B tiles of 64 or 128 rows");
  static constexpr int kStages = BN == 64 ? 3 : 2;
  static constexpr int64_t kUnitB = 3LL * BN * kTcBK * 2;  // 24 KB / 48 KB
  static constexpr int kStageBytes = (int)(kTcUnitA + kUnitB);  // 72 KB / 96 KB
  static constexpr int kBarOffset = kStages * kStageBytes + kPadBytes;
  static constexpr int kSmemBytes = kBarOffset + 1024;
  static constexpr uint32_t kTmemCols = kAcc * BN;  // FP32: 2 x BN columns x 128 lanes
  static_assert(kSmemBytes <= 227 * 1024, "tcgen05 GEMM: shared memory budget");
};

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for an mbarrier phase with a wall-clock limit; false on timeout.
__device__ __forceinline__ bool wait_phase(uint64_t *bar, uint32_t parity) {
  if (tc::mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (true) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kWaitNs) return false;
  }
}

// FP32 -> FP64 by bit manipulation on the integer pipes (exact for normal
// numbers; sub-normal FP32 values, below 1.2e-38, become zero): the FP64
// conversion instruction would run on this GPU's narrow FP64 pipe.
__device__ __forceinline__ double widen_f32(float v) {
  const uint32_t u = __float_as_uint(v);
  const uint64_t sign = (uint64_t)(u >> 31) << 63;
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint64_t m = (uint64_t)(u & 0x7FFFFFu) << 29;
  uint64_t d;
  if (e == 0)
    d = sign;
  else if (e == 0xFFu)
    d = sign | (0x7FFull << 52) | m;
  else
    d = sign | ((uint64_t)(e + 896u) << 52) | m;
  return __longlong_as_double((long long)d);
}

// Byte offset of element (r, k) inside one plane of a TR x 64 tile.
__device__ __forceinline__ int canon_off(int r, int k, int tr) {
  return (((k >> 3) * (tr >> 3) + (r >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1);
}

template <typename T>
__device__ __forceinline__ void split3(T x, __nv_bfloat16 &h, __nv_bfloat16 &m,
                                       __nv_bfloat16 &l);
template <>
__device__ __forceinline__ void split3<float>(float x, __nv_bfloat16 &h, __nv_bfloat16 &m,
                                              __nv_bfloat16 &l) {
  h = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(h);
  m = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(m);
  l = __float2bfloat16_rn(r2);
}

// FP64 -> FP32, round to nearest even, on the integer pipes (the conversion
// instruction would use this GPU's narrow FP64 pipe).  |x| below the FP32
// normal range (1.2e-38) becomes zero, overflow becomes infinity.
__device__ __forceinline__ float narrow_f64(double x) {
  const uint64_t d = (uint64_t)__double_as_longlong(x);
  const uint32_t sign = (uint32_t)(d >> 63) << 31;
  const int e = (int)((d >> 52) & 0x7FF);
  const uint64_t mant = d & 0xFFFFFFFFFFFFFull;
  if (e == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (mant ? 0x400000u : 0u));
  int fe = e - 1023 + 127;
  if (fe >= 255) return __uint_as_float(sign | 0x7F800000u);
  if (fe <= 0) return __uint_as_float(sign);
  uint32_t fm = (uint32_t)(mant >> 29);
  const uint64_t rest = mant & 0x1FFFFFFFull;
  if (rest > 0x10000000ull || (rest == 0x10000000ull && (fm & 1u))) {
    if (++fm == 0x800000u) {
      fm = 0;
      if (++fe >= 255) return __uint_as_float(sign | 0x7F800000u);
    }
  }
  return __uint_as_float(sign | ((uint32_t)fe << 23) | fm);
}

__device__ __forceinline__ float to_f32(float x) { return x; }
__device__ __forceinline__ float to_f32(double x) { return narrow_f64(x); }

__device__ __forceinline__ uint32_t pack_bf16x2(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// x = hi + mid + lo, each the BF16 rounding of the remainder (exact
// differences in FP32), eight values into three 16-byte plane segments.
__device__ __forceinline__ void split8(const float (&x)[8], uint4 &h, uint4 &m, uint4 &l) {
  uint32_t ph[4], pm[4], pl[4];
#pragma unroll
  for (int j = 0; j < 8; j += 2) {
    __nv_bfloat16 hv[2], mv[2], lv[2];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      hv[t] = __float2bfloat16_rn(x[j + t]);
      const float r1 = x[j + t] - __bfloat162float(hv[t]);
      mv[t] = __float2bfloat16_rn(r1);
      lv[t] = __float2bfloat16_rn(r1 - __bfloat162float(mv[t]));
    }
    ph[j >> 1] = pack_bf16x2(hv[0], hv[1]);
    pm[j >> 1] = pack_bf16x2(mv[0], mv[1]);
    pl[j >> 1] = pack_bf16x2(lv[0], lv[1]);
  }
  h = make_uint4(ph[0], ph[1], ph[2], ph[3]);
  m = make_uint4(pm[0], pm[1], pm[2], pm[3]);
  l = make_uint4(pl[0], pl[1], pl[2], pl[3]);
}

// Plane pairs (A plane, B plane) of the six split products.
__device__ __constant__ int kProdA[6] = {0, 0, 1, 0, 1, 2};
__device__ __constant__ int kProdB[6] = {0, 1, 0, 2, 1, 0};

// Barriers and the TMEM address slot after the stage buffers.  full/empty per
// shared-memory stage (producers -> MMA -> producers), tfull/tempty per TMEM
// accumulator (MMA -> epilogue -> MMA), fin: all MMAs of the CTA completed.
struct TcBars {
  uint64_t *full, *empty, *tfull, *tempty, *fin;
  uint32_t *tmem_slot;
  volatile int *abort_flag;
};

template <int BN>
__device__ __forceinline__ TcBars tc_bars(uint8_t *smem) {
  using S = TcShape<BN>;
  TcBars b;
  b.full = (uint64_t *)(smem + S::kBarOffset);
  b.empty = b.full + S::kStages;
  b.tfull = b.empty + S::kStages;
  b.tempty = b.tfull + kAcc;
  b.fin = b.tempty + kAcc;
  b.tmem_slot = (uint32_t *)(b.fin + 1);
  b.abort_flag = (volatile int *)(b.tmem_slot + 1);
  return b;
}

// Barrier initialisation (thread 0; a full barrier completes after
// full_count arrivals and its transaction bytes), TMEM allocation (warp
// alloc_warp) and the block-wide synchronisation; returns the TMEM base.
template <int BN>
__device__ __forceinline__ uint32_t tc_setup(const TcBars &b, uint32_t full_count,
                                             int alloc_warp) {
  using S = TcShape<BN>;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    for (int s = 0; s < S::kStages; ++s) {
      tc::mbar_init(&b.full[s], full_count);
      tc::mbar_init(&b.empty[s], 1);
    }
    for (int a = 0; a < kAcc; ++a) {
      tc::mbar_init(&b.tfull[a], 1);
      tc::mbar_init(&b.tempty[a], 4);  // one arrival per epilogue warp
    }
    tc::mbar_init(b.fin, 1);
    *b.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == alloc_warp) {
    tc::tmem_alloc(b.tmem_slot, S::kTmemCols);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  return *b.tmem_slot;
}

template <int BN>
__device__ __forceinline__ void tc_teardown(uint32_t tmem, int alloc_warp) {
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if ((int)(threadIdx.x >> 5) == alloc_warp) tc::tmem_dealloc(tmem, TcShape<BN>::kTmemCols);
}

__device__ __forceinline__ void tc_fail(const TcBars &b, int *err, int code) {
  atomicExch(err, code);
  *b.abort_flag = 1;
}

// MMA issue (one thread) over the CTA's tiles (static schedule
// t = blockIdx.x + i * gridDim.x): for each K chunk, wait for its stage,
// issue the six split products per 16-deep K step, release the stage; after
// the last chunk, hand the accumulator to the epilogue.
template <int BN>
__device__ __forceinline__ void tc_mma_role(const TcTile *__restrict__ tiles, int ntiles,
                                            const TcGroup *__restrict__ groups, uint8_t *smem,
                                            const TcBars &b, uint32_t tmem, int *err) {
  using S = TcShape<BN>;
  constexpr uint32_t idesc = tc::idesc_bf16_f32(kTcBM, BN);
  uint32_t G = 0, i = 0;
  for (int t = blockIdx.x; t < ntiles && !*b.abort_flag; t += gridDim.x, ++i) {
    const TcGroup g = groups[tiles[t].group];
    const uint32_t acc = i & 1;
    if (i >= kAcc && !wait_phase(&b.tempty[acc], ((i >> 1) - 1) & 1)) {
      tc_fail(b, err, 4);
      break;
    }
    tc::fence_after_sync();
    const uint32_t dcol = tmem + acc * BN;
    bool ok = true;
    for (int c = 0; c < g.kc; ++c, ++G) {
      const uint32_t s = G % S::kStages;
      if (!wait_phase(&b.full[s], (G / S::kStages) & 1)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint32_t sa = tc::smem_u32(smem + s * S::kStageBytes);
      const uint32_t sb = sa + (uint32_t)kTcUnitA;
      constexpr uint32_t planeA = kTcBM * kTcBK * 2, planeB = BN * kTcBK * 2;
#pragma unroll
      for (int ks = 0; ks < kTcBK / 16; ++ks) {
#pragma unroll
        for (int p = 0; p < 6; ++p) {
          // K step ks covers core-matrix columns 2ks, 2ks+1
          const uint64_t ad = tc::make_desc(
              sa + kProdA[p] * planeA + ks * 2 * (kTcBM / 8) * 128, (kTcBM / 8) * 128, 128);
          const uint64_t bd = tc::make_desc(
              sb + kProdB[p] * planeB + ks * 2 * (BN / 8) * 128, (BN / 8) * 128, 128);
          tc::mma_bf16(dcol, ad, bd, idesc, (c > 0 || ks > 0 || p > 0) ? 1u : 0u);
        }
      }
      tc::mma_commit(&b.empty[s]);  // the stage is free once these MMAs completed
    }
    if (!ok) {
      tc_fail(b, err, 1);
      break;
    }
    tc::mma_commit(&b.tfull[acc]);  // the accumulator is complete
  }
  tc::mma_commit(b.fin);  // every MMA of this CTA has completed
  if (!wait_phase(b.fin, 0)) tc_fail(b, err, 3);
}

// Epilogue: warp q (0..3, the TMEM lane quarter it may access) drains
// accumulator rows 32 q .. 32 q + 31 of every tile, one row per lane.
template <int BN>
__device__ __forceinline__ void tc_epilogue_role(int q, int lane,
                                                 const TcTile *__restrict__ tiles, int ntiles,
                                                 const TcGroup *__restrict__ groups,
                                                 const int64_t *__restrict__ rowaddr, void *out,
                                                 int out_kind, double alpha, const TcBars &b,
                                                 uint32_t tmem, int *err) {
    const int m = q * 32 + lane;
    uint32_t i = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
      const TcTile tile = tiles[t];
      const TcGroup g = groups[tile.group];
      const uint32_t acc = i & 1;
      if (*b.abort_flag) break;
      if (!wait_phase(&b.tfull[acc], (i >> 1) & 1)) {
        if (lane == 0) tc_fail(b, err, 2);
        break;
      }
      tc::fence_after_sync();
      const int64_t grow = (int64_t)tile.mtile * kTcBM + m;
      const bool row_ok = grow < g.M;
      const int64_t base = row_ok ? rowaddr[g.row0 + grow] : 0;
      const int n0 = tile.ntile * BN;
      // epilogue math in FP32 (the accumulator's precision); no FP64 instruction
      const float af = (float)alpha;
#pragma unroll
      for (int cb = 0; cb < BN / 16; ++cb) {
        uint32_t r[16];
        tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + acc * BN + cb * 16, r);
        tc::tmem_wait_ld();
        if (row_ok) {
          // 16-byte stores where the row position allows (four FP32 or two
          // FP64 values per store; a lane writes one row)
          const int nc = n0 + cb * 16;
          float v[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = g.kc > 0 ? af * __uint_as_float(r[j]) : 0.0f;
          if (out_kind == kTcOutC128) {
            // columns [0, N/2): real parts, [N/2, N): imaginary parts of the
            // interleaved complex row at base
            const int half = g.N >> 1;
            double *o = (double *)out + base;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int n = nc + j;
              if (n < g.N) o[n < half ? 2 * n : 2 * (n - half) + 1] = widen_f32(v[j]);
            }
          } else if (out_kind == kTcOutF64) {
            double *o = (double *)out + base + nc;
            const bool vec = (((base + nc) & 1) == 0);
#pragma unroll
            for (int j = 0; j < 16; j += 2) {
              if (vec && nc + j + 1 < g.N) {
                *(double2 *)(o + j) = make_double2(widen_f32(v[j]), widen_f32(v[j + 1]));
              } else {
                if (nc + j < g.N) o[j] = widen_f32(v[j]);
                if (nc + j + 1 < g.N) o[j + 1] = widen_f32(v[j + 1]);
              }
            }
          } else {
            float *o = (float *)out + base + nc;
            const bool vec = (((base + nc) & 3) == 0);
#pragma unroll
            for (int j = 0; j < 16; j += 4) {
              if (vec && nc + j + 3 < g.N) {
                *(float4 *)(o + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
              } else {
#pragma unroll
                for (int t = 0; t < 4; ++t)
                  if (nc + j + t < g.N) o[j + t] = v[j + t];
              }
            }
          }
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&b.tempty[acc]);
    }
}

}  // namespace

}  // namespace udmrg
