// tcgen05 split-BF16 grouped GEMM and the image packing kernel.
#include <algorithm>

#include "tc_common.cuh"
#include "tc_gemm.hpp"

namespace udmrg {

namespace {

constexpr int kStages = 3;
constexpr int kThreads = 192;  // warp 0: loads, warp 1: MMA issue, warps 2-5: epilogue
constexpr int kAcc = 2;        // TMEM accumulators (epilogue of tile i overlaps tile i+1)
constexpr int kStageBytes = (int)(kTcUnitA + kTcUnitB);  // 72 KB
// Headroom after the stage buffers: no descriptor read can leave the
// allocation even if a stride field were misread.
constexpr int kPadBytes = 8 * 1024;
constexpr int kBarOffset = kStages * kStageBytes + kPadBytes;
constexpr int kSmemBytes = kBarOffset + 1024;
static_assert(kSmemBytes <= 227 * 1024, "tc_gemm: shared memory budget");
constexpr uint32_t kTmemCols = kAcc * kTcBN;  // FP32 accumulators: 2 x BN columns x 128 lanes
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s: a wait this long means a fault

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

// Pack sub-matrices into split-BF16 images, one 32 x 64 tile of one op per
// work item (the tiles of all ops are spread over the grid, so one large
// block does not serialise on one CTA).  The tile is staged in shared memory
// (as FP32), loaded along whichever source direction is contiguous; then each
// thread splits one row's 8 consecutive K values into three BF16 planes and
// writes each plane with one 16-byte store (canonical layout: 8 consecutive
// K values of a row are 16 contiguous bytes).
template <typename T>
__global__ void __launch_bounds__(256)
    pack_kernel(const PackOp *__restrict__ ops, const PackTile *__restrict__ tiles, int ntiles,
                const T *__restrict__ src, uint8_t *__restrict__ img) {
  __shared__ float tile[64][33];  // [k][r]
  const int tid = threadIdx.x;
  for (int w = blockIdx.x; w < ntiles; w += gridDim.x) {
    const PackTile pt = tiles[w];
    const PackOp op = ops[pt.op];
    const int64_t plane = (int64_t)op.tr * kTcBK * 2;
    const int ts = op.tr == 128 ? 7 : 6;
    const bool rows_contig = op.src_rs == 1 && op.src_cs != 1;
    __syncthreads();  // the previous tile has been read
    for (int e = tid; e < 32 * 64; e += 256) {
      int r, k;
      if (rows_contig) {
        r = e & 31;
        k = e >> 5;
      } else {
        k = e & 63;
        r = e >> 6;
      }
      const int rr = pt.r0 + r, kk = pt.k0 + k;
      float v = 0.f;
      if (rr < op.rows && kk < op.cols) {
        const T x = src[op.src_off + (int64_t)rr * op.src_rs + (int64_t)kk * op.src_cs];
        v = to_f32(x);
        if (op.neg) v = -v;
      }
      tile[k][r] = v;
    }
    __syncthreads();
    const int r = tid >> 3, g = tid & 7;
    const int rs = pt.r0 + r, ks = pt.k0 + g * 8;
    if (rs >= op.rows || ks >= op.cols) continue;
    const int rr = op.r0 + rs;
    const int64_t rowbase = op.img_off + (int64_t)(rr >> ts) * op.kc * 3 * plane;
    const int rin = rr & (op.tr - 1);
    const int kk = op.k0 + ks;
    if ((kk & 7) == 0) {
      // eight values (zeros past the op's columns: padding) -> 3 x 16 bytes
      uint32_t ph[4], pm[4], pl[4];
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        __nv_bfloat16 h0, m0, l0, h1, m1, l1;
        split3<float>(tile[g * 8 + j][r], h0, m0, l0);
        split3<float>(tile[g * 8 + j + 1][r], h1, m1, l1);
        ph[j >> 1] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
        pm[j >> 1] = (uint32_t)__bfloat16_as_ushort(m0) | ((uint32_t)__bfloat16_as_ushort(m1) << 16);
        pl[j >> 1] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
      }
      const int64_t off = rowbase + (int64_t)(kk >> 6) * 3 * plane + canon_off(rin, kk & 63, op.tr);
      *(uint4 *)(img + off) = make_uint4(ph[0], ph[1], ph[2], ph[3]);
      *(uint4 *)(img + off + plane) = make_uint4(pm[0], pm[1], pm[2], pm[3]);
      *(uint4 *)(img + off + 2 * plane) = make_uint4(pl[0], pl[1], pl[2], pl[3]);
    } else {
      for (int j = 0; j < 8 && ks + j < op.cols; ++j) {
        __nv_bfloat16 h, m, l;
        split3<float>(tile[g * 8 + j][r], h, m, l);
        const int kj = kk + j;
        const int64_t off =
            rowbase + (int64_t)(kj >> 6) * 3 * plane + canon_off(rin, kj & 63, op.tr);
        *(__nv_bfloat16 *)(img + off) = h;
        *(__nv_bfloat16 *)(img + off + plane) = m;
        *(__nv_bfloat16 *)(img + off + 2 * plane) = l;
      }
    }
  }
}

// Plane pairs (A plane, B plane) of the six split products.
__device__ __constant__ int kProdA[6] = {0, 0, 1, 0, 1, 2};
__device__ __constant__ int kProdB[6] = {0, 1, 0, 2, 1, 0};

// Warp-specialised persistent kernel over the tile list (static schedule
// t = blockIdx.x + i * gridDim.x).  Barriers: full/empty per shared-memory
// stage (bulk copies -> MMA -> copies), tfull/tempty per TMEM accumulator
// (MMA -> epilogue -> MMA).  Every wait is bounded; a timeout sets *err and the
// abort flag, and every role leaves its loop.
__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_kernel(const TcTile *__restrict__ tiles, int ntiles, const TcGroup *__restrict__ groups,
                   const uint8_t *__restrict__ aimg, const uint8_t *__restrict__ bimg,
                   const int64_t *__restrict__ rowaddr, void *__restrict__ out, int out_kind,
                   double alpha, int *__restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t *full = (uint64_t *)(smem + kBarOffset);
  uint64_t *empty = full + kStages;
  uint64_t *tfull = empty + kStages;
  uint64_t *tempty = tfull + kAcc;
  uint64_t *fin = tempty + kAcc;
  uint32_t *tmem_slot = (uint32_t *)(fin + 1);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < kAcc; ++a) {
      tc::mbar_init(&tfull[a], 1);
      tc::mbar_init(&tempty[a], 4);  // one arrival per epilogue warp
    }
    tc::mbar_init(fin, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, kTmemCols);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  constexpr uint32_t idesc = tc::idesc_bf16_f32(kTcBM, kTcBN);
  auto fail = [&](int code) {
    atomicExch(err, code);
    *abort_flag = 1;
  };

  if (warp == 0) {
    if (lane == 0) {  // producer: one bulk copy per operand unit and chunk
      uint32_t G = 0;
      for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
        const TcTile tile = tiles[t];
        const TcGroup g = groups[tile.group];
        const uint8_t *abase = aimg + g.a_img + (int64_t)tile.mtile * g.kc * kTcUnitA;
        const uint8_t *bbase = bimg + g.b_img + (int64_t)tile.ntile * g.kc * kTcUnitB;
        for (int c = 0; c < g.kc; ++c, ++G) {
          const uint32_t s = G % kStages;
          if (G >= kStages && !wait_phase(&empty[s], ((G / kStages) - 1) & 1)) {
            fail(1);
            break;
          }
          uint8_t *st = smem + s * kStageBytes;
          tc::mbar_expect_tx(&full[s], (uint32_t)(kTcUnitA + kTcUnitB));
          tc::bulk_g2s(st, abase + (int64_t)c * kTcUnitA, (uint32_t)kTcUnitA, &full[s]);
          tc::bulk_g2s(st + kTcUnitA, bbase + (int64_t)c * kTcUnitB, (uint32_t)kTcUnitB, &full[s]);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issue: six split products per 16-deep K step
      uint32_t G = 0, i = 0;
      for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x, ++i) {
        const TcGroup g = groups[tiles[t].group];
        const uint32_t acc = i & 1;
        if (i >= kAcc && !wait_phase(&tempty[acc], ((i >> 1) - 1) & 1)) {
          fail(4);
          break;
        }
        tc::fence_after_sync();
        const uint32_t dcol = tmem + acc * kTcBN;
        bool ok = true;
        for (int c = 0; c < g.kc; ++c, ++G) {
          const uint32_t s = G % kStages;
          if (!wait_phase(&full[s], (G / kStages) & 1)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t sa = tc::smem_u32(smem + s * kStageBytes);
          const uint32_t sb = sa + (uint32_t)kTcUnitA;
          constexpr uint32_t planeA = kTcBM * kTcBK * 2, planeB = kTcBN * kTcBK * 2;
#pragma unroll
          for (int ks = 0; ks < kTcBK / 16; ++ks) {
#pragma unroll
            for (int p = 0; p < 6; ++p) {
              // K step ks covers core-matrix columns 2ks, 2ks+1
              const uint64_t ad = tc::make_desc(
                  sa + kProdA[p] * planeA + ks * 2 * (kTcBM / 8) * 128, (kTcBM / 8) * 128, 128);
              const uint64_t bd = tc::make_desc(
                  sb + kProdB[p] * planeB + ks * 2 * (kTcBN / 8) * 128, (kTcBN / 8) * 128, 128);
              tc::mma_bf16(dcol, ad, bd, idesc, (c > 0 || ks > 0 || p > 0) ? 1u : 0u);
            }
          }
          tc::mma_commit(&empty[s]);  // the stage is free once these MMAs completed
        }
        if (!ok) {
          fail(1);
          break;
        }
        tc::mma_commit(&tfull[acc]);  // the accumulator is complete
      }
      tc::mma_commit(fin);  // every MMA of this CTA has completed
      if (!wait_phase(fin, 0)) fail(3);
    }
  } else {  // epilogue: warp w drains TMEM lanes 32 (w % 4) ...
    const int q = warp & 3;
    const int m = q * 32 + lane;
    uint32_t i = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
      const TcTile tile = tiles[t];
      const TcGroup g = groups[tile.group];
      const uint32_t acc = i & 1;
      if (*abort_flag) break;
      if (!wait_phase(&tfull[acc], (i >> 1) & 1)) {
        if (lane == 0) fail(2);
        break;
      }
      tc::fence_after_sync();
      const int64_t grow = (int64_t)tile.mtile * kTcBM + m;
      const bool row_ok = grow < g.M;
      const int64_t base = row_ok ? rowaddr[g.row0 + grow] : 0;
      const int n0 = tile.ntile * kTcBN;
      // epilogue math in FP32 (the accumulator's precision); no FP64 instruction
      const float af = (float)alpha;
#pragma unroll
      for (int cb = 0; cb < kTcBN / 16; ++cb) {
        uint32_t r[16];
        tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + acc * kTcBN + cb * 16, r);
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
      if (lane == 0) tc::mbar_arrive(&tempty[acc]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

}  // namespace

int64_t tc_image_bytes(int64_t rows, int64_t K, int tr) {
  const int64_t rt = (rows + tr - 1) / tr, kc = (K + kTcBK - 1) / kTcBK;
  return rt * kc * 3 * tr * kTcBK * 2;
}

TcPlan::~TcPlan() {
  if (!ctx) return;
  ctx->free(d_groups);
  ctx->free(d_tiles);
  ctx->free(d_rowaddr);
  ctx->free(d_err);
}

void TcPlan::add_group(int64_t a_img, int64_t b_img, int32_t M, int32_t N, int32_t K,
                       const std::vector<int64_t> &rows) {
  UDMRG_REQUIRE((int64_t)rows.size() == M, "tc plan: one output row address per row");
  if (M == 0 || N == 0) return;
  TcGroup g{};
  g.a_img = a_img;
  g.b_img = b_img;
  g.row0 = (int64_t)rowaddr.size();
  g.M = M;
  g.N = N;
  g.K = K;
  g.mt = (M + kTcBM - 1) / kTcBM;
  g.nt = (N + kTcBN - 1) / kTcBN;
  g.kc = (K + kTcBK - 1) / kTcBK;
  rowaddr.insert(rowaddr.end(), rows.begin(), rows.end());
  const int32_t gid = (int32_t)groups.size();
  groups.push_back(g);
  for (int mt = 0; mt < g.mt; ++mt)
    for (int nt = 0; nt < g.nt; ++nt) tiles.push_back({gid, mt, nt, 0});
  flops += 2.0 * (double)M * (double)N * (double)K;
}

template <typename V>
static V *upload(Ctx *ctx, const std::vector<V> &v) {
  if (v.empty()) return nullptr;
  V *d = (V *)ctx->alloc(v.size() * sizeof(V));
  UDMRG_CHECK_CUDA(
      cudaMemcpyAsync(d, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, ctx->stream));
  return d;
}

void TcPlan::finalize() {
  std::stable_sort(tiles.begin(), tiles.end(), [&](const TcTile &a, const TcTile &b) {
    return groups[a.group].kc > groups[b.group].kc;
  });
  d_groups = upload(ctx, groups);
  d_tiles = upload(ctx, tiles);
  d_rowaddr = upload(ctx, rowaddr);
  d_err = (int *)ctx->alloc(sizeof(int));
  UDMRG_CHECK_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  ctx->sync();
}

std::vector<PackTile> pack_tiles(const std::vector<PackOp> &ops) {
  std::vector<PackTile> t;
  for (size_t o = 0; o < ops.size(); ++o)
    for (int32_t r0 = 0; r0 < ops[o].rows; r0 += 32)
      for (int32_t k0 = 0; k0 < ops[o].cols; k0 += 64) t.push_back({(int32_t)o, r0, k0, 0});
  return t;
}

PackList::~PackList() {
  if (!ctx) return;
  ctx->free(d_ops);
  ctx->free(d_tiles);
}

void PackList::upload(Ctx &c) {
  ctx = &c;
  tiles = pack_tiles(ops);
  d_ops = udmrg::upload(ctx, ops);
  d_tiles = udmrg::upload(ctx, tiles);
}

static void launch_pack(Ctx &ctx, const PackOp *d_ops, const PackTile *d_tiles, int ntiles,
                        const void *src, bool src_f64, uint8_t *img) {
  if (ntiles == 0) return;
  const int grid = std::min(ntiles, 16 * ctx.num_sms);
  if (src_f64)
    pack_kernel<double><<<grid, 256, 0, ctx.stream>>>(d_ops, d_tiles, ntiles, (const double *)src,
                                                      img);
  else
    pack_kernel<float><<<grid, 256, 0, ctx.stream>>>(d_ops, d_tiles, ntiles, (const float *)src,
                                                     img);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

void run_pack(Ctx &ctx, const PackList &pl, const void *src, bool src_f64, uint8_t *img) {
  launch_pack(ctx, pl.d_ops, pl.d_tiles, (int)pl.tiles.size(), src, src_f64, img);
}

void run_pack(Ctx &ctx, const std::vector<PackOp> &ops, const void *src, bool src_f64,
              uint8_t *img) {
  if (ops.empty()) return;
  PackList pl;
  pl.ops = ops;
  pl.upload(ctx);
  launch_pack(ctx, pl.d_ops, pl.d_tiles, (int)pl.tiles.size(), src, src_f64, img);
  ctx.sync();  // the lists are freed on return
}

void run_tc_gemm(Ctx &ctx, const TcPlan &plan, const uint8_t *a_img, const uint8_t *b_img,
                 void *out, int out_kind, double alpha) {
  const int ntiles = (int)plan.tiles.size();
  if (ntiles == 0) return;
  static bool attr_set = false;
  if (!attr_set) {
    UDMRG_CHECK_CUDA(cudaFuncSetAttribute(tc_gemm_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          kSmemBytes));
    attr_set = true;
  }
  const int grid = std::min(ntiles, ctx.num_sms);
  tc_gemm_kernel<<<grid, kThreads, kSmemBytes, ctx.stream>>>(
      plan.d_tiles, ntiles, plan.d_groups, a_img, b_img, plan.d_rowaddr, out, out_kind, alpha,
      plan.d_err);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

int tc_check(Ctx &ctx, const TcPlan &plan) {
  int h = 0;
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(&h, plan.d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  if (h) UDMRG_CHECK_CUDA(cudaMemsetAsync(plan.d_err, 0, sizeof(int), ctx.stream));
  return h;
}

}  // namespace udmrg
