// tcgen05 split-BF16 grouped GEMM and the image packing kernel.
#include <algorithm>

#include "tc_roles.cuh"

namespace udmrg {

namespace {

constexpr int kThreads = 192;  // warp 0: loads, warp 1: MMA issue, warps 2-5: epilogue

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

// Warp-specialised persistent kernel over the tile list (static schedule
// t = blockIdx.x + i * gridDim.x): warp 0 stages both operands by bulk copies
// from their images, warp 1 issues the MMAs, warps 2-5 drain the
// accumulators.
template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_kernel(const TcTile *__restrict__ tiles, int ntiles, const TcGroup *__restrict__ groups,
                   const uint8_t *__restrict__ aimg, const uint8_t *__restrict__ bimg,
                   const int64_t *__restrict__ rowaddr, void *__restrict__ out, int out_kind,
                   double alpha, int *__restrict__ err) {
  using S = TcShape<BN>;
  extern __shared__ __align__(1024) uint8_t smem[];
  const TcBars b = tc_bars<BN>(smem);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t tmem = tc_setup<BN>(b, 1, 0);
  tc::pdl_wait();  // the images (and outputs) of the previous kernel
  if (warp == 0) {
    if (lane == 0) {  // producer: one bulk copy per operand unit and chunk
      uint32_t G = 0;
      for (int t = blockIdx.x; t < ntiles && !*b.abort_flag; t += gridDim.x) {
        const TcTile tile = tiles[t];
        const TcGroup g = groups[tile.group];
        const uint8_t *abase = aimg + g.a_img + (int64_t)tile.mtile * g.kc * kTcUnitA;
        const uint8_t *bbase = bimg + g.b_img + (int64_t)tile.ntile * g.kc * S::kUnitB;
        for (int c = 0; c < g.kc; ++c, ++G) {
          const uint32_t s = G % S::kStages;
          if (G >= S::kStages && !wait_phase(&b.empty[s], ((G / S::kStages) - 1) & 1)) {
            tc_fail(b, err, 1);
            break;
          }
          uint8_t *st = smem + s * S::kStageBytes;
          tc::mbar_expect_tx(&b.full[s], (uint32_t)(kTcUnitA + S::kUnitB));
          tc::bulk_g2s(st, abase + (int64_t)c * kTcUnitA, (uint32_t)kTcUnitA, &b.full[s]);
          tc::bulk_g2s(st + kTcUnitA, bbase + (int64_t)c * S::kUnitB, (uint32_t)S::kUnitB,
                       &b.full[s]);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) tc_mma_role<BN>(tiles, ntiles, groups, smem, b, tmem, err);
  } else {  // epilogue: warp w drains TMEM lanes 32 (w % 4) ...
    tc_epilogue_role<BN>(warp & 3, lane, tiles, ntiles, groups, rowaddr, out, out_kind, alpha,
                         b, tmem, err);
  }
  tc::pdl_launch_dependents();
  tc_teardown<BN>(tmem, 0);
}

// The same images for sources whose rows are (nearly) contiguous (psi: b
// runs), when every op starts at a K column that is a multiple of 8: no
// shared memory.  One work item per warp, 32 rows x 8 K columns of one op
// (psi's ops are small, about 20 x 20, so items of a whole block would leave
// most warps idle); lane l takes row l: each of the eight loads is coalesced
// across the warp (consecutive rows), and the three 16-byte plane stores of 32
// consecutive rows fill 512 contiguous bytes of the canonical layout.
template <typename T>
__global__ void __launch_bounds__(256)
    pack_rows_kernel(const PackOp *__restrict__ ops, const PackTile *__restrict__ items,
                     int nitems, const T *__restrict__ src, uint8_t *__restrict__ img) {
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  for (int w = blockIdx.x * wpb + (threadIdx.x >> 5); w < nitems; w += gridDim.x * wpb) {
    const PackTile pt = items[w];
    const PackOp op = ops[pt.op];
    const int rs = pt.r0 + lane, ks = pt.k0;
    if (rs >= op.rows) continue;
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float v = 0.f;
      if (ks + j < op.cols)
        v = to_f32(src[op.src_off + (int64_t)rs * op.src_rs + (int64_t)(ks + j) * op.src_cs]);
      x[j] = op.neg ? -v : v;
    }
    uint4 hi, mi, lo;
    split8(x, hi, mi, lo);
    const int64_t plane = (int64_t)op.tr * kTcBK * 2;
    const int ts = op.tr == 128 ? 7 : 6;
    const int rr = op.r0 + rs, kk = op.k0 + ks;
    const int64_t off = op.img_off + ((int64_t)(rr >> ts) * op.kc + (kk >> 6)) * 3 * plane +
                        canon_off(rr & (op.tr - 1), kk & 63, op.tr);
    *(uint4 *)(img + off) = hi;
    *(uint4 *)(img + off + plane) = mi;
    *(uint4 *)(img + off + 2 * plane) = lo;
  }
  tc::pdl_launch_dependents();
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
  g.nt = (N + bn - 1) / bn;
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

std::vector<PackTile> pack_tiles(const std::vector<PackOp> &ops, int kstep) {
  std::vector<PackTile> t;
  for (size_t o = 0; o < ops.size(); ++o)
    for (int32_t r0 = 0; r0 < ops[o].rows; r0 += 32)
      for (int32_t k0 = 0; k0 < ops[o].cols; k0 += kstep) t.push_back({(int32_t)o, r0, k0, 0});
  return t;
}

PackList::~PackList() {
  if (!ctx) return;
  ctx->free(d_ops);
  ctx->free(d_tiles);
}

void PackList::upload(Ctx &c) {
  ctx = &c;
  rows_src = !ops.empty();
  for (const PackOp &op : ops) rows_src = rows_src && op.src_rs <= 2 && op.k0 % 8 == 0;
  tiles = pack_tiles(ops, rows_src ? 8 : 64);
  d_ops = udmrg::upload(ctx, ops);
  d_tiles = udmrg::upload(ctx, tiles);
}

static void launch_pack(Ctx &ctx, const PackOp *d_ops, const PackTile *d_tiles, int ntiles,
                        const void *src, bool src_f64, uint8_t *img, bool rows_src = false) {
  if (ntiles == 0) return;
  const int grid = rows_src ? std::min((ntiles + 7) / 8, 32 * ctx.num_sms)
                            : std::min(ntiles, 16 * ctx.num_sms);
  if (rows_src && src_f64)
    pack_rows_kernel<double><<<grid, 256, 0, ctx.stream>>>(d_ops, d_tiles, ntiles,
                                                           (const double *)src, img);
  else if (rows_src)
    pack_rows_kernel<float><<<grid, 256, 0, ctx.stream>>>(d_ops, d_tiles, ntiles,
                                                          (const float *)src, img);
  else if (src_f64)
    pack_kernel<double><<<grid, 256, 0, ctx.stream>>>(d_ops, d_tiles, ntiles, (const double *)src,
                                                      img);
  else
    pack_kernel<float><<<grid, 256, 0, ctx.stream>>>(d_ops, d_tiles, ntiles, (const float *)src,
                                                     img);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
}

void run_pack(Ctx &ctx, const PackList &pl, const void *src, bool src_f64, uint8_t *img) {
  launch_pack(ctx, pl.d_ops, pl.d_tiles, (int)pl.tiles.size(), src, src_f64, img, pl.rows_src);
}

void run_pack(Ctx &ctx, const std::vector<PackOp> &ops, const void *src, bool src_f64,
              uint8_t *img) {
  if (ops.empty()) return;
  PackList pl;
  pl.ops = ops;
  pl.upload(ctx);
  launch_pack(ctx, pl.d_ops, pl.d_tiles, (int)pl.tiles.size(), src, src_f64, img, pl.rows_src);
  ctx.sync();  // the lists are freed on return
}

template <int BN>
static void launch_tc_gemm(Ctx &ctx, const TcPlan &plan, const uint8_t *a_img,
                           const uint8_t *b_img, void *out, int out_kind, double alpha) {
  const int ntiles = (int)plan.tiles.size();
  static bool attr_set = false;
  if (!attr_set) {
    UDMRG_CHECK_CUDA(cudaFuncSetAttribute(tc_gemm_kernel<BN>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          TcShape<BN>::kSmemBytes));
    attr_set = true;
  }
  const int grid = std::min(ntiles, ctx.num_sms);
  UDMRG_CHECK_CUDA(tc::launch_pdl(tc_gemm_kernel<BN>, dim3(grid), dim3(kThreads),
                                  (size_t)TcShape<BN>::kSmemBytes, ctx.stream, plan.d_tiles,
                                  ntiles, plan.d_groups, a_img, b_img, plan.d_rowaddr, out,
                                  out_kind, alpha, plan.d_err));
  ctx.launches++;
}

void run_tc_gemm(Ctx &ctx, const TcPlan &plan, const uint8_t *a_img, const uint8_t *b_img,
                 void *out, int out_kind, double alpha) {
  if (plan.tiles.empty()) return;
  if (plan.bn == 128)
    launch_tc_gemm<128>(ctx, plan, a_img, b_img, out, out_kind, alpha);
  else
    launch_tc_gemm<64>(ctx, plan, a_img, b_img, out, out_kind, alpha);
}

int tc_check(Ctx &ctx, const TcPlan &plan) {
  int h = 0;
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(&h, plan.d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  if (h) UDMRG_CHECK_CUDA(cudaMemsetAsync(plan.d_err, 0, sizeof(int), ctx.stream));
  return h;
}

}  // namespace udmrg
