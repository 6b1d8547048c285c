// Mixed-precision grouped GEMM on the tcgen05 tensor cores (split BF16).
//
// Operands are stored in HBM as "tile images": the exact shared-memory
// layout the MMA reads (no swizzle, K-major canonical layout of 8-row x
// 16-byte core matrices), pre-split into three BF16 planes (x = hi + mid + lo,
// each the BF16 rounding of the remainder, ~24 significant bits together).
// A tile image unit holds TR rows x 64 K for the three planes; units are
// ordered [row tile][K chunk].  The kernel fills shared memory with one bulk
// asynchronous copy per unit (cp.async.bulk, completion on an mbarrier), one
// elected thread issues the six cross products hi*hi, hi*mid, mid*hi, hi*lo,
// mid*mid, lo*hi per 16-deep K step into an FP32 accumulator in tensor
// memory, and all four warps drain the accumulator (tcgen05.ld) into FP32 or
// FP64 outputs addressed through a per-row address table.
#pragma once

#include "btensor.hpp"

namespace udmrg {

constexpr int kTcBM = 128;  // rows of an A tile (UMMA M)
constexpr int kTcBN = 64;   // default rows of a B tile (UMMA N); 64 or 128 per plan
constexpr int kTcBK = 64;   // K per chunk (four K=16 MMA steps)
constexpr int64_t kTcUnitA = 3LL * kTcBM * kTcBK * 2;  // 48 KB

// Pack one strided sub-matrix into an image (element type of the source:
// FP64 or FP32).  Element (r, k) of the sub-matrix is
// src[src_off + r*src_rs + k*src_cs] and lands at image row r0 + r, column
// k0 + k.  When k0 is a multiple of 8, the image columns from k0 + cols up to
// the next multiple of 8 are written as zeros (16-byte stores): the planners
// leave those columns as padding.
struct PackOp {
  int64_t src_off, src_rs, src_cs;
  int64_t img_off;  // byte offset of the image
  int32_t rows, cols;
  int32_t r0, k0;
  int32_t kc;  // K chunks of the image
  int32_t tr;  // rows per tile of the image (kTcBM or kTcBN)
  int32_t neg, pad;  // neg: pack the negated values
};

// One dense GEMM C(MxN) = alpha * A(MxK) * B(NxK)^T between two images.
struct TcGroup {
  int64_t a_img, b_img;  // byte offsets into the A / B image arenas
  int64_t row0;          // first entry of this group in the row address table
  int32_t M, N, K;
  int32_t mt, nt, kc;
};

struct TcTile {
  int32_t group, mtile, ntile, pad;
};

// kTcOutC128: the N columns are the real parts (first half) and imaginary
// parts (second half) of N/2 interleaved complex values per output row.
enum TcOut : int { kTcOutF32 = 0, kTcOutF64 = 1, kTcOutC128 = 2 };

struct TcPlan {
  Ctx *ctx = nullptr;
  int bn = kTcBN;  // rows of a B tile (64 or 128; the B images are packed with it)
  std::vector<TcGroup> groups;
  std::vector<TcTile> tiles;
  std::vector<int64_t> rowaddr;  // output element offset of each output row
  TcGroup *d_groups = nullptr;
  TcTile *d_tiles = nullptr;
  int64_t *d_rowaddr = nullptr;
  int *d_err = nullptr;
  double flops = 0;  // algorithmic 2*M*N*K
  TcPlan() = default;
  TcPlan(const TcPlan &) = delete;
  TcPlan &operator=(const TcPlan &) = delete;
  ~TcPlan();
  void add_group(int64_t a_img, int64_t b_img, int32_t M, int32_t N, int32_t K,
                 const std::vector<int64_t> &rows);
  void finalize();  // sort tiles (largest K first), upload
};

int64_t tc_image_bytes(int64_t rows, int64_t K, int tr);

// One work item of the pack kernel: a 32-row x 64-column tile of one op.
struct PackTile {
  int32_t op, r0, k0, pad;
};
// Work items: 32 rows x kstep K columns of one op each (64 for the staged
// kernel, 8 for the one-warp items of rows-contiguous sources).
std::vector<PackTile> pack_tiles(const std::vector<PackOp> &ops, int kstep = 64);

// A pack list resident on the device (ops and their tiles uploaded once).
struct PackList {
  Ctx *ctx = nullptr;
  std::vector<PackOp> ops;
  std::vector<PackTile> tiles;
  PackOp *d_ops = nullptr;
  PackTile *d_tiles = nullptr;
  bool rows_src = false;  // every op reads rows with stride <= 2 from a K column % 8 == 0
                          // (tiles are then one-warp items of 32 x 8)
  PackList() = default;
  PackList(const PackList &) = delete;
  PackList &operator=(const PackList &) = delete;
  ~PackList();
  void upload(Ctx &c);  // builds the tiles from ops
};

void run_pack(Ctx &ctx, const PackList &pl, const void *src, bool src_f64, uint8_t *img);
// One-shot form: uploads the ops and tiles, packs, frees them.
void run_pack(Ctx &ctx, const std::vector<PackOp> &ops, const void *src, bool src_f64,
              uint8_t *img);

void run_tc_gemm(Ctx &ctx, const TcPlan &plan, const uint8_t *a_img, const uint8_t *b_img,
                 void *out, int out_kind, double alpha);
// Returns and clears the device error flag of the plan (nonzero: a bounded
// wait inside the kernel ran out).
int tc_check(Ctx &ctx, const TcPlan &plan);

}  // namespace udmrg
