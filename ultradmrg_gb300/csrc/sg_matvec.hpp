// Mixed-precision two-site matvec on the tensor cores, regrouped by sector.
//
// H_eff psi = L . (W1 W2) . R . psi is computed as
//   step 1 (tcgen05): for every ket sector A of L, one dense GEMM
//          T1_A[(a',w) x (s1 s2 b)] = L_A[(a',w) x a] . Psi_A[a x (s1 s2 b)],
//          where L_A stacks all L blocks (A',W,A) and Psi_A all psi blocks
//          (A,S1,S2,B); every entry of T1_A is a T1 block entry, none padding;
//   step 2 (CUDA cores): T3[a',s1',s2',w2,b] = sum W1 W2 T1 over (w, s1, s2)
//          with the two MPO tensors contracted over their shared bond,
//          written straight into split-BF16 tile images of the step-3 operand;
//   step 3 (tcgen05): for every bra sector B' of R, one dense GEMM
//          res_B'[(a',s1',s2') x b'] = T3_B'[(a',s1',s2') x (w2,b)] . R_B'[b' x (w2,b)]^T.
// L_A and R_B' images are packed once per plan (the environments are fixed
// during a Lanczos solve); psi is packed every matvec.  Complex L, R and psi
// (real MPO coefficients) run through the real embedding: step 1 is
// [T1r; T1i] = [[Lr, -Li], [Li, Lr]] [psi_r; psi_i] (2M x 2K GEMMs), the MPO
// step maps both halves, step 3 is res = [T3r | T3i] [[Rr | -Ri]; [Ri | Rr]]^T
// whose 2 dB' columns the epilogue interleaves into complex values.  T1 is FP32.
//
// Padding: every run of the b index (a psi block's columns (s1, s2, b) in T1
// and in the psi image, an R block's K columns (w2, b) in the step-3 images)
// is padded to a multiple of 8, and complex data put their imaginary K half
// at a multiple of 8.  So each 8-wide chunk of b is 32-byte aligned in T1 and
// one 16-byte canonical row segment of the step-3 image: the MPO step moves
// it with vector loads and stores.  Padded entries are zero (the images are
// zeroed once; T1 pad columns are products with zero image rows).
#pragma once

#include "gemm.hpp"
#include "mpo_step.hpp"
#include "tc_gemm.hpp"

namespace udmrg {

// One MPO-step target: a T3 block (a', s1', s2', w2, b) in the step-3 image.
struct MpoTarget {
  int64_t img_off;     // byte offset of the group's A image (step-3 arena)
  int32_t row0;        // first image row of the block (a' = 0, s1' = s2' = 0)
  int32_t k0;          // first image column (w2 = 0, b = 0)
  int32_t kc;          // K chunks of the image
  int32_t da, db;      // a' and b sector dims
  int32_t dbp;         // db rounded up to 8 (image columns per w2)
  int32_t nout;        // output channels per (a', b): ds1' * ds2' * dw2
  int32_t ds12p;       // ds1' * ds2'
  int32_t dw2;
  int32_t src0, nsrc;  // source list
  int32_t kim;         // complex data: first image column of the imaginary half
};

// One MPO-step source: a T1 block (a', w, s1, s2, b) in T1_A and its
// coefficient matrix coef[(w s1 s2) x (s1' s2' w2)].
struct MpoSource {
  int64_t t1_off;      // element offset of entry (a'=0, w=0, s1=s2=0, b=0) in T1
  int64_t t1_im;       // complex data: offset of the imaginary half
  int64_t row_pitch;   // T1 elements between consecutive (a', w) rows (N_A)
  int32_t dw, ds12;    // w dim, ds1 * ds2
  int32_t coef_off;    // offset into the coefficient array
  int32_t bstride;     // T1 columns between consecutive (s1, s2) (db rounded up to 8)
};

// The MPO step regrouped by (A', B) sector pair: every T1 block (w, s1, s2)
// channel of the pair is an input channel (a' rows x b columns), every T3
// block (s1', s2', w2) channel an output channel, and
// out[o] = sum_i coef[o][i] in[i] at each (a', b).
struct MpoPair {
  int32_t in0, nin, out0, nout;
  int32_t row0, da, db, dbp;  // row0: first CSR row (output channel) of the pair
};
// Input channel of a pair (planning).
struct MpoIn {
  int64_t base;     // T1 element offset of (a' = 0, b = 0)
  int64_t astride;  // T1 elements between consecutive a'
};
// Nonzero of a pair's coefficient matrix (CSR over the pair's output
// channels), with its input channel's location: the kernel reads the chunk
// at t1 + base + a' * astride + b.  base and astride are multiples of 8.
struct MpoNzRec {
  int64_t base;
  int32_t astride;
  float v;
};
// Work of one warp: 32 consecutive units (a', 8-wide b chunk) of one pair.
struct MpoTask {
  int32_t pair, u0;
};
struct MpoOut {
  int64_t img_off;  // byte offset of the step-3 A image of the target's group
  int32_t row0, rstride, col0, kc;  // image row = row0 + a' * rstride, column = col0 + b
};

// Fused form of the MPO step and the .R GEMM (tc_mpo_gemm.cu): the GEMM's
// producer warps compute each 128-row x 64-K tile of T3 from T1 into shared
// memory (the CSR walk of the unfused MPO step), so the T3 image is neither
// written nor read.  Per step-3 group: where its tables start and their sizes.
struct MpoGroupMap {
  int64_t row0;   // first MpoRowInfo of the group (one per GEMM row)
  int64_t kch0;   // first MpoKChunk (one per 8-wide K chunk)
  int64_t tgt0;   // first MpoTgtRef ((half, row block, K block) table)
  int32_t nrb, nkb;  // row blocks (psi blocks (A', S1', S2')) and K blocks (R blocks (W2, B))
  int32_t nkch, pad;  // K chunks (the real and, for complex data, imaginary halves)
};
struct MpoRowInfo {
  int32_t rb, a, s12p, pad;  // row block, a', (s1', s2') index
};
struct MpoKChunk {
  int32_t kb, w2, c8, half;  // K block, w2, first b of the chunk, imaginary half
};
struct MpoTgtRef {
  int32_t csr0;  // CSR row of output channel (s1's2' = 0, w2 = 0); -1: no coupling
  int32_t dw2;
};

struct SgMatvecPlan {
  Ctx *ctx = nullptr;
  int64_t psi_size = 0;
  bool cplx = false;  // complex data through the real embedding
  // images
  uint8_t *l_img = nullptr, *psi_img = nullptr, *t3_img = nullptr, *r_img = nullptr;
  int64_t l_bytes = 0, psi_bytes = 0, t3_bytes = 0, r_bytes = 0;
  float *t1 = nullptr;
  int64_t t1_size = 0;
  // psi pack ops (device resident)
  PackList psi_pack;
  // GEMM plans
  TcPlan g1, g3;
  // MPO step
  std::vector<MpoTarget> targets;
  std::vector<MpoSource> sources;
  std::vector<float> coefs;
  // pair-grouped form (the one the kernel runs)
  std::vector<MpoPair> pairs;
  std::vector<MpoIn> ins;       // planning only
  std::vector<MpoOut> outs;
  std::vector<int32_t> rowptr;  // CSR row pointers over all output channels (+1)
  std::vector<MpoNzRec> nz;
  std::vector<MpoTask> tasks;   // warp tasks, most expensive pair first
  MpoPair *d_pairs = nullptr;
  MpoOut *d_outs = nullptr;
  int32_t *d_rowptr = nullptr;
  MpoNzRec *d_nz = nullptr;
  MpoTask *d_tasks = nullptr;
  int max_nin = 0, max_nout = 0;
  // B-tile rows of the two tcgen05 GEMMs (their B images are packed with
  // them); tuned: chosen by timed trials for this plan's shape class
  int bn1 = kTcBN, bn3 = kTcBN;
  bool tuned = false;
  // fused MPO step + .R GEMM (off by default: at the Hubbard 4x16 D=2000
  // centre bond the fused kernel takes 0.43 ms against 0.21 ms for the two
  // kernels, its producers being latency bound and recomputing a T3 tile for
  // every N tile; both forms give bit-identical results)
  bool fused = false;
  std::vector<MpoGroupMap> gmap;
  std::vector<MpoRowInfo> rowinfo;
  std::vector<MpoKChunk> kchunks;
  std::vector<MpoTgtRef> tgtref;
  MpoGroupMap *d_gmap = nullptr;
  MpoRowInfo *d_rowinfo = nullptr;
  MpoKChunk *d_kchunks = nullptr;
  MpoTgtRef *d_tgtref = nullptr;
  double mixed_flops = 0;  // tensor-core work actually issued (2MNK per group, x6 products)
  double mpo_bytes = 0;    // MPO step: 4 B per T1 entry read, 3 x 2 B per T3 entry written
  double t1_read_bytes = 0;  // 4 B per T1 entry the MPO step reads
  // host seconds spent building this plan: its tables (host_sec) and its
  // device part (allocations, operand packing, uploads; dev_sec)
  double host_sec = 0, dev_sec = 0;
  // planning only: the pack ops of L's and R's images (dropped once packed)
  std::vector<PackOp> l_ops, r_ops;
  ~SgMatvecPlan();
  void apply(const double *psi_in, double *out);
  // apply with CUDA events between the stages: ms[0] psi pack, ms[1] GEMM
  // L.psi, ms[2] MPO step, ms[3] GEMM .R
  void apply_timed(const double *psi_in, double *out, float ms[4]);
};

// L(a',w,a), R(b',w2,b) FP64 (real, or complex through the real embedding);
// S the Krylov structure of psi; fm: the fused W1 W2 coefficients (shared
// with the FP64 form's MPO step), which carry all the MPO tensors take part in.
std::unique_ptr<SgMatvecPlan> plan_sg_matvec(Ctx &ctx, const BTensor &L, const BTensor &R,
                                             const BTensor &S, FusedMpo &fm, int bn1 = kTcBN,
                                             int bn3 = kTcBN);
// The same in two parts: the host tables (no device call, so it may run on a
// host thread, with a FusedMpo of its own), then the device part (images
// allocated and packed from L's and R's data, tables uploaded).
std::unique_ptr<SgMatvecPlan> plan_sg_tables(const BTensor &L, const BTensor &R, const BTensor &S,
                                             FusedMpo &fm, int bn1, int bn3);
void plan_sg_device(Ctx &ctx, SgMatvecPlan &p, const BTensor &L, const BTensor &R);
// Shape class of the tile autotuner: element type, log2 of the Krylov
// structure's size, log2 of its largest right-bond sector.
std::array<int64_t, 3> sg_shape_class(const BTensor &S);
// B-tile rows fixed by the context or already chosen for S's shape class.
bool sg_tiles_known(const Ctx &ctx, const BTensor &S, int *bn1, int *bn3);

// The plan with the B-tile rows of the context (ctx.tc_bn1 / tc_bn3), or, where
// those are 0, the tile autotuner's: the first plan of a shape class is built
// with 64- and with 128-row B tiles, matvecs of the two alternate over four
// trials timed per stage (CUDA events, best of four), and each GEMM keeps its
// faster tile; later plans of the class reuse the choice.
std::unique_ptr<SgMatvecPlan> plan_sg_matvec_tuned(Ctx &ctx, const BTensor &L, const BTensor &R,
                                                   const BTensor &S, FusedMpo &fm);

void run_mpo_step(Ctx &ctx, const SgMatvecPlan &p);
// T3 computed in the producers of the .R GEMM: res = (W1 W2 T1) R^T
void run_tc_mpo_gemm(Ctx &ctx, const SgMatvecPlan &p, double *out);

}  // namespace udmrg
