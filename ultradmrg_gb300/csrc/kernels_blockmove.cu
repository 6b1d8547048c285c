// Block rearrangements of block-sparse tensors (transpose, index fusion,
// expansion along an index): every source block is scattered into a
// destination block through arbitrary per-axis destination strides.
#include "blockmove.hpp"

namespace udmrg {

namespace {

// dst[dst_off + sum_k x_k dst_st[k]] = src[src_off + row-major(x)] for every
// multi-index x of the source block (dims[0..rank-1]); one CTA per operation.
__global__ void block_scatter_kernel(const BlockScatter *__restrict__ ops, int nops,
                                     const double *__restrict__ src, double *__restrict__ dst,
                                     int cplx) {
  for (int o = blockIdx.x; o < nops; o += gridDim.x) {
    const BlockScatter op = ops[o];
    int64_t tot = 1;
    for (int k = 0; k < op.rank; ++k) tot *= op.dims[k];
    for (int64_t e = threadIdx.x; e < tot; e += blockDim.x) {
      int64_t rem = e, d = op.dst_off;
      for (int k = op.rank - 1; k >= 0; --k) {
        const int64_t q = rem / op.dims[k];
        d += (rem - q * op.dims[k]) * op.dst_st[k];
        rem = q;
      }
      if (cplx)
        ((double2 *)dst)[d] = ((const double2 *)src)[op.src_off + e];
      else
        dst[d] = src[op.src_off + e];
    }
  }
}

}  // namespace

void run_block_scatter(Ctx &ctx, const std::vector<BlockScatter> &ops, const double *src,
                       double *dst, bool cplx) {
  if (ops.empty()) return;
  BlockScatter *d = (BlockScatter *)ctx.alloc(ops.size() * sizeof(BlockScatter));
  UDMRG_CHECK_CUDA(cudaMemcpyAsync(d, ops.data(), ops.size() * sizeof(BlockScatter),
                                   cudaMemcpyHostToDevice, ctx.stream));
  const int grid = (int)std::min<size_t>(ops.size(), 8 * (size_t)ctx.num_sms);
  block_scatter_kernel<<<grid, 256, 0, ctx.stream>>>(d, (int)ops.size(), src, dst, cplx ? 1 : 0);
  UDMRG_CHECK_CUDA(cudaGetLastError());
  ctx.launches++;
  ctx.free(d);
  ctx.sync();  // the host vector `ops` must outlive the upload
}

}  // namespace udmrg
