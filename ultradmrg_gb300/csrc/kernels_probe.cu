// FP64 throughput probe: independent DFMA chains, no memory traffic.  Gives
// the FP64 roofline denominator on the running GPU (the plain FP64 form of
// the block GEMMs is bound by this pipe).
#include "../../include/ultradmrg_gb300.h"
#include "btensor.hpp"

namespace udmrg {

namespace {

__global__ void dfma_probe_kernel(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 1.2345) out[0] = s;  // keeps the chains alive
}

}  // namespace

double probe_fp64_tflops(Ctx &ctx) {
  double *d = (double *)ctx.alloc(sizeof(double));
  const int threads = 256, blocks = ctx.num_sms * 8, iters = 1 << 14;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  dfma_probe_kernel<<<blocks, threads, 0, ctx.stream>>>(d, 256, 1.0000001, 1e-9);  // warm-up
  cudaEventRecord(e0, ctx.stream);
  dfma_probe_kernel<<<blocks, threads, 0, ctx.stream>>>(d, iters, 1.0000001, 1e-9);
  cudaEventRecord(e1, ctx.stream);
  UDMRG_CHECK_CUDA(cudaEventSynchronize(e1));
  UDMRG_CHECK_CUDA(cudaGetLastError());
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx.launches += 2;
  ctx.free(d);
  const double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace udmrg
