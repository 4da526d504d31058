// Measured FP32 (non-tensor) FMA throughput of the device: the denominator of the pair
// kernel's roofline (it is FP32 SIMT compute, not a contraction). Each thread runs 8
// independent FMA chains; one persistent wave of blocks per SM.
#include "common.hpp"

namespace {

__global__ void fma_peak_kernel(float *out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1e-7f, x2 = x0 + 2e-7f, x3 = x0 + 3e-7f;
  float x4 = x0 + 4e-7f, x5 = x0 + 5e-7f, x6 = x0 + 6e-7f, x7 = x0 + 7e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      x0 = fmaf(x0, a, b), x1 = fmaf(x1, a, b), x2 = fmaf(x2, a, b), x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b), x5 = fmaf(x5, a, b), x6 = fmaf(x6, a, b), x7 = fmaf(x7, a, b);
    }
  }
  float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" int rs_fp32_peak(rs_ctx *ctx, double *tflops) {
  return rsg::guard([&] {
    ctx->use();
    int per_sm = 0;
    RSG_CUDA("launch", cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fma_peak_kernel, 256, 0));
    int grid = ctx->sm_count * (per_sm > 0 ? per_sm : 1);
    rsg::DevBuf<float> out((size_t)grid);
    const int iters = 4096;
    cudaEvent_t a, b;
    RSG_CUDA("launch", cudaEventCreate(&a));
    RSG_CUDA("launch", cudaEventCreate(&b));
    float best = 1e30f;
    for (int r = 0; r < 4; ++r) {
      RSG_CUDA("launch", cudaEventRecord(a, ctx->stream));
      fma_peak_kernel<<<grid, 256, 0, ctx->stream>>>(out.p, iters, 0.9999999f, 1e-7f);
      RSG_LAUNCHED(ctx, "fma_peak");
      RSG_CUDA("launch", cudaEventRecord(b, ctx->stream));
      RSG_CUDA("launch", cudaEventSynchronize(b));
      float ms = 0.f;
      RSG_CUDA("launch", cudaEventElapsedTime(&ms, a, b));
      if (r > 0 && ms < best) best = ms;  // first run warms up
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    double flops = 2.0 * 8 * 16 * (double)iters * 256.0 * grid;
    *tflops = flops / (best * 1e-3) / 1e12;
  });
}
