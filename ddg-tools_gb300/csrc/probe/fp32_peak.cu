// Measured FP32 (non-tensor) FMA throughput of a device: the denominator of the pair kernel's
// roofline (FP32 SIMT compute, not a contraction). A measurement aid built as its own library
// (librsprobe.so), outside the product's C ABI. Each thread runs 8 independent FMA chains; one
// resident wave of 256-thread blocks per SM; the best of three timed launches after a warm-up.
#include <cuda_runtime.h>

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

// TFLOP/s of FP32 FMA on device `ordinal`; returns 0 or the CUDA error code.
extern "C" int rsp_fp32_peak(int ordinal, double *tflops) {
  cudaError_t e = cudaSetDevice(ordinal);
  if (e != cudaSuccess) return (int)e;
  int sms = 0, per_sm = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ordinal)) != cudaSuccess) return (int)e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fma_peak_kernel, 256, 0)) != cudaSuccess)
    return (int)e;
  const int grid = sms * (per_sm > 0 ? per_sm : 1), iters = 4096;
  float *out = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  float best = 1e30f;
  if ((e = cudaMalloc(&out, sizeof(float) * grid)) != cudaSuccess) return (int)e;
  if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) goto done;
  if ((e = cudaEventCreate(&a)) != cudaSuccess || (e = cudaEventCreate(&b)) != cudaSuccess) goto done;
  for (int r = 0; r < 4 && e == cudaSuccess; ++r) {
    cudaEventRecord(a, s);
    fma_peak_kernel<<<grid, 256, 0, s>>>(out, iters, 0.9999999f, 1e-7f);
    cudaEventRecord(b, s);
    if ((e = cudaEventSynchronize(b)) != cudaSuccess) break;
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    float ms = 0.f;
    if ((e = cudaEventElapsedTime(&ms, a, b)) != cudaSuccess) break;
    if (r > 0 && ms < best) best = ms;  // the first launch warms up
  }
  if (e == cudaSuccess) *tflops = 2.0 * 8 * 16 * (double)iters * 256.0 * grid / (best * 1e-3) / 1e12;
done:
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (s) cudaStreamDestroy(s);
  cudaFree(out);
  return (int)e;
}
