// probe.cu - FP32 FMA throughput probe: the denominator of the pair pass's roofline.
//
// The pair pass is bound by FP32 CUDA-core issue, not by HBM or tensor cores; its roofline
// peak is measured here on the device it runs on: every thread runs 8 independent FMA chains
// for a fixed number of iterations over a grid of 8 CTAs per SM, timed with CUDA events.
#include "common.cuh"

namespace pmgb {

__global__ void __launch_bounds__(256) fma_probe_kernel(float* out, int iters, float b, float c) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
  float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
      a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
    }
  }
  const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678f) out[0] = s;  // keeps the chains live
}

}  // namespace pmgb

extern "C" int pmgb_fp32_peak_probe(float* tflops) {
  using namespace pmgb;
  if (!tflops) return set_error("null argument"), PMGB_EINVAL;
  int dev = 0, sms = 0;
  PMGB_CUDA_TRY(cudaGetDevice(&dev));
  PMGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  float* out = nullptr;
  PMGB_CUDA_TRY(cudaMalloc(&out, sizeof(float)));
  cudaEvent_t e0, e1;
  PMGB_CUDA_TRY(cudaEventCreate(&e0));
  PMGB_CUDA_TRY(cudaEventCreate(&e1));
  const int blocks = sms * 8, threads = 256, iters = 4096;
  fma_probe_kernel<<<blocks, threads>>>(out, 64, 0.9999f, 1e-6f);  // warm-up
  PMGB_CUDA_TRY(cudaEventRecord(e0));
  fma_probe_kernel<<<blocks, threads>>>(out, iters, 0.9999f, 1e-6f);
  PMGB_CUDA_TRY(cudaEventRecord(e1));
  PMGB_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  *tflops = (float)(flops / (ms * 1e-3) / 1e12);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return PMGB_OK;
}
