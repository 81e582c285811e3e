// FP64 FMA throughput probe: the denominator of the FP64 pair kernels' roofline.
// Each thread runs 8 independent FMA chains so the pipe, not latency, limits it.
#include <cuda_runtime.h>

#include "psph.h"

namespace {

__global__ void dfma_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int k = 0; k < iters; ++k) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 0.123456789) out[blockIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" psph_status psph_probe_fp64_peak(double* tflops) {
  if (!tflops) return PSPH_ERR_INVALID_ARGUMENT;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PSPH_ERR_NO_DEVICE;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return PSPH_ERR_NO_DEVICE;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * 4096) != cudaSuccess) return PSPH_ERR_OUT_OF_MEMORY;
  const int blocks = sms * 8, threads = 256, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  dfma_probe<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  const int reps = 5;
  for (int r = 0; r < reps; ++r) dfma_probe<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return PSPH_ERR_CUDA;
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads * reps;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return PSPH_OK;
}
