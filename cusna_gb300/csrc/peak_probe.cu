// peak_probe.cu -- measured float64 FMA throughput of the device, the
// denominator of the simulator's float64 roofline (the simulator is bound by
// the FP64 pipe, whose peak the copy/GEMM peak measurements do not cover).
#include <cuda_runtime.h>

#include "libcusna.h"

namespace {

// 8 independent FMA chains per thread keep the pipe fed; the result is
// written so the work cannot be removed.
__global__ void dfma_loop(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) x[q] = (double)(threadIdx.x + q);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = fma(x[q], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) s += x[q];
  if (s == 1.2345e300) out[0] = s;
}

}  // namespace

extern "C" CUSNA_API cusna_status cusna_measure_fp64_tflops(double *tflops) {
  if (!tflops) return CUSNA_ERR_NULL_ARG;
  int dev = 0, sms = 0, count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1) {
    cudaGetLastError();
    return CUSNA_ERR_NO_CUDA;
  }
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return CUSNA_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  double best = 0.0;
  for (int rep = 0; rep < 6; ++rep) {
    cudaEventRecord(e0);
    dfma_loop<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    if (rep > 0 && ms > 0.f) best = best > flops / (ms * 1e-3) ? best : flops / (ms * 1e-3);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return CUSNA_ERR_CUDA;
  *tflops = best / 1e12;
  return CUSNA_OK;
}
