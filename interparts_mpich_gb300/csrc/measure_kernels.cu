// measure_kernels.cu -- FP64 issue-rate calibration for the roofline of the
// FP64-bound kernels (no counterpart in the reference).  Independent chains
// of fused multiply-adds in every thread of a grid that fills all SMs; the
// achieved rate is the denominator the bench divides FP64-bound kernels by.
#include <cuda_runtime.h>

#include "../../include/ibm_rk3.h"

namespace {

constexpr int FMA_CHAINS = 8, FMA_ITERS = 4096;

__global__ void __launch_bounds__(256) k_fp64_fma(double *out, double b, double c) {
  double a[FMA_CHAINS];
#pragma unroll
  for (int q = 0; q < FMA_CHAINS; ++q) a[q] = 1e-3 * (threadIdx.x + q);
  for (int it = 0; it < FMA_ITERS; ++it)
#pragma unroll
    for (int q = 0; q < FMA_CHAINS; ++q) a[q] = fma(a[q], b, c);
  double s = 0.;
#pragma unroll
  for (int q = 0; q < FMA_CHAINS; ++q) s += a[q];
  if (s == 12345.678) out[blockIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" int ibm_fp64_peak(double *tflops) {
  if (!tflops) return IBM_E_INVALID;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return IBM_E_CUDA;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return IBM_E_CUDA;
  double *out = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = IBM_OK;
  const int blocks = nsm * 8, threads = 256;
  float best = 0.f;
  if (cudaMalloc((void **)&out, blocks * sizeof(double)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    st = IBM_E_CUDA;
  } else {
    for (int rep = 0; rep < 4 && st == IBM_OK; ++rep) {
      cudaEventRecord(e0, s);
      k_fp64_fma<<<blocks, threads, 0, s>>>(out, 0.999999, 1e-9);
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) != cudaSuccess) { st = IBM_E_CUDA; break; }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // the first launch warms up
    }
  }
  if (st == IBM_OK && cudaGetLastError() != cudaSuccess) st = IBM_E_CUDA;
  if (st == IBM_OK) {
    const double flops = 2.0 * FMA_CHAINS * FMA_ITERS * (double)blocks * threads;
    *tflops = best > 0.f ? flops / (best * 1e-3) / 1e12 : 0.;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  if (out) cudaFree(out);
  return st;
}
