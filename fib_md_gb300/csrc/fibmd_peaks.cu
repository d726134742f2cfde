// fibmd_peaks.cu — measured FMA issue rates of this GPU.
//
// The force kernel is bound by the binary64 (plain path) or binary32
// (mixed path) arithmetic pipes, neither of which has a vendor-measured
// figure in the run's peak table. These loops time independent FMA chains
// (8 per thread, enough to hide the pipe latency) over a grid that fills
// every SM, and report TFLOP/s with an FMA counted as 2 flops.
#include <cuda_runtime.h>

#include "fibmd_internal.cuh"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_loop(T* out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = (T)(threadIdx.x + k) * (T)1e-3;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = x[k] * a + b;
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  if (s == (T)12345.678) out[0] = s;  // keeps the chains live
}

template <typename T>
double time_fma(int sms, int iters) {
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return -1.0;
  const int blocks = sms * 8, threads = 256;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_loop<T><<<blocks, threads>>>(out, iters / 8, (T)0.999999, (T)1e-7);  // warm-up
  cudaEventRecord(e0);
  k_fma_loop<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
  const double fmas = (double)blocks * threads * 8.0 * iters;
  return 2.0 * fmas / (ms * 1e-3) / 1e12;
}

}  // namespace

extern "C" int fibmd_gpu_pipe_peaks(double* fp64_tflops, double* fp32_tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FIBMD_ECUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (fp64_tflops) *fp64_tflops = time_fma<double>(sms, 1 << 12);
  if (fp32_tflops) *fp32_tflops = time_fma<float>(sms, 1 << 16);
  return (fp64_tflops && *fp64_tflops < 0) || (fp32_tflops && *fp32_tflops < 0) ? FIBMD_ECUDA
                                                                               : FIBMD_OK;
}
