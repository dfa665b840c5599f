// diag.cu -- pipe-peak microbenchmarks used as roofline denominators.
//
// The plain form is bound by the FP64 pipe and the batched form by the FP32
// pipe; neither peak is a library figure, so they are measured: every thread
// runs kChains independent FMA chains (enough to cover the pipe latency), the
// grid fills every SM, and the rate is 2 flops per FMA over the event-timed
// duration.  No reference counterpart (measurement only).

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mantaray_gpu.h"

namespace {

constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(256) fma_chain_kernel(T *sink, int iters, T a, T b) {
  T acc[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) acc[c] = T(threadIdx.x + c) * T(1e-3);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) acc[c] = fma(acc[c], a, b);
  }
  T s = T(0);
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += acc[c];
  if (s == T(-1234.5)) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

template <typename T>
int measure(double *tflops, int iters) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MR_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return MR_ERR_CUDA;
  const int blocks = sms * 8, threads = 256;
  T *sink = nullptr;
  if (cudaMalloc(&sink, sizeof(T) * blocks * threads) != cudaSuccess) return MR_ERR_OUT_OF_MEMORY;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // warm-up launch, then the timed one
  fma_chain_kernel<T><<<blocks, threads>>>(sink, iters / 8, T(0.999999), T(1e-7));
  cudaEventRecord(e0);
  fma_chain_kernel<T><<<blocks, threads>>>(sink, iters, T(0.999999), T(1e-7));
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess || ms <= 0.0f) return MR_ERR_CUDA;
  const double fmas = double(blocks) * threads * kChains * double(iters);
  *tflops = 2.0 * fmas / (double(ms) * 1e-3) / 1e12;
  return MR_OK;
}

}  // namespace

extern "C" int mr_measure_fma_peak(int fp64, double *tflops) {
  if (!tflops) return MR_ERR_INVALID_ARGUMENT;
  return fp64 ? measure<double>(tflops, 1 << 14) : measure<float>(tflops, 1 << 18);
}
