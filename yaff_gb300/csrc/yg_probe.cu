// yg_probe.cu -- measures the FP32 / FP64 FMA throughput of the device.
//
// The pair and Ewald kernels run on the FP32 (mixed) or FP64 (plain) CUDA-core
// pipes, not on the tensor cores, so their roofline denominator is the FMA
// issue rate of those pipes.  This probe runs independent FMA chains on every
// SM and reports TFLOP/s (one FMA = 2 flops).  It is bounded: a fixed number
// of iterations, no waits, no atomics.
#include "yg_internal.cuh"

namespace {

template <typename T, int CH>
__global__ void __launch_bounds__(256) k_fma_chain(T *out, int iters, T a, T b) {
  T x[CH];
#pragma unroll
  for (int c = 0; c < CH; c++) x[c] = (T)(threadIdx.x + c);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < CH; c++) x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < CH; c++) s += x[c];
  if (s == (T)12345.678) out[threadIdx.x] = s;  // keeps the chains live
}

template <typename T>
double run_probe(cudaStream_t st) {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  T *out = nullptr;
  if (cudaMalloc(&out, 256 * sizeof(T)) != cudaSuccess) return -1.0;
  const int CH = 8;
  const int iters = sizeof(T) == 8 ? 256 : 8192;
  const int blocks = nsm * 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chain<T, CH><<<blocks, 256, 0, st>>>(out, iters, (T)0.999, (T)0.001);
  cudaEventRecord(e0, st);
  for (int r = 0; r < 5; r++) k_fma_chain<T, CH><<<blocks, 256, 0, st>>>(out, iters, (T)0.999, (T)0.001);
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
  double flops = 5.0 * 2.0 * CH * (double)iters * blocks * 256.0;
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace

extern "C" double yg_probe_peak(int fp64, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  return fp64 ? run_probe<double>(st) : run_probe<float>(st);
}
