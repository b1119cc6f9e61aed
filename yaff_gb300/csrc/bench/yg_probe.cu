// yg_probe.cu -- measures the FP32 / FP64 FMA throughput of the device.
//
// The pair and Ewald kernels run on the FP32 (mixed) or FP64 (plain) CUDA-core
// pipes, not on the tensor cores, so their roofline denominator is the FMA
// issue rate of those pipes.  This probe runs independent FMA chains on every
// SM and reports TFLOP/s (one FMA = 2 flops): scalar FP32, FP64, or packed
// FP32 pairs (f32x2, two FMAs per instruction), so the FP32 denominator can be
// taken as the larger of the scalar and packed rates.  It is bounded: a fixed
// number of iterations, no waits, no atomics.
#include "../yg_internal.cuh"

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

// CH chains of float pairs: every step is one packed f32x2 FMA per chain.
template <int CH>
__global__ void __launch_bounds__(256) k_fma2_chain(float *out, int iters, float a, float b) {
  float2 x[CH];
#pragma unroll
  for (int c = 0; c < CH; c++) x[c] = make_float2((float)(threadIdx.x + c), (float)(threadIdx.x - c));
  const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < CH; c++) x[c] = __ffma2_rn(x[c], a2, b2);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < CH; c++) s += x[c].x + x[c].y;
  if (s == 12345.678f) out[threadIdx.x] = s;  // keeps the chains live
}

// CH chains of float pairs (packed FMAs) interleaved with CH scalar chains:
// measures whether the two instruction forms share one pipe.
template <int CH>
__global__ void __launch_bounds__(256) k_fma_mix_chain(float *out, int iters, float a, float b) {
  float2 x[CH];
  float y[CH];
#pragma unroll
  for (int c = 0; c < CH; c++) {
    x[c] = make_float2((float)(threadIdx.x + c), (float)(threadIdx.x - c));
    y[c] = (float)(threadIdx.x * 3 + c);
  }
  const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < CH; c++) {
      x[c] = __ffma2_rn(x[c], a2, b2);
      y[c] = fmaf(y[c], a, b);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < CH; c++) s += x[c].x + x[c].y + y[c];
  if (s == 12345.678f) out[threadIdx.x] = s;  // keeps the chains live
}

// Warp-level tensor-core MMA chains (register operands): TF32 m16n8k8 or
// FP16 m16n8k16 with FP32 accumulation, CH independent accumulators per warp.
template <int CH, bool F16>
__global__ void __launch_bounds__(256) k_mma_chain(float *out, int iters) {
  float c[CH][4];
#pragma unroll
  for (int q = 0; q < CH; q++)
#pragma unroll
    for (int e = 0; e < 4; e++) c[q][e] = 0.f;
  const unsigned lane = threadIdx.x & 31;
  unsigned a[4], b[2];
#pragma unroll
  for (int e = 0; e < 4; e++) a[e] = 0x3c003c00u ^ (lane << (e + 1));
  b[0] = 0x3c003c00u ^ lane;
  b[1] = 0x3c003c00u ^ (lane << 3);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int q = 0; q < CH; q++) {
      if (F16)
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};"
            : "+f"(c[q][0]), "+f"(c[q][1]), "+f"(c[q][2]), "+f"(c[q][3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
      else
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};"
            : "+f"(c[q][0]), "+f"(c[q][1]), "+f"(c[q][2]), "+f"(c[q][3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
    }
  }
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < CH; q++) s += c[q][0] + c[q][1] + c[q][2] + c[q][3];
  if (s == 12345.678f) out[threadIdx.x] = s;  // keeps the chains live
}

// kind: 0 scalar FP32, 1 FP64, 2 packed FP32 pairs, 3 packed and scalar
// FP32 interleaved, 4 TF32 warp MMA (m16n8k8), 5 FP16 warp MMA (m16n8k16);
// MMA flops = 2 M N K per instruction.
double run_probe(int kind, cudaStream_t st) {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  double *out = nullptr;
  if (cudaMalloc(&out, 256 * sizeof(double)) != cudaSuccess) return -1.0;
  const int CH = 8;
  const int iters = kind == 1 ? 256 : (kind >= 4 ? 2048 : 8192);
  const int blocks = nsm * 8;
  auto launch = [&]() {
    if (kind == 0)
      k_fma_chain<float, CH><<<blocks, 256, 0, st>>>((float *)out, iters, 0.999f, 0.001f);
    else if (kind == 1)
      k_fma_chain<double, CH><<<blocks, 256, 0, st>>>(out, iters, 0.999, 0.001);
    else if (kind == 2)
      k_fma2_chain<CH><<<blocks, 256, 0, st>>>((float *)out, iters, 0.999f, 0.001f);
    else if (kind == 3)
      k_fma_mix_chain<CH / 2><<<blocks, 256, 0, st>>>((float *)out, iters, 0.999f, 0.001f);
    else if (kind == 4)
      k_mma_chain<CH, false><<<blocks, 256, 0, st>>>((float *)out, iters);
    else
      k_mma_chain<CH, true><<<blocks, 256, 0, st>>>((float *)out, iters);
  };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();
  cudaEventRecord(e0, st);
  for (int r = 0; r < 5; r++) launch();
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
  double flops;
  if (kind >= 4) {
    // per warp and step: CH MMAs of 16 x 8 x (8 or 16)
    const double mnk = 16.0 * 8.0 * (kind == 4 ? 8.0 : 16.0);
    flops = 5.0 * 2.0 * mnk * CH * (double)iters * blocks * (256.0 / 32.0);
  } else {
    const double fma_per_step = (kind == 2 ? 2.0 * CH : (kind == 3 ? 1.5 * CH : 1.0 * CH));
    flops = 5.0 * 2.0 * fma_per_step * (double)iters * blocks * 256.0;
  }
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace

extern "C" double yg_probe_peak(int kind, void *stream) {
  if (kind < 0 || kind > 5) return -1.0;
  return run_probe(kind, (cudaStream_t)stream);
}
