// Throughput probes for the roofline denominators of the CUDA-core kernels
// (FP64 and FP32 FMA rate, MUFU rsqrt rate). Built as libwbem_peaks.so and
// used by bench.py only; not part of the wbem.h ABI.
#include <cuda_runtime.h>

template <typename T>
__global__ void k_fma(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
    x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)-1.2345) out[0] = s;
}

// Packed FP32 pairs (fma.rn.f32x2): two FMAs per instruction.
__device__ __forceinline__ unsigned long long ffma2(unsigned long long a, unsigned long long b,
                                                    unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

__global__ void k_fma2(float* out, int iters, float a, float b) {
  const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
  const unsigned long long A = *reinterpret_cast<const unsigned long long*>(&a2);
  const unsigned long long B = *reinterpret_cast<const unsigned long long*>(&b2);
  unsigned long long x[8];
  for (int k = 0; k < 8; ++k) {
    const float2 v = make_float2(threadIdx.x + k, threadIdx.x + 2 * k);
    x[k] = *reinterpret_cast<const unsigned long long*>(&v);
  }
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
#pragma unroll
      for (int j = 0; j < 8; ++j) x[j] = ffma2(x[j], A, B);
    }
  }
  float s = 0.f;
  for (int k = 0; k < 8; ++k) {
    const float2 v = *reinterpret_cast<const float2*>(&x[k]);
    s += v.x + v.y;
  }
  if (s == -1.2345f) out[0] = s;
}

__global__ void k_rsqrt(float* out, int iters) {
  float x0 = threadIdx.x + 1.f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 = rsqrtf(x0); x1 = rsqrtf(x1); x2 = rsqrtf(x2); x3 = rsqrtf(x3);
    }
  }
  float s = x0 + x1 + x2 + x3;
  if (s == -1.2345f) out[0] = s;
}

extern "C" {
// kind 0: FP64 FMA, 1: FP32 FMA, 2: FP32 rsqrt, 3: packed FP32x2 FMA.
// Returns G(flop or op)/s, <0 on error.
double wbem_peak_probe(int kind) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  void* buf = nullptr;
  if (cudaMalloc(&buf, 64) != cudaSuccess) return -1;
  const int blocks = sms * 8, threads = 256;
  const int iters = kind == 0 ? 256 : 4096;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(a);
    if (kind == 0) k_fma<double><<<blocks, threads>>>((double*)buf, iters, 1.0000001, 1e-9);
    else if (kind == 1) k_fma<float><<<blocks, threads>>>((float*)buf, iters, 1.0000001f, 1e-9f);
    else if (kind == 3) k_fma2<<<blocks, threads>>>((float*)buf, iters, 1.0000001f, 1e-9f);
    else k_rsqrt<<<blocks, threads>>>((float*)buf, iters);
    cudaEventRecord(b);
    if (cudaEventSynchronize(b) != cudaSuccess) return -1;
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    // flop per inner step and thread: 8 chains x 2 (FMA) [x 2 lanes for f32x2]
    const double ops = (double)blocks * threads * iters * 16 *
                       (kind == 2 ? 4.0 : kind == 3 ? 32.0 : 16.0);
    if (rep > 0) best = ops / (ms * 1e-3) / 1e9 > best ? ops / (ms * 1e-3) / 1e9 : best;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  return best;
}
}
