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
// kind 0: FP64 FMA, 1: FP32 FMA, 2: FP32 rsqrt. Returns G(flop or op)/s, <0 on error.
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
    else k_rsqrt<<<blocks, threads>>>((float*)buf, iters);
    cudaEventRecord(b);
    if (cudaEventSynchronize(b) != cudaSuccess) return -1;
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    const double ops = (double)blocks * threads * iters * 16 * (kind == 2 ? 4 : 8) * (kind == 2 ? 1 : 2);
    if (rep > 0) best = ops / (ms * 1e-3) / 1e9 > best ? ops / (ms * 1e-3) / 1e9 : best;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  return best;
}
}
