// Host-side helpers shared by the translation units that orchestrate kernels.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>
#include "context.h"

namespace wbem {

inline int fail(wbem_context* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

template <typename T>
int dev_alloc(wbem_context* h, T** p, size_t n) {
  if (*p) {
    cudaFree(*p);
    *p = nullptr;
  }
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(h, WBEM_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  return WBEM_OK;
}

template <typename T>
int upload(wbem_context* h, T** p, const std::vector<T>& v) {
  int s = dev_alloc(h, p, v.size());
  if (s != WBEM_OK) return s;
  if (!v.empty()) {
    cudaError_t e = cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(h, WBEM_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
  }
  return WBEM_OK;
}

int check_device_error(wbem_context* h, const char* what);

// Frees the device pointers held in the listed variables when it goes out of
// scope. The variables are read at that point, so buffers allocated after the
// guard was set up are freed on every return path, early error returns
// included.
struct DeviceFreeGuard {
  std::vector<void**> slots;
  ~DeviceFreeGuard() {
    for (void** s : slots)
      if (*s) cudaFree(*s);
  }
};

struct EvTimer {
  cudaEvent_t a, b;
  cudaStream_t s;
  explicit EvTimer(cudaStream_t st) : s(st) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
  }
  double ms() {
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float t = 0;
    cudaEventElapsedTime(&t, a, b);
    cudaEventRecord(a, s);
    return t;
  }
  ~EvTimer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

}  // namespace wbem

#define WB_CU(call)                                                                          \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return ::wbem::fail(h, e_ == cudaErrorMemoryAllocation ? WBEM_ERR_NOMEM : WBEM_ERR_CUDA, \
                          std::string(#call) + ": " + cudaGetErrorString(e_));               \
  } while (0)

#define WB_CHK(expr)               \
  do {                             \
    int s_ = (expr);               \
    if (s_ != WBEM_OK) return s_;  \
  } while (0)
