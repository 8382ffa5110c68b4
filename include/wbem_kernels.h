/*
 * wbem_kernels.h - lower-level entry points of the GB300 BEM library, for
 * kernel-level tests and benchmarks. They have no counterpart in the
 * reference's BEMProblem interface (include/bem_problem.h of the reference):
 * they expose the building blocks of the solve on device pointers.
 */
#ifndef WBEM_KERNELS_H
#define WBEM_KERNELS_H

#ifdef __cplusplus
extern "C" {
#endif

/* C (M x Nc, row-major, ld Nc) -= A (M x K, row-major) * B^T (B: Nc x K,
 * row-major), all FP32 device pointers. A and B are split into BF16 hi/lo
 * parts and multiplied as Ahi Bhi + Ahi Blo + Alo Bhi on the tcgen05 tensor
 * cores with FP32 accumulation in TMEM (the trailing update of the LU).
 * K must be a positive multiple of 64. Runs on the legacy default stream and
 * synchronizes. Returns a wbem.h status. */
int wbem_test_gemm_bf16x3(int M, int Nc, int K, const float* dA, const float* dB, float* dC);

/* Run all later work of the handle on the given cudaStream_t (NULL: back to
 * a private non-blocking stream). Lets a caller order the library's kernels
 * with its own work and time them with events on that stream. */
struct wbem_context;
int wbem_set_stream(struct wbem_context* h, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* WBEM_KERNELS_H */
