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

/* Hull force from device-resident fields without touching the allocator.
 * No counterpart in the reference. For callers that must not allocate device
 * memory: a time loop that evaluates the force after every Newton iteration
 * on its own stream (allocating and freeing device memory synchronises the
 * whole device) or that runs with device memory owned by another framework's
 * caching allocator. Same integral as wbem_hull_force, but hull_cells
 * (n_hull panel indices, caller numbering), phi and dphi_dn (caller order) and
 * force (one double) are DEVICE pointers; U is a host array of 3 doubles.
 * The work is queued on `stream` (NULL: the handle's stream) and the call
 * returns without waiting; *force is valid once that stream has reached it.
 * Per-panel partial sums live in a fixed 512 KB array inside the library, so
 * n_hull is limited to 65536 (WBEM_ERR_ARG beyond). The first call on a device
 * looks up that array's device address (cudaGetSymbolAddress); make the first
 * call before any stream capture. All calls on a device share the array:
 * calls whose work overlaps on the GPU (other streams, other handles) race and
 * must be serialised by the caller. An out-of-range panel index gives NaN. */
int wbem_hull_force_noalloc(struct wbem_context* h, const int* hull_cells, int n_hull,
                            const double* U, int dir, const double* phi, const double* dphi_dn,
                            double* force, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* WBEM_KERNELS_H */
