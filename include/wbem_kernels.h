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
 * K must be a positive multiple of 32. Runs on the legacy default stream and
 * synchronizes. Returns a wbem.h status. */
int wbem_test_gemm_bf16x3(int M, int Nc, int K, const float* dA, const float* dB, float* dC);

/* The same update as one TF32 product (kind::tf32 tcgen05.mma on the FP32
 * operands, FP32 accumulation in TMEM): the LU's trailing update. Same
 * arguments, conditions and synchronisation as wbem_test_gemm_bf16x3. */
int wbem_test_gemm_tf32(int M, int Nc, int K, const float* dA, const float* dB, float* dC);

/* The mixed-precision system matrix and its LU factors, for factor tests.
 * After wbem_assemble (WBEM_PREC_MIXED) and wbem_set_bc: forms the FP32
 * system matrix S (the constrained operator with alpha on its diagonal, rows
 * and columns in the library's internal dof order) and copies it to A_host
 * (n_dofs x n_dofs, row-major), factors it and copies the packed factors
 * (unit-lower L below the diagonal, U on and above it) to LU_host; perm_host
 * receives the internal order (perm_host[k] = caller dof of internal dof k).
 * Any of the three pointers may be NULL. The factors then serve the next
 * wbem_solve_system with WBEM_SOLVER_LU. Returns a wbem.h status. */
struct wbem_context;
int wbem_test_lu_factors(struct wbem_context* h, float* A_host, float* LU_host, int* perm_host);

/* z = M^{-1} v (transpose: M^{-T}) with the current LU factors M = L U, host
 * vectors of n_dofs doubles in the internal dof order (the order of
 * wbem_test_lu_factors). Call after wbem_test_lu_factors or a solve with
 * WBEM_SOLVER_LU. Returns a wbem.h status. */
int wbem_test_lu_apply(struct wbem_context* h, const double* v, double* z, int transpose);

/* Kernel profiling. With profiling on, the LU factorisation runs on the
 * handle's stream alone (no look-ahead overlap) and every launch of the
 * kernel classes below is bracketed by CUDA events on that stream, so the
 * sums are the kernels' own device times. Meant for a separate, instrumented
 * pass next to the timed one. The profile covers the last factorisation and
 * the solves since then (reset by each factorisation). */
typedef struct {
  double gemm_ms;       /* k_gemm_tc<TF32>: tensor-core trailing updates */
  double gemm_flop;     /*   their work: 2 M N K per launch (one TF32 product) */
  int gemm_launches;
  double diag_ms;       /* k_diag_block: 128 x 128 diagonal LU + triangle inverses */
  int diag_launches;
  double panel_ms;      /* k_panel_gemm + k_rowpanel_update (FP32 SIMT panels) */
  int panel_launches;
  double matvec_ms;     /* system mat-vecs of the refinement (k_matvec_mixed) */
  double matvec_bytes;  /*   matrix bytes they stream: 8 N^2 per launch */
  int matvec_launches;
  double trsv_ms;       /* k_trsv_wave: block triangular sweeps */
  double trsv_bytes;    /*   factor bytes they stream: 2 N^2 per sweep */
  int trsv_launches;
  int reserved[8];
} wbem_kernel_profile;
int wbem_set_profiling(struct wbem_context* h, int on);
int wbem_get_kernel_profile(struct wbem_context* h, wbem_kernel_profile* p);

/* Run all later work of the handle on the given cudaStream_t (NULL: back to
 * a private non-blocking stream). Lets a caller order the library's kernels
 * with its own work and time them with events on that stream. */
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
 * looks up that array's device address (cudaGetSymbolAddress, once per device
 * and thread-safe); make the first call before any stream capture, and reload
 * the library after a cudaDeviceReset. All calls on a device share the array:
 * calls whose work overlaps on the GPU (other streams, other handles) race and
 * must be serialised by the caller. The quadrature rule is the handle's, the
 * one wbem_hull_force uses. The calling thread's current device is the same
 * on return as on entry. An out-of-range panel index gives NaN. */
int wbem_hull_force_noalloc(struct wbem_context* h, const int* hull_cells, int n_hull,
                            const double* U, int dir, const double* phi, const double* dphi_dn,
                            double* force, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* WBEM_KERNELS_H */
