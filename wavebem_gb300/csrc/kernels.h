// Launch wrappers shared between the CUDA translation units and the host
// orchestration (wbem_api.cu). All pointers are device pointers in the
// library's internal dof order unless stated otherwise.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "common.cuh"

namespace wbem {

constexpr int kRowsPerTile = 128;  // collocation rows per assembly CTA (one per thread)
constexpr int kColsPerTile = 20;   // dofs per surface patch: the column tile of the mixed far field
constexpr int kTileGroupF64 = 4;   // consecutive patches per column tile of the FP64 far field
constexpr int kColsPerTileF64 = kColsPerTile * kTileGroupF64;
constexpr int kRowsF64 = 64;       // collocation rows per CTA of the FP64 far field
constexpr int kMaxSet = 8;         // max size of a double-node set
constexpr int kMaxQ1 = 8;          // max regular quadrature order per direction
constexpr int kMaxSingular = 2 * 8 * 8;  // max points of a vertex-singular rule
constexpr int kBJ = 128;           // block-Jacobi block size
constexpr int kMaxDev = 64;        // devices a process may drive (per-device launch caches)

// per-panel metadata of a staged chunk (tile entry, vertex dofs, near-test data)
struct ChunkMeta {
  int cell;
  uint32_t slots;
  int owner;
  int pad;
  int4 dofs;
  float4 geo;
};

// quadrature tables (constant memory, per translation unit that uses them)
struct QuadTables {
  int q1;                            // regular order per direction
  int nsp;                           // points of each vertex-singular rule
  double gp[kMaxQ1 * kMaxQ1][3];     // regular rule: xi, eta, w
  double phi[kMaxQ1 * kMaxQ1][4];    // shape values at the regular points
  double sp[4][kMaxSingular][3];     // singular rules per vertex: xi, eta, w
  float gpf[kMaxQ1 * kMaxQ1][3];     // FP32 copies of gp / phi
  float phif[kMaxQ1 * kMaxQ1][4];
};

cudaError_t upload_quadrature(const QuadTables& t);

// ---- assembly (FP64 plain form)
cudaError_t launch_cell_records_fp64(int C, const double* X, const int4* cell_dofs, double* rec,
                                     int q1, cudaStream_t s);
cudaError_t launch_tile_fp64(int N, int q1, const double* X, const int* dnset, int n_tiles,
                             const int* tile_ptr, const int2* tile_ent, const int4* cell_dofs,
                             const double* rec, double* Nm, double* Dm, DevErr* err,
                             cudaStream_t s);
cudaError_t launch_singular_fp64(int N, const double* X, const int* dnset, const int* sptr,
                                 const int* scell, const int4* cell_dofs, double* Nm, double* Dm,
                                 DevErr* err, cudaStream_t s);
cudaError_t launch_alpha_rowsum(int N, const double* Nm, double* alpha, cudaStream_t s);

// ---- assembly (mixed form): A2 / B2 hold the selected (hi, lo) float pairs
// of the system and right-hand-side operators (context.h)
// A2, B2 of the columns in flips[0..nflip) after their boundary condition
// changed: (A2, B2) <- (-B2, -A2)
cudaError_t launch_reselect_pairs(int N, int nflip, const int* flips, float2* A2, float2* B2,
                                  cudaStream_t s);

// ---- operators and solver pieces
// y = sum_j sel(i,j) x_j (+ diagonal term), sel per mode:
//   mode 0 (system, vmult):   mask_j ? -D_ij : N_ij ; y_i += (1-mask_i) alpha_i x_i
//   mode 1 (rhs):             mask_j ? -N_ij : D_ij ; y_i -= mask_i alpha_i x_i
cudaError_t launch_matvec_fp64(int N, int mode, const double* Nm, const double* Dm,
                               const uint8_t* mask, const double* alpha, const double* x,
                               double* y, cudaStream_t s);
// mixed form: P = A2 (mode 0) or B2 (mode 1), the selection already applied
cudaError_t launch_matvec_mixed(int N, int mode, const float2* P, const uint8_t* mask,
                                const double* alpha, const double* x, double* y, cudaStream_t s);
// transposed system operator: y_j = sum_i sel(i,j) x_i (+ diagonal)
cudaError_t launch_matvec_t_fp64(int N, const double* Nm, const double* Dm, const uint8_t* mask,
                                 const double* alpha, const double* x, double* y, double* part,
                                 cudaStream_t s);
// mixed form: y_j = sum_i P_ij x_i (+ (1 - mask_j) alpha_j x_j if alpha)
cudaError_t launch_matvec_t_mixed(int N, const float2* P, const uint8_t* mask, const double* alpha,
                                  const double* x, double* y, double* part, cudaStream_t s);
// constrained rows: y_i = x_i - sum c_ij x_j
cudaError_t launch_constraint_rows(int nrows, const int* crow, const int* cptr, const int* ccol,
                                   const double* cval, const double* x, double* y,
                                   cudaStream_t s);
// constrained rows of the transposed operator (scatter form, deterministic)
cudaError_t launch_constraint_rows_t(int N, int nrows, const int* crow, const int* cptr,
                                     const int* ccol, const double* cval, const int* tptr,
                                     const int* tsrc, const double* tval,
                                     const uint8_t* cflag, const double* x, double* y,
                                     cudaStream_t s);
cudaError_t launch_set_rows(int nrows, const int* crow, const double* val, double* y,
                            cudaStream_t s);

// block-Jacobi (FP64)
cudaError_t launch_matvec_s32(int N, int ld, const float* S, const double* x, double* y,
                              cudaStream_t s);
cudaError_t launch_matvec_s32_t(int N, int ld, const float* S, const double* x, double* y,
                                double* part, cudaStream_t s);
// block-Jacobi of the system operator, from N and D (FP64), from the selected
// pairs A2 (mixed) or from precomputed diagonal blocks (FMA near field)
cudaError_t launch_bj_build(int N, const double* Nm, const double* Dm, const float2* A2,
                            const double* blocks, const uint8_t* mask, const double* alpha,
                            const uint8_t* cflag, const int* cptr_full, const int* ccol_full,
                            const double* cval_full, double* binv, DevErr* err, cudaStream_t s);
cudaError_t launch_bj_apply(int N, const double* binv, const double* x, double* y, int transpose,
                            cudaStream_t s);

// Krylov helpers (FP64)
cudaError_t launch_multidot(int N, int k, const double* V, const double* w, double* part,
                            double* out, cudaStream_t s);
cudaError_t launch_axpy_basis(int N, int k, const double* V, const double* h, double* w,
                              double sign, cudaStream_t s);
cudaError_t launch_scale(int N, const double* x, double a, double* y, cudaStream_t s);
cudaError_t launch_axpby(int N, double a, const double* x, double b, double* y, cudaStream_t s);
cudaError_t launch_nrm2(int N, const double* x, double* part, double* out, cudaStream_t s);
cudaError_t launch_gather(int N, const int* idx, const double* x, double* y, cudaStream_t s);
cudaError_t launch_scatter(int N, const int* idx, const double* x, double* y, cudaStream_t s);
// out[r][q] = A[ip[r0 + r]][ip[q]] for r < nr (caller-order rows of an
// internal-order matrix). When A is NULL the entry is read from the pairs:
// sel_j ? -P1 : P0 (N: P0 = A2, P1 = B2; D: P0 = B2, P1 = A2)
cudaError_t launch_gather_rows(int N, int r0, int nr, const int* ip, const double* A,
                               const float2* P0, const float2* P1, const uint8_t* sel, double* out,
                               cudaStream_t s);

// hull force and adjoint
cudaError_t launch_hull_force(int nh, const int4* hull_dofs, const double* X, const double* U,
                              int dir, const double* phi, const double* dphi, double* part,
                              cudaStream_t s);
cudaError_t launch_hull_force_grad(int nh, const int4* hull_dofs, const double* X,
                                   const double* U, int dir, const double* phi, const double* dphi,
                                   double* gX_cell, double* gphi_cell, double* gdphi_cell,
                                   cudaStream_t s);

}  // namespace wbem
