// Operators of the mixed Dirichlet/Neumann system and the pieces of the
// Krylov solvers.
//
// The system is never formed in full: the GMRES mat-vec streams N and D once
// and picks, per column, the block that the column's boundary condition needs
// (BEMProblem<3>::vmult, source/bem_problem.cc:620-670: A x = -D (x s) + N (x o)
// + alpha (x o)); the right-hand side uses the complementary blocks
// (compute_rhs, :673-706). Constrained rows are replaced afterwards
// (ConstrainedOperator::vmult / distribute_rhs, include/constrained_matrix.h:72-94).
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include "kernels.h"
#include "../../include/wbem.h"

namespace wbem {

constexpr int kMvChunk = 2048;  // columns staged per chunk
constexpr int kMvWarps = 8;     // rows per block (one warp each)

// y_i = sum_j sel(i,j) x_j + diag. FP64 matrices.
__global__ void __launch_bounds__(kMvWarps * 32)
    k_matvec_fp64(int N, int mode, const double* __restrict__ Nm, const double* __restrict__ Dm,
                  const uint8_t* __restrict__ mask, const double* __restrict__ alpha,
                  const double* __restrict__ x, double* __restrict__ y) {
  __shared__ double xs[kMvChunk];
  __shared__ uint8_t ms[kMvChunk];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * kMvWarps + warp;
  const bool active = row < N;
  // mode 0: mask ? -D : N ; mode 1: mask ? -N : D
  const double* A0 = (mode == 0) ? Nm : Dm;  // used where mask == 0
  const double* A1 = (mode == 0) ? Dm : Nm;  // used (negated) where mask == 1
  const double* r0 = A0 + (size_t)(active ? row : 0) * N;
  const double* r1 = A1 + (size_t)(active ? row : 0) * N;
  double acc = 0.0;
  for (int c0 = 0; c0 < N; c0 += kMvChunk) {
    const int cn = min(kMvChunk, N - c0);
    __syncthreads();
    for (int k = threadIdx.x; k < cn; k += blockDim.x) {
      xs[k] = x[c0 + k];
      ms[k] = mask[c0 + k];
    }
    __syncthreads();
    if (active) {
#pragma unroll 8
      for (int k = lane; k < cn; k += 32) {
        const int j = c0 + k;
        const double v = ms[k] ? -__ldcs(r1 + j) : __ldcs(r0 + j);
        acc = fma(v, xs[k], acc);
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (active && lane == 0) {
    const double xi = x[row];
    if (mode == 0) {
      if (!mask[row]) acc = fma(alpha[row], xi, acc);
    } else {
      if (mask[row]) acc = fma(-alpha[row], xi, acc);
    }
    y[row] = acc;
  }
}

cudaError_t launch_matvec_fp64(int N, int mode, const double* Nm, const double* Dm,
                               const uint8_t* mask, const double* alpha, const double* x,
                               double* y, cudaStream_t s) {
  k_matvec_fp64<<<(N + kMvWarps - 1) / kMvWarps, kMvWarps * 32, 0, s>>>(N, mode, Nm, Dm, mask,
                                                                         alpha, x, y);
  return cudaGetLastError();
}

// Same operator with (hi, lo) float pairs whose boundary-condition selection
// was applied at assembly (P = A2 for mode 0, B2 for mode 1): one contiguous
// matrix per apply. entry = hi + lo; products and sums in double-float on
// FP32 units, x given in FP64 and split on the fly.
__global__ void __launch_bounds__(kMvWarps * 32)
    k_matvec_mixed(int N, int mode, const float2* __restrict__ P, const uint8_t* __restrict__ mask,
                   const double* __restrict__ alpha, const double* __restrict__ x,
                   double* __restrict__ y) {
  __shared__ float2 xs[kMvChunk];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * kMvWarps + warp;
  const bool active = row < N;
  const float2* r0 = P + (size_t)(active ? row : 0) * N;
  df acc = {0.f, 0.f};
  for (int c0 = 0; c0 < N; c0 += kMvChunk) {
    const int cn = min(kMvChunk, N - c0);
    __syncthreads();
    for (int k = threadIdx.x; k < cn; k += blockDim.x) {
      const df v = df_from_double(x[c0 + k]);
      xs[k] = make_float2(v.hi, v.lo);
    }
    __syncthreads();
    if (active) {
#pragma unroll 8
      for (int k = lane; k < cn; k += 32) {
        const float2 a = __ldcs(r0 + c0 + k);
        const float2 xv = xs[k];
        df p = two_prod(a.x, xv.x);
        p.lo = __fmaf_rn(a.x, xv.y, __fmaf_rn(a.y, xv.x, p.lo));
        acc = df_add(acc, p);
      }
    }
  }
  double s = df_to_double(acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (active && lane == 0) {
    const double xi = x[row];
    if (mode == 0) {
      if (!mask[row]) s = fma(alpha[row], xi, s);
    } else {
      if (mask[row]) s = fma(-alpha[row], xi, s);
    }
    y[row] = s;
  }
}

cudaError_t launch_matvec_mixed(int N, int mode, const float2* P, const uint8_t* mask,
                                const double* alpha, const double* x, double* y, cudaStream_t s) {
  k_matvec_mixed<<<(N + kMvWarps - 1) / kMvWarps, kMvWarps * 32, 0, s>>>(N, mode, P, mask, alpha,
                                                                          x, y);
  return cudaGetLastError();
}

// y = S x for the FP32 system matrix S (row-major, leading dimension ld, the
// constrained operator with alpha on its diagonal): the inner operator of the
// refinement solver. One warp per row, each lane streams float4 quads of the
// row; products and sums in FP32 with the lane sums moved into FP64 after
// every chunk of kMvChunk columns (64 terms per FP32 partial sum), so the
// operator is S to about 1e-6 relative, at 4 bytes of HBM traffic per entry.
__global__ void __launch_bounds__(kMvWarps * 32)
    k_matvec_s32(int N, int ld, const float* __restrict__ S, const double* __restrict__ x,
                 double* __restrict__ y) {
  __shared__ __align__(16) float xs[kMvChunk];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * kMvWarps + warp;
  const bool active = row < N;
  const float* sr = S + (size_t)(active ? row : 0) * ld;
  double acc = 0.0;
  for (int c0 = 0; c0 < N; c0 += kMvChunk) {
    const int cn = min(kMvChunk, N - c0);
    __syncthreads();
    for (int k = threadIdx.x; k < kMvChunk; k += blockDim.x)
      xs[k] = (k < cn) ? (float)x[c0 + k] : 0.f;
    __syncthreads();
    if (active) {
      float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
      const int cq = cn & ~3;  // whole quads (row starts are 16-byte aligned)
#pragma unroll 4
      for (int k = 4 * lane; k < cq; k += 128) {
        const float4 v = __ldcs(reinterpret_cast<const float4*>(sr + c0 + k));
        const float4 xv = *reinterpret_cast<const float4*>(xs + k);
        a0 = __fmaf_rn(v.x, xv.x, a0);
        a1 = __fmaf_rn(v.y, xv.y, a1);
        a2 = __fmaf_rn(v.z, xv.z, a2);
        a3 = __fmaf_rn(v.w, xv.w, a3);
      }
      for (int k = cq + lane; k < cn; k += 32) a0 = __fmaf_rn(sr[c0 + k], xs[k], a0);
      acc += ((double)a0 + (double)a1) + ((double)a2 + (double)a3);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (active && lane == 0) y[row] = acc;
}

cudaError_t launch_matvec_s32(int N, int ld, const float* S, const double* x, double* y,
                              cudaStream_t s) {
  k_matvec_s32<<<(N + kMvWarps - 1) / kMvWarps, kMvWarps * 32, 0, s>>>(N, ld, S, x, y);
  return cudaGetLastError();
}

// Transposed system operator y_j = sum_i sel(i,j) x_i + (1 - mask_j) alpha_j x_j.
// Blocks own column strips of 256 columns and a slice of rows; partial sums
// go to part[slice][N] and are added in a fixed order (deterministic).
constexpr int kMvtCols = 256;
constexpr int kMvtSlices = 32;

template <typename T>
__device__ __forceinline__ double load_entry(const T* p);
template <>
__device__ __forceinline__ double load_entry<double>(const double* p) {
  return __ldcs(p);
}

// sel: the column mask that picks N or -D (NULL: Nm already holds the
// selected operator)
template <typename T>
__global__ void k_matvec_t(int N, const T* __restrict__ Nm, const T* __restrict__ Dm,
                           const uint8_t* __restrict__ sel, const double* __restrict__ x,
                           double* __restrict__ part) {
  const int col = blockIdx.x * kMvtCols + threadIdx.x;
  const int slice = blockIdx.y;
  const int rows_per = (N + kMvtSlices - 1) / kMvtSlices;
  const int r0 = slice * rows_per, r1 = min(N, r0 + rows_per);
  if (col >= N) return;
  const bool m = sel != nullptr && sel[col] != 0;
  const T* A = m ? Dm : Nm;
  double acc = 0.0;
  for (int i = r0; i < r1; ++i) acc = fma(load_entry<T>(A + (size_t)i * N + col), x[i], acc);
  part[(size_t)slice * N + col] = m ? -acc : acc;
}

__global__ void k_matvec_t_finish(int N, const uint8_t* __restrict__ mask,
                                  const double* __restrict__ alpha, const double* __restrict__ x,
                                  const double* __restrict__ part, double* __restrict__ y) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  double s = 0;
  for (int k = 0; k < kMvtSlices; ++k) s += part[(size_t)k * N + j];
  if (alpha && !mask[j]) s = fma(alpha[j], x[j], s);
  y[j] = s;
}

cudaError_t launch_matvec_t_fp64(int N, const double* Nm, const double* Dm, const uint8_t* mask,
                                 const double* alpha, const double* x, double* y, double* part,
                                 cudaStream_t s) {
  dim3 g((N + kMvtCols - 1) / kMvtCols, kMvtSlices);
  k_matvec_t<double><<<g, kMvtCols, 0, s>>>(N, Nm, Dm, mask, x, part);
  k_matvec_t_finish<<<(N + 255) / 256, 256, 0, s>>>(N, mask, alpha, x, part, y);
  return cudaGetLastError();
}

// Transposed operator with (hi, lo) float pairs (P = A2 or B2, selection
// applied at assembly): threads own columns, blocks own a column strip and a
// slice of rows; the slice's x is split into float pairs in shared memory and
// products and sums run in double-float on FP32 units, as in k_matvec_mixed.
constexpr int kMvtChunk = 256;
__global__ void __launch_bounds__(kMvtCols)
    k_matvec_t_mixed(int N, const float2* __restrict__ P, const double* __restrict__ x,
                     double* __restrict__ part) {
  __shared__ float2 xs[kMvtChunk];
  const int col = blockIdx.x * kMvtCols + threadIdx.x;
  const int slice = blockIdx.y;
  const int rows_per = (N + kMvtSlices - 1) / kMvtSlices;
  const int r0 = slice * rows_per, r1 = min(N, r0 + rows_per);
  const bool active = col < N;
  df acc = {0.f, 0.f};
  for (int i0 = r0; i0 < r1; i0 += kMvtChunk) {
    const int n = min(kMvtChunk, r1 - i0);
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += kMvtCols) {
      const df v = df_from_double(x[i0 + k]);
      xs[k] = make_float2(v.hi, v.lo);
    }
    __syncthreads();
    if (active) {
      const float2* a_col = P + (size_t)i0 * N + col;
#pragma unroll 8
      for (int k = 0; k < n; ++k) {
        const float2 a = __ldcs(a_col + (size_t)k * N);
        const float2 xv = xs[k];
        df p = two_prod(a.x, xv.x);
        p.lo = __fmaf_rn(a.x, xv.y, __fmaf_rn(a.y, xv.x, p.lo));
        acc = df_add(acc, p);
      }
    }
  }
  if (active) part[(size_t)slice * N + col] = df_to_double(acc);
}

cudaError_t launch_matvec_t_mixed(int N, const float2* P, const uint8_t* mask, const double* alpha,
                                  const double* x, double* y, double* part, cudaStream_t s) {
  dim3 g((N + kMvtCols - 1) / kMvtCols, kMvtSlices);
  k_matvec_t_mixed<<<g, kMvtCols, 0, s>>>(N, P, x, part);
  k_matvec_t_finish<<<(N + 255) / 256, 256, 0, s>>>(N, mask, alpha, x, part, y);
  return cudaGetLastError();
}

// y = S^T x for the FP32 system matrix: threads own columns, blocks own a
// column strip and a slice of rows; FP32 partial sums over 64 rows at a time,
// moved into FP64, then the slices are added in a fixed order.
__global__ void k_matvec_s32_t(int N, int ld, const float* __restrict__ S,
                               const double* __restrict__ x, double* __restrict__ part) {
  const int col = blockIdx.x * kMvtCols + threadIdx.x;
  const int slice = blockIdx.y;
  const int rows_per = (N + kMvtSlices - 1) / kMvtSlices;
  const int r0 = slice * rows_per, r1 = min(N, r0 + rows_per);
  if (col >= N) return;
  double acc = 0.0;
  for (int i0 = r0; i0 < r1; i0 += 64) {
    const int i1 = min(r1, i0 + 64);
    float a = 0.f;
    for (int i = i0; i < i1; ++i) a = __fmaf_rn(__ldcs(S + (size_t)i * ld + col), (float)x[i], a);
    acc += (double)a;
  }
  part[(size_t)slice * N + col] = acc;
}

cudaError_t launch_matvec_s32_t(int N, int ld, const float* S, const double* x, double* y,
                                double* part, cudaStream_t s) {
  dim3 g((N + kMvtCols - 1) / kMvtCols, kMvtSlices);
  k_matvec_s32_t<<<g, kMvtCols, 0, s>>>(N, ld, S, x, part);
  k_matvec_t_finish<<<(N + 255) / 256, 256, 0, s>>>(N, nullptr, nullptr, x, part, y);
  return cudaGetLastError();
}

// Constrained rows: y_i = x_i - sum_j c_ij x_j.
__global__ void k_constraint_rows(int nrows, const int* __restrict__ crow,
                                  const int* __restrict__ cptr, const int* __restrict__ ccol,
                                  const double* __restrict__ cval, const double* __restrict__ x,
                                  double* __restrict__ y) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nrows) return;
  const int i = crow[k];
  double v = x[i];
  for (int e = cptr[k]; e < cptr[k + 1]; ++e) v -= cval[e] * x[ccol[e]];
  y[i] = v;
}

cudaError_t launch_constraint_rows(int nrows, const int* crow, const int* cptr, const int* ccol,
                                   const double* cval, const double* x, double* y,
                                   cudaStream_t s) {
  if (nrows == 0) return cudaSuccess;
  k_constraint_rows<<<(nrows + 127) / 128, 128, 0, s>>>(nrows, crow, cptr, ccol, cval, x, y);
  return cudaGetLastError();
}

// Transposed constrained operator. With C the set of constrained rows,
// (A_c^T y)_j = [j in C] y_j - sum_{i in C} c_ij y_i + [j not... ] the
// unconstrained part sum_{i not in C} A_ij y_i. The caller zeroes y_i for
// i in C before the transposed mat-vec; this kernel adds the constraint
// part: out_j += [j in C] y_j - sum_{i in C, (i,j) entry} c_ij y_i, using the
// column-major (transposed) entry lists tptr/tsrc/tval.
__global__ void k_constraint_rows_t(int N, const int* __restrict__ tptr,
                                    const int* __restrict__ tsrc, const double* __restrict__ tval,
                                    const uint8_t* __restrict__ cflag,
                                    const double* __restrict__ yin, double* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  double v = out[j];
  if (cflag[j]) v += yin[j];
  for (int e = tptr[j]; e < tptr[j + 1]; ++e) v -= tval[e] * yin[tsrc[e]];
  out[j] = v;
}

cudaError_t launch_constraint_rows_t(int N, int nrows, const int* crow, const int* cptr,
                                     const int* ccol, const double* cval, const int* tptr,
                                     const int* tsrc, const double* tval, const uint8_t* cflag,
                                     const double* x, double* y, cudaStream_t s) {
  (void)nrows; (void)crow; (void)cptr; (void)ccol; (void)cval;
  k_constraint_rows_t<<<(N + 255) / 256, 256, 0, s>>>(N, tptr, tsrc, tval, cflag, x, y);
  return cudaGetLastError();
}

__global__ void k_set_rows(int nrows, const int* __restrict__ crow, const double* __restrict__ val,
                           double* __restrict__ y) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nrows) return;
  y[crow[k]] = val[k];
}

cudaError_t launch_set_rows(int nrows, const int* crow, const double* val, double* y,
                            cudaStream_t s) {
  if (nrows == 0) return cudaSuccess;
  k_set_rows<<<(nrows + 127) / 128, 128, 0, s>>>(nrows, crow, val, y);
  return cudaGetLastError();
}

// ------------------------------------------------------------ block-Jacobi
// Diagonal blocks of the constrained system, inverted by Gauss-Jordan with
// partial pivoting, one CTA per block. binv[b] holds the inverse transposed
// (column k of the inverse contiguous) for coalesced application.
__global__ void __launch_bounds__(kBJ)
    k_bj_build(int N, const double* __restrict__ Nm, const double* __restrict__ Dm,
               const float2* __restrict__ A2, const double* __restrict__ blocks,
               const uint8_t* __restrict__ mask,
               const double* __restrict__ alpha,
               const uint8_t* __restrict__ cflag, const int* __restrict__ cptr,
               const int* __restrict__ ccol, const double* __restrict__ cval,
               double* __restrict__ binv, DevErr* err) {
  extern __shared__ __align__(16) unsigned char smem_bj[];
  double* A = reinterpret_cast<double*>(smem_bj);  // [kBJ][kBJ + 1]
  constexpr int LD = kBJ + 1;
  __shared__ int perm[kBJ];
  __shared__ double redv[kBJ];
  __shared__ int redi[kBJ];
  const int b = blockIdx.x;
  const int r = threadIdx.x;
  const int i = b * kBJ + r;
  const int c0 = b * kBJ;
  // gather the block row of thread r
  for (int c = 0; c < kBJ; ++c) {
    const int j = c0 + c;
    double v;
    if (i >= N || j >= N) {
      v = (r == c) ? 1.0 : 0.0;
    } else if (cflag[i]) {
      v = (r == c) ? 1.0 : 0.0;
    } else if (blocks) {  // the system's diagonal block, free term included
      v = blocks[((size_t)b * kBJ + r) * kBJ + c];
    } else {
      const size_t o = (size_t)i * N + j;
      if (Nm) v = mask[j] ? -Dm[o] : Nm[o];
      else v = (double)A2[o].x + (double)A2[o].y;  // selected at assembly
      if (i == j && !mask[j]) v += alpha[i];
    }
    A[r * LD + c] = v;
  }
  if (i < N && cflag[i]) {
    for (int e = cptr[i]; e < cptr[i + 1]; ++e) {
      const int j = ccol[e];
      if (j >= c0 && j < c0 + kBJ) A[r * LD + (j - c0)] -= cval[e];
    }
  }
  perm[r] = r;
  __syncthreads();
  for (int k = 0; k < kBJ; ++k) {
    // pivot search over rows >= k
    redv[r] = (r >= k) ? fabs(A[r * LD + k]) : -1.0;
    redi[r] = r;
    __syncthreads();
    for (int s = kBJ / 2; s > 0; s >>= 1) {
      if (r < s && redv[r + s] > redv[r]) {
        redv[r] = redv[r + s];
        redi[r] = redi[r + s];
      }
      __syncthreads();
    }
    const int p = redi[0];
    const double pv = redv[0];
    if (!(pv > 0.0)) {
      if (r == 0) dev_fail(err, WBEM_ERR_SINGULAR, 31, b, k);
      return;
    }
    if (p != k) {
      for (int c = r; c < kBJ; c += blockDim.x) {
        const double t = A[k * LD + c];
        A[k * LD + c] = A[p * LD + c];
        A[p * LD + c] = t;
      }
      if (r == 0) {
        const int t = perm[k];
        perm[k] = perm[p];
        perm[p] = t;
      }
    }
    __syncthreads();
    const double inv = 1.0 / A[k * LD + k];
    __syncthreads();
    if (r == k) {
      for (int c = 0; c < kBJ; ++c) A[k * LD + c] *= inv;
      A[k * LD + k] = inv;
    }
    __syncthreads();
    if (r != k) {
      const double f = A[r * LD + k];
      if (f != 0.0) {
        for (int c = 0; c < kBJ; ++c)
          if (c != k) A[r * LD + c] -= f * A[k * LD + c];
        A[r * LD + k] = -f * A[k * LD + k];
      }
    }
    __syncthreads();
  }
  // The in-place Gauss-Jordan above computed inv(P A) with P the row
  // permutation; inv(A) = inv(P A) P, i.e. column perm[k] of inv(A) is column
  // k of the computed matrix. Store transposed: binv[col][row].
  double* out = binv + (size_t)b * kBJ * kBJ;
  for (int c = 0; c < kBJ; ++c) out[(size_t)perm[c] * kBJ + r] = A[r * LD + c];
}

cudaError_t launch_bj_build(int N, const double* Nm, const double* Dm, const float2* A2,
                            const double* blocks, const uint8_t* mask, const double* alpha,
                            const uint8_t* cflag, const int* cptr_full, const int* ccol_full,
                            const double* cval_full, double* binv, DevErr* err, cudaStream_t s) {
  const size_t smem = (size_t)kBJ * (kBJ + 1) * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(k_bj_build, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  const int nb = (N + kBJ - 1) / kBJ;
  k_bj_build<<<nb, kBJ, smem, s>>>(N, Nm, Dm, A2, blocks, mask, alpha, cflag, cptr_full, ccol_full,
                                   cval_full, binv, err);
  return cudaGetLastError();
}

__global__ void k_bj_apply(int N, const double* __restrict__ binv, const double* __restrict__ x,
                           double* __restrict__ y, int transpose) {
  __shared__ double xs[kBJ];
  const int b = blockIdx.x, r = threadIdx.x;
  const int i = b * kBJ + r;
  xs[r] = (i < N) ? x[i] : 0.0;
  __syncthreads();
  const double* B = binv + (size_t)b * kBJ * kBJ;
  double s = 0;
  if (!transpose) {
    for (int k = 0; k < kBJ; ++k) s = fma(B[(size_t)k * kBJ + r], xs[k], s);
  } else {
    for (int k = 0; k < kBJ; ++k) s = fma(B[(size_t)r * kBJ + k], xs[k], s);
  }
  if (i < N) y[i] = s;
}

cudaError_t launch_bj_apply(int N, const double* binv, const double* x, double* y, int transpose,
                            cudaStream_t s) {
  k_bj_apply<<<(N + kBJ - 1) / kBJ, kBJ, 0, s>>>(N, binv, x, y, transpose);
  return cudaGetLastError();
}

// ------------------------------------------------------------ Krylov helpers
constexpr int kRedBlocks = 120;

__global__ void k_multidot(int N, int k, const double* __restrict__ V, const double* __restrict__ w,
                           double* __restrict__ part) {
  __shared__ double red[256];
  const int per = (N + gridDim.x - 1) / gridDim.x;
  const int i0 = blockIdx.x * per, i1 = min(N, i0 + per);
  for (int j = 0; j < k; ++j) {
    double s = 0;
    const double* v = V + (size_t)j * N;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) s = fma(v[i], w[i], s);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[(size_t)j * gridDim.x + blockIdx.x] = red[0];
    __syncthreads();
  }
}

__global__ void k_multidot_finish(int k, int nb, const double* __restrict__ part,
                                  double* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  double s = 0;
  for (int b = 0; b < nb; ++b) s += part[(size_t)j * nb + b];
  out[j] = s;
}

cudaError_t launch_multidot(int N, int k, const double* V, const double* w, double* part,
                            double* out, cudaStream_t s) {
  k_multidot<<<kRedBlocks, 256, 0, s>>>(N, k, V, w, part);
  k_multidot_finish<<<(k + 127) / 128, 128, 0, s>>>(k, kRedBlocks, part, out);
  return cudaGetLastError();
}

__global__ void k_axpy_basis(int N, int k, const double* __restrict__ V, const double* __restrict__ h,
                             double* __restrict__ w, double sign) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double s = 0;
  for (int j = 0; j < k; ++j) s = fma(h[j], V[(size_t)j * N + i], s);
  w[i] = fma(sign, s, w[i]);
}

cudaError_t launch_axpy_basis(int N, int k, const double* V, const double* h, double* w,
                              double sign, cudaStream_t s) {
  k_axpy_basis<<<(N + 255) / 256, 256, 0, s>>>(N, k, V, h, w, sign);
  return cudaGetLastError();
}

__global__ void k_scale(int N, const double* __restrict__ x, double a, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) y[i] = a * x[i];
}
cudaError_t launch_scale(int N, const double* x, double a, double* y, cudaStream_t s) {
  k_scale<<<(N + 255) / 256, 256, 0, s>>>(N, x, a, y);
  return cudaGetLastError();
}

__global__ void k_axpby(int N, double a, const double* __restrict__ x, double b,
                        double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) y[i] = fma(a, x[i], b * y[i]);
}
cudaError_t launch_axpby(int N, double a, const double* x, double b, double* y, cudaStream_t s) {
  k_axpby<<<(N + 255) / 256, 256, 0, s>>>(N, a, x, b, y);
  return cudaGetLastError();
}

__global__ void k_nrm2_part(int N, const double* __restrict__ x, double* __restrict__ part) {
  __shared__ double red[256];
  double s = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    s = fma(x[i], x[i], s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
__global__ void k_nrm2_finish(int nb, const double* __restrict__ part, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0;
    for (int b = 0; b < nb; ++b) s += part[b];
    out[0] = sqrt(s);
  }
}
cudaError_t launch_nrm2(int N, const double* x, double* part, double* out, cudaStream_t s) {
  k_nrm2_part<<<kRedBlocks, 256, 0, s>>>(N, x, part);
  k_nrm2_finish<<<1, 32, 0, s>>>(kRedBlocks, part, out);
  return cudaGetLastError();
}

__global__ void k_gather(int N, const int* __restrict__ idx, const double* __restrict__ x,
                         double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) y[i] = x[idx[i]];
}
cudaError_t launch_gather(int N, const int* idx, const double* x, double* y, cudaStream_t s) {
  k_gather<<<(N + 255) / 256, 256, 0, s>>>(N, idx, x, y);
  return cudaGetLastError();
}
__global__ void k_scatter(int N, const int* __restrict__ idx, const double* __restrict__ x,
                          double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) y[idx[i]] = x[i];
}
cudaError_t launch_scatter(int N, const int* idx, const double* x, double* y, cudaStream_t s) {
  k_scatter<<<(N + 255) / 256, 256, 0, s>>>(N, idx, x, y);
  return cudaGetLastError();
}

// Caller-order rows of an internal-order matrix: out[r][q] = A[ip[r0+r]][ip[q]],
// or from the selected pairs: sel_j ? -P1 : P0.
__global__ void k_gather_rows(int N, int r0, const int* __restrict__ ip, const double* __restrict__ A,
                              const float2* __restrict__ P0, const float2* __restrict__ P1,
                              const uint8_t* __restrict__ sel, double* __restrict__ out) {
  const int r = blockIdx.y;
  const size_t src = (size_t)ip[r0 + r] * N;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x) {
    const int j = ip[q];
    double v;
    if (A) {
      v = A[src + j];
    } else if (sel[j]) {
      const float2 t = P1[src + j];
      v = -((double)t.x + (double)t.y);
    } else {
      const float2 t = P0[src + j];
      v = (double)t.x + (double)t.y;
    }
    out[(size_t)r * N + q] = v;
  }
}
cudaError_t launch_gather_rows(int N, int r0, int nr, const int* ip, const double* A,
                               const float2* P0, const float2* P1, const uint8_t* sel, double* out,
                               cudaStream_t s) {
  dim3 g(std::min(64, (N + 255) / 256), nr);
  k_gather_rows<<<g, 256, 0, s>>>(N, r0, ip, A, P0, P1, sel, out);
  return cudaGetLastError();
}

// After a boundary-condition change of the columns flips[0..nflip): the
// selected pairs swap roles, A2' = sel' ? -D : N = -B2 and B2' = -A2.
__global__ void k_reselect_pairs(int N, int nflip, const int* __restrict__ flips,
                                 float2* __restrict__ A2, float2* __restrict__ B2) {
  for (int i = blockIdx.y; i < N; i += gridDim.y)
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nflip; k += gridDim.x * blockDim.x) {
      const size_t o = (size_t)i * N + flips[k];
      const float2 a = A2[o], b = B2[o];
      A2[o] = make_float2(-b.x, -b.y);
      B2[o] = make_float2(-a.x, -a.y);
    }
}
cudaError_t launch_reselect_pairs(int N, int nflip, const int* flips, float2* A2, float2* B2,
                                  cudaStream_t s) {
  if (nflip == 0) return cudaSuccess;
  dim3 g(std::min(64, (nflip + 255) / 256), std::min(N, 65535));
  k_reselect_pairs<<<g, 256, 0, s>>>(N, nflip, flips, A2, B2);
  return cudaGetLastError();
}

}  // namespace wbem
