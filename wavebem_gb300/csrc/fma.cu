// Fast multipole alternative of the dense collocation operators: the role of
// the reference's BEMFMA (source/bem_fma.cc:56-1196, the mat-vec at :886-1097,
// selected by "Solution method = FMA" in source/bem_problem.cc:87, :646-664,
// :700-712, :974-987). An O(N) mat-vec
//     y = N a + D b      (N = dG/dn, D = G of the collocation system)
// for meshes too large for dense N x N storage, with
//   - an octree over the collocation points and the panel centres; panels
//     are attached to the leaf of their centre;
//   - a near field: every (row, panel) pair whose leaves are adjacent,
//     integrated as in the dense assembly (vertex-singular rule for panels
//     that hold a double-node partner of the row, FP64 Gauss rule within two
//     panel diameters, FP32 evaluation of FP64 offsets beyond) and stored per
//     row as 4 N and 4 D values per panel;
//   - the far field through Chebyshev-interpolation expansions of order n
//     per direction (n^3 coefficients per box; the kernel-independent form of
//     the multipole / local expansions): P2M at the leaves (charges
//     JxW phi_j b_j and dipoles n JxW phi_j a_j of the quadrature points),
//     M2M up the tree, M2L over the interaction lists (kernel 1/r evaluated
//     between Chebyshev nodes), L2L down the tree and L2P at the collocation
//     points. Boxes are interpolated over their cube enlarged by kFmaExpand,
//     so that a panel attached by its centre lies inside its leaf's box.
// The reference expands in spherical harmonics (its truncation order 3 by
// default); this form trades that for dense n^3 x n^3 translations, which
// map onto the GPU as plain loops. The preconditioner of the GMRES solve is
// block-Jacobi on the near field (the reference: UMFPACK on its near-field
// matrix, source/bem_fma.cc:1099-1196).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>
#include "context.h"
#include "host_util.h"
#include "kernels.h"

namespace wbem {

constexpr double kFmaExpand = 1.25;  // interpolation cube / box edge
constexpr int kFmaMaxOrder = 8;      // Chebyshev points per direction
constexpr int kFmaMinLevel = 2;      // the first level with interaction lists
constexpr double kInv4PiF = 0.07957747154594766788;

struct FmaConst {
  int n, n3, nq;
  float inv_n;                            // 1 / n
  float t[kFmaMaxOrder];                  // Chebyshev nodes on [-1, 1]
  float Tt[kFmaMaxOrder][kFmaMaxOrder];   // T_j(t_k) for j, k < n, zero elsewhere
  float phi[kMaxQ1 * kMaxQ1][4];          // shape values at the regular points
};
// Passed by value to every kernel of the FMA (a __grid_constant__ parameter,
// read through the constant bank), so that handles share no device state.

// ------------------------------------------------------------ device helpers
// Interpolation weights S_n(u, t_k) = 1/n + 2/n sum_{j=1}^{n-1} T_j(u) T_j(t_k)
// and their derivatives in u, k = 0..n-1. Every loop runs over the fixed
// kFmaMaxOrder with the table T_j(t_k) zero for j >= n, so that the arrays
// stay in registers (entries k >= n are left meaningless).
__device__ __forceinline__ void cheb_weights(const FmaConst& c_fma, float u, float* S,
                                             float* dS) {
  float T[kFmaMaxOrder], dT[kFmaMaxOrder];
  T[0] = 1.f;
  dT[0] = 0.f;
  T[1] = u;
  dT[1] = 1.f;
#pragma unroll
  for (int j = 2; j < kFmaMaxOrder; ++j) {
    T[j] = 2.f * u * T[j - 1] - T[j - 2];
    dT[j] = 2.f * T[j - 1] + 2.f * u * dT[j - 1] - dT[j - 2];
  }
  const float inv = c_fma.inv_n, inv2 = 2.f * c_fma.inv_n;
#pragma unroll
  for (int k = 0; k < kFmaMaxOrder; ++k) {
    float s = inv, ds = 0.f;
#pragma unroll
    for (int j = 1; j < kFmaMaxOrder; ++j) {
      const float tt = c_fma.Tt[j][k];
      s = fmaf(inv2 * T[j], tt, s);
      ds = fmaf(inv2 * dT[j], tt, ds);
    }
    S[k] = s;
    if (dS) dS[k] = ds;
  }
}

__device__ __forceinline__ bool fma_in_set(const int* set, int v) {
  bool r = false;
#pragma unroll
  for (int k = 0; k < kMaxSet; ++k) r |= (set[k] == v);
  return r;
}

// ------------------------------------------------------------ near field
// One thread per (row, near panel) pair: 4 N and 4 D entries (the dense
// assembly's contributions of that panel to the row), stored as
// val[8 * pair + 0..3] = N, [4..7] = D.
__global__ void k_fma_near(int npairs, const int* __restrict__ pair_row,
                           const int* __restrict__ pair_pan, const double* __restrict__ X,
                           const int* __restrict__ dnset, const int4* __restrict__ cell_dofs,
                           const double* __restrict__ rec, double* __restrict__ val,
                           const QuadTables* __restrict__ qt) {
  const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npairs) return;
  const int row = pair_row[k], cell = pair_pan[k];
  const double xi = X[3 * (size_t)row], yi = X[3 * (size_t)row + 1], zi = X[3 * (size_t)row + 2];
  int set[kMaxSet];
#pragma unroll
  for (int s = 0; s < kMaxSet; ++s) set[s] = dnset[(size_t)row * kMaxSet + s];
  const int4 d = cell_dofs[cell];
  const int id[4] = {d.x, d.y, d.z, d.w};
  double ln[4] = {0, 0, 0, 0}, ld[4] = {0, 0, 0, 0};
  int v = -1;
  for (int j = 0; j < 4 && v < 0; ++j)
    if (fma_in_set(set, id[j])) v = j;
  double P[4][3];
  for (int j = 0; j < 4; ++j)
    for (int e = 0; e < 3; ++e) P[j][e] = X[3 * (size_t)id[j] + e];
  if (v >= 0) {
    // vertex-singular rule at local vertex v (source/bem_problem.cc:478-522)
    for (int q = 0; q < qt->nsp; ++q) {
      const double s = qt->sp[v][q][0], t = qt->sp[v][q][1], w = qt->sp[v][q][2] * kInv4PiF;
      const double a0 = (1 - s) * (1 - t), a1 = s * (1 - t), a2 = (1 - s) * t, a3 = s * t;
      double x[3], jx[3], je[3];
      for (int e = 0; e < 3; ++e) {
        x[e] = a0 * P[0][e] + a1 * P[1][e] + a2 * P[2][e] + a3 * P[3][e];
        jx[e] = (1 - t) * (P[1][e] - P[0][e]) + t * (P[3][e] - P[2][e]);
        je[e] = (1 - s) * (P[2][e] - P[0][e]) + s * (P[3][e] - P[1][e]);
      }
      const double cr[3] = {jx[1] * je[2] - jx[2] * je[1], jx[2] * je[0] - jx[0] * je[2],
                            jx[0] * je[1] - jx[1] * je[0]};
      const double det = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      const double Rx = x[0] - xi, Ry = x[1] - yi, Rz = x[2] - zi;
      const double ri = rsqrt(fma(Rx, Rx, fma(Ry, Ry, Rz * Rz)));
      const double sq = ri * det * w;
      const double dq = -(Rx * cr[0] + Ry * cr[1] + Rz * cr[2]) * (ri * ri * ri) * w;
      const double ph[4] = {a0, a1, a2, a3};
      for (int j = 0; j < 4; ++j) {
        ln[j] = fma(dq, ph[j], ln[j]);
        ld[j] = fma(sq, ph[j], ld[j]);
      }
    }
  } else {
    // FP64 within two panel diameters of the centre, FP32 beyond
    double c[3], dia = 0;
    for (int e = 0; e < 3; ++e) c[e] = 0.25 * (P[0][e] + P[1][e] + P[2][e] + P[3][e]);
    for (int e = 0; e < 3; ++e) {
      dia = fmax(dia, fabs(P[3][e] - P[0][e]));
      dia = fmax(dia, fabs(P[2][e] - P[1][e]));
    }
    const double dx = c[0] - xi, dy = c[1] - yi, dz = c[2] - zi;
    const bool close = dx * dx + dy * dy + dz * dz < 4.0 * 3.0 * dia * dia;
    const int nq = qt->q1 * qt->q1;
    const double* r = rec + (size_t)cell * nq * 8;
    if (close) {
      for (int q = 0; q < nq; ++q) {
        const double Rx = r[8 * q] - xi, Ry = r[8 * q + 1] - yi, Rz = r[8 * q + 2] - zi;
        const double ri = rsqrt(fma(Rx, Rx, fma(Ry, Ry, Rz * Rz)));
        const double sq = ri * r[8 * q + 3];
        const double dq = -fma(Rx, r[8 * q + 4], fma(Ry, r[8 * q + 5], Rz * r[8 * q + 6])) * (ri * ri * ri);
        for (int j = 0; j < 4; ++j) {
          ln[j] = fma(dq, qt->phi[q][j], ln[j]);
          ld[j] = fma(sq, qt->phi[q][j], ld[j]);
        }
      }
    } else {
      float lnf[4] = {0, 0, 0, 0}, ldf[4] = {0, 0, 0, 0};
      for (int q = 0; q < nq; ++q) {
        const float Rx = (float)(r[8 * q] - xi), Ry = (float)(r[8 * q + 1] - yi),
                    Rz = (float)(r[8 * q + 2] - zi);
        const float ri = rsqrtf(fmaf(Rx, Rx, fmaf(Ry, Ry, Rz * Rz)));
        const float sq = ri * (float)r[8 * q + 3];
        const float dq = -fmaf(Rx, (float)r[8 * q + 4], fmaf(Ry, (float)r[8 * q + 5], Rz * (float)r[8 * q + 6])) *
                         (ri * ri * ri);
        for (int j = 0; j < 4; ++j) {
          lnf[j] = fmaf(dq, qt->phif[q][j], lnf[j]);
          ldf[j] = fmaf(sq, qt->phif[q][j], ldf[j]);
        }
      }
      for (int j = 0; j < 4; ++j) {
        ln[j] = lnf[j];
        ld[j] = ldf[j];
      }
    }
  }
  double* o = val + 8 * (size_t)k;
  for (int j = 0; j < 4; ++j) {
    o[j] = ln[j];
    o[4 + j] = ld[j];
  }
}

// The near-field entries of the diagonal 128-blocks of the system operator
// (sel_j ? -D_ij : N_ij, plus alpha on Neumann diagonals): one thread per row
// writes its own block row (blocks zeroed before).
__global__ void k_fma_near_blocks(int N, const int* __restrict__ near_ptr,
                                  const int* __restrict__ pair_pan, const double* __restrict__ val,
                                  const int4* __restrict__ cell_dofs, const uint8_t* __restrict__ mask,
                                  const double* __restrict__ alpha, double* __restrict__ blocks) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int b = i / kBJ, r = i % kBJ;
  double* row = blocks + ((size_t)b * kBJ + r) * kBJ;
  for (int k = near_ptr[i]; k < near_ptr[i + 1]; ++k) {
    const int4 d = cell_dofs[pair_pan[k]];
    const int id[4] = {d.x, d.y, d.z, d.w};
    for (int j = 0; j < 4; ++j) {
      const int c = id[j];
      if (c / kBJ != b) continue;
      row[c % kBJ] += mask[c] ? -val[8 * (size_t)k + 4 + j] : val[8 * (size_t)k + j];
    }
  }
  if (!mask[i]) row[r] += alpha[i];
}

// ------------------------------------------------------------ far field
// P2M: one CTA per leaf, thread m < n^3 holds coefficient m = (i, j, k) of
// the leaf's expansion; the points are staged in chunks (strengths and the
// 1-D interpolation weights per direction).
constexpr int kP2MChunk = 64;
__global__ void k_fma_p2m(const int* __restrict__ leaf_pptr, const int* __restrict__ leaf_pan,
                          const double* __restrict__ rec, const int4* __restrict__ cell_dofs,
                          const double* __restrict__ a, const double* __restrict__ b,
                          const double* __restrict__ cen, double half, float* __restrict__ W,
                          const __grid_constant__ FmaConst c_fma) {
  const int leaf = blockIdx.x;
  const int n = c_fma.n, n3 = c_fma.n3, nq = c_fma.nq;
  __shared__ float sg[kP2MChunk], mu[kP2MChunk][3];
  __shared__ float Sw[kP2MChunk][3][kFmaMaxOrder], dSw[kP2MChunk][3][kFmaMaxOrder];
  const int tid = threadIdx.x;
  const int p0 = leaf_pptr[leaf], p1 = leaf_pptr[leaf + 1];
  const int npts = (p1 - p0) * nq;
  const double cx = cen[3 * leaf], cy = cen[3 * leaf + 1], cz = cen[3 * leaf + 2];
  const int mi = tid / (n * n), mj = (tid / n) % n, mk = tid % n;
  float acc = 0.f;
  for (int base = 0; base < npts; base += kP2MChunk) {
    if (tid < kP2MChunk) {
      const int f = base + tid;
      if (f < npts) {
        const int cell = leaf_pan[p0 + f / nq], q = f % nq;
        const double* r = rec + ((size_t)cell * nq + q) * 8;
        const int4 d = cell_dofs[cell];
        const int id[4] = {d.x, d.y, d.z, d.w};
        double sb = 0, sa = 0;
        for (int j = 0; j < 4; ++j) {
          sb += c_fma.phi[q][j] * b[id[j]];
          sa += c_fma.phi[q][j] * a[id[j]];
        }
        sg[tid] = (float)(r[3] * sb);
        mu[tid][0] = (float)(r[4] * sa);
        mu[tid][1] = (float)(r[5] * sa);
        mu[tid][2] = (float)(r[6] * sa);
        cheb_weights(c_fma, (float)((r[0] - cx) / half), Sw[tid][0], dSw[tid][0]);
        cheb_weights(c_fma, (float)((r[1] - cy) / half), Sw[tid][1], dSw[tid][1]);
        cheb_weights(c_fma, (float)((r[2] - cz) / half), Sw[tid][2], dSw[tid][2]);
      } else {
        sg[tid] = 0.f;
        mu[tid][0] = mu[tid][1] = mu[tid][2] = 0.f;
        for (int k = 0; k < kFmaMaxOrder; ++k)
          Sw[tid][0][k] = Sw[tid][1][k] = Sw[tid][2][k] = dSw[tid][0][k] = dSw[tid][1][k] = dSw[tid][2][k] = 0.f;
      }
    }
    __syncthreads();
    if (tid < n3) {
      const int cnt = min(kP2MChunk, npts - base);
      const float ih = (float)(1.0 / half);
      for (int p = 0; p < cnt; ++p) {
        const float sx = Sw[p][0][mi], sy = Sw[p][1][mj], sz = Sw[p][2][mk];
        const float g = mu[p][0] * dSw[p][0][mi] * sy * sz + mu[p][1] * sx * dSw[p][1][mj] * sz +
                        mu[p][2] * sx * sy * dSw[p][2][mk];
        acc = fmaf(sg[p], sx * sy * sz, fmaf(g, ih, acc));
      }
    }
    __syncthreads();
  }
  if (tid < n3) W[(size_t)leaf * n3 + tid] = acc;
}

// M2M: one CTA per parent box; W_P[M] = sum_children sum_m T[oct][m][M] W_c[m]
// (T: the parent's interpolation weights at the child's nodes).
__global__ void k_fma_m2m(const int* __restrict__ child_ptr, const int* __restrict__ child,
                          const int* __restrict__ child_oct, const float* __restrict__ T,
                          const float* __restrict__ Wc, float* __restrict__ Wp,
                          const __grid_constant__ FmaConst c_fma) {
  const int p = blockIdx.x, M = threadIdx.x, n3 = c_fma.n3;
  __shared__ float w[kFmaMaxOrder * kFmaMaxOrder * kFmaMaxOrder];
  float acc = 0.f;
  for (int e = child_ptr[p]; e < child_ptr[p + 1]; ++e) {
    __syncthreads();
    if (M < n3) w[M] = Wc[(size_t)child[e] * n3 + M];
    __syncthreads();
    if (M < n3) {
      const float* To = T + (size_t)child_oct[e] * n3 * n3;
      for (int m = 0; m < n3; ++m) acc = fmaf(To[(size_t)m * n3 + M], w[m], acc);
    }
  }
  if (M < n3) Wp[(size_t)p * n3 + M] = acc;
}

// M2L: one CTA per target box of a level; L_T[a] = sum_{B in the
// interaction list} sum_m W_B[m] / |x_a - y_m| (node offsets relative to the
// box centres, the centre difference in FP64).
__global__ void k_fma_m2l(const int* __restrict__ il_ptr, const int* __restrict__ il,
                          const double* __restrict__ cen, double half, const float* __restrict__ W,
                          float* __restrict__ Lx, const __grid_constant__ FmaConst c_fma) {
  const int t = blockIdx.x, a = threadIdx.x;
  const int n = c_fma.n, n3 = c_fma.n3;
  __shared__ float w[kFmaMaxOrder * kFmaMaxOrder * kFmaMaxOrder];
  __shared__ float off[kFmaMaxOrder * kFmaMaxOrder * kFmaMaxOrder][3];
  const float h = (float)half;
  if (a < n3) {
    off[a][0] = h * c_fma.t[a / (n * n)];
    off[a][1] = h * c_fma.t[(a / n) % n];
    off[a][2] = h * c_fma.t[a % n];
  }
  const double tx = cen[3 * t], ty = cen[3 * t + 1], tz = cen[3 * t + 2];
  float acc = 0.f;
  for (int e = il_ptr[t]; e < il_ptr[t + 1]; ++e) {
    const int s = il[e];
    __syncthreads();
    if (a < n3) w[a] = W[(size_t)s * n3 + a];
    __syncthreads();
    if (a < n3) {
      const float dx = (float)(tx - cen[3 * s]) + off[a][0];
      const float dy = (float)(ty - cen[3 * s + 1]) + off[a][1];
      const float dz = (float)(tz - cen[3 * s + 2]) + off[a][2];
      for (int m = 0; m < n3; ++m) {
        const float rx = dx - off[m][0], ry = dy - off[m][1], rz = dz - off[m][2];
        acc = fmaf(w[m], rsqrtf(fmaf(rx, rx, fmaf(ry, ry, rz * rz))), acc);
      }
    }
  }
  if (a < n3) Lx[(size_t)t * n3 + a] = acc;
}

// L2L: one CTA per child box; L_c[a] += sum_A T[oct][a][A] L_P[A].
__global__ void k_fma_l2l(const int* __restrict__ parent, const int* __restrict__ oct,
                          const float* __restrict__ T, const float* __restrict__ Lp,
                          float* __restrict__ Lc, const __grid_constant__ FmaConst c_fma) {
  const int c = blockIdx.x, a = threadIdx.x, n3 = c_fma.n3;
  __shared__ float l[kFmaMaxOrder * kFmaMaxOrder * kFmaMaxOrder];
  const int p = parent[c];
  if (a < n3) l[a] = Lp[(size_t)p * n3 + a];
  __syncthreads();
  if (a < n3) {
    const float* To = T + (size_t)oct[c] * n3 * n3 + (size_t)a * n3;
    float acc = Lc[(size_t)c * n3 + a];
    for (int A = 0; A < n3; ++A) acc = fmaf(To[A], l[A], acc);
    Lc[(size_t)c * n3 + a] = acc;
  }
}

// L2P and the near field, one thread per collocation point:
// y_i = sum_a S_a(x_i) L_leaf[a] + sum_{near pairs} (N a + D b) (the record
// weights carry the 1 / (4 pi)).
__global__ void k_fma_eval(int N, const double* __restrict__ X, const int* __restrict__ tgt_leaf,
                           const double* __restrict__ cen, double half, const float* __restrict__ Lx,
                           const int* __restrict__ near_ptr, const int* __restrict__ pair_pan,
                           const double* __restrict__ val, const int4* __restrict__ cell_dofs,
                           const double* __restrict__ a, const double* __restrict__ b,
                           double* __restrict__ y, const __grid_constant__ FmaConst c_fma) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int n = c_fma.n, n3 = c_fma.n3;
  const int lf = tgt_leaf[i];
  double far = 0.0;
  if (Lx) {
    float Sx[kFmaMaxOrder], Sy[kFmaMaxOrder], Sz[kFmaMaxOrder];
    cheb_weights(c_fma, (float)((X[3 * (size_t)i] - cen[3 * lf]) / half), Sx, nullptr);
    cheb_weights(c_fma, (float)((X[3 * (size_t)i + 1] - cen[3 * lf + 1]) / half), Sy, nullptr);
    cheb_weights(c_fma, (float)((X[3 * (size_t)i + 2] - cen[3 * lf + 2]) / half), Sz, nullptr);
    const float* L = Lx + (size_t)lf * n3;
    float s = 0.f;
    for (int u = 0; u < n; ++u)
      for (int v = 0; v < n; ++v) {
        const float sxy = Sx[u] * Sy[v];
        for (int w = 0; w < n; ++w) s = fmaf(sxy * Sz[w], L[(u * n + v) * n + w], s);
      }
    far = (double)s;
  }
  double nearv = 0.0;
  for (int k = near_ptr[i]; k < near_ptr[i + 1]; ++k) {
    const int4 d = cell_dofs[pair_pan[k]];
    const double* v = val + 8 * (size_t)k;
    nearv += v[0] * a[d.x] + v[1] * a[d.y] + v[2] * a[d.z] + v[3] * a[d.w] + v[4] * b[d.x] +
             v[5] * b[d.y] + v[6] * b[d.z] + v[7] * b[d.w];
  }
  y[i] = far + nearv;
}

// Inputs of one FMA product: mode 0 (vmult): a = x o, b = -x s;
// mode 1 (compute_rhs): a = -x s, b = x o; mode 2 (alpha): a = 1, b = 0.
__global__ void k_fma_inputs(int N, int mode, const uint8_t* __restrict__ mask,
                             const double* __restrict__ x, double* __restrict__ a,
                             double* __restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (mode == 2) {
    a[i] = 1.0;
    b[i] = 0.0;
    return;
  }
  const bool s = mask[i] != 0;
  const double v = x[i];
  if (mode == 0) {
    a[i] = s ? 0.0 : v;
    b[i] = s ? -v : 0.0;
  } else {
    a[i] = s ? -v : 0.0;
    b[i] = s ? 0.0 : v;
  }
}

// The free term of the product: mode 0: y += (1 - s) alpha x; mode 1:
// y -= s alpha x; mode 2: alpha = -y.
__global__ void k_fma_finish(int N, int mode, const uint8_t* __restrict__ mask,
                             const double* __restrict__ alpha, const double* __restrict__ x,
                             double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (mode == 2) {
    y[i] = -y[i];
    return;
  }
  const bool s = mask[i] != 0;
  if (mode == 0 && !s) y[i] += alpha[i] * x[i];
  if (mode == 1 && s) y[i] -= alpha[i] * x[i];
}

// ------------------------------------------------------------ host: tree
namespace {

struct Key3 {
  int x, y, z;
  bool operator==(const Key3& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct Key3Hash {
  size_t operator()(const Key3& k) const {
    return ((size_t)(unsigned)k.x * 73856093u) ^ ((size_t)(unsigned)k.y * 19349663u) ^
           ((size_t)(unsigned)k.z * 83492791u);
  }
};

// 1-D interpolation weights on the host (double).
void cheb_weights_host(int n, double u, const std::vector<double>& t, double* S) {
  std::vector<double> T(n), Tt(n);
  T[0] = 1;
  if (n > 1) T[1] = u;
  for (int j = 2; j < n; ++j) T[j] = 2 * u * T[j - 1] - T[j - 2];
  for (int k = 0; k < n; ++k) {
    double s = 1.0 / n;
    double tk0 = 1, tk1 = t[k];
    for (int j = 1; j < n; ++j) {
      const double tj = (j == 1) ? tk1 : 2 * t[k] * tk1 - tk0;
      if (j >= 2) {
        tk0 = tk1;
        tk1 = tj;
      }
      s += 2.0 / n * T[j] * tj;
    }
    S[k] = s;
  }
}

}  // namespace

struct FmaLevel {
  int nbox = 0;
  double half = 0;               // half-width of the interpolation cube
  double* d_cen = nullptr;       // nbox x 3
  int* d_il_ptr = nullptr;       // interaction lists (same level)
  int* d_il = nullptr;
  int* d_child_ptr = nullptr;    // children at the next level, CSR
  int* d_child = nullptr;
  int* d_child_oct = nullptr;
  int* d_parent = nullptr;       // parent at the previous level
  int* d_oct = nullptr;          // octant in the parent
  float* d_W = nullptr;          // nbox x n^3
  float* d_L = nullptr;
  std::vector<int> parent, oct, il_ptr;  // host copies (scheduling)
};

struct FmaState {
  int L = 0, n = 0;
  std::vector<FmaLevel> lev;
  int nleaf = 0;
  int* d_leaf_pptr = nullptr;
  int* d_leaf_pan = nullptr;
  int* d_tgt_leaf = nullptr;
  int* d_near_ptr = nullptr;
  int* d_pair_row = nullptr;
  int* d_pair_pan = nullptr;
  double* d_near_val = nullptr;
  size_t npairs = 0;
  float* d_T = nullptr;          // 8 x n^3 x n^3: T[oct][child node m][parent node M]
  double* d_blocks = nullptr;    // near-field diagonal blocks of the system
  double* d_a = nullptr;         // product inputs (N each)
  double* d_b = nullptr;
  QuadTables* d_qt = nullptr;
  FmaConst cst{};                // expansion constants, a parameter of every kernel
  std::vector<void*> owned;
};

static void fma_free(FmaState* F) {
  if (!F) return;
  for (void* p : F->owned)
    if (p) cudaFree(p);
  delete F;
}

void free_fma(wbem_context* h) {
  fma_free(static_cast<FmaState*>(h->fma_state));
  h->fma_state = nullptr;
}

template <typename T>
static int fma_upload(wbem_context* h, FmaState* F, T** p, const std::vector<T>& v) {
  *p = nullptr;
  WB_CHK(upload(h, p, v));
  F->owned.push_back(*p);
  return WBEM_OK;
}

template <typename T>
static int fma_alloc(wbem_context* h, FmaState* F, T** p, size_t n) {
  *p = nullptr;
  WB_CHK(dev_alloc(h, p, n));
  F->owned.push_back(*p);
  return WBEM_OK;
}

// Octree, lists and near-field pair structure for the handle's mesh.
static int fma_build(wbem_context* h, FmaState* F, const QuadTables& qt) {
  const int N = h->N, C = h->C;
  // positions in the internal order (targets) and panel centres / radii
  std::vector<double> Xi(3 * (size_t)N);
  for (int i = 0; i < N; ++i)
    for (int d = 0; d < 3; ++d) Xi[3 * (size_t)i + d] = h->X[3 * (size_t)h->perm[i] + d];
  std::vector<double> pc(3 * (size_t)C);
  double rho = 0;
  for (int c = 0; c < C; ++c) {
    const int* cc = &h->cells[4 * (size_t)c];
    for (int d = 0; d < 3; ++d)
      pc[3 * (size_t)c + d] = 0.25 * (h->X[3 * (size_t)cc[0] + d] + h->X[3 * (size_t)cc[1] + d] +
                                      h->X[3 * (size_t)cc[2] + d] + h->X[3 * (size_t)cc[3] + d]);
    for (int k = 0; k < 4; ++k) {
      double r2 = 0;
      for (int d = 0; d < 3; ++d) {
        const double e = h->X[3 * (size_t)cc[k] + d] - pc[3 * (size_t)c + d];
        r2 += e * e;
      }
      rho = std::max(rho, std::sqrt(r2));
    }
  }
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < N; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], Xi[3 * (size_t)i + d]);
      hi[d] = std::max(hi[d], Xi[3 * (size_t)i + d]);
    }
  for (int c = 0; c < C; ++c)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], pc[3 * (size_t)c + d]);
      hi[d] = std::max(hi[d], pc[3 * (size_t)c + d]);
    }
  double S = 0;
  for (int d = 0; d < 3; ++d) S = std::max(S, hi[d] - lo[d]);
  S = S * (1 + 1e-9) + 1e-12;
  // leaf level: the deepest level whose interpolation margin covers every
  // panel ((expand - 1) s / 2 >= panel radius) and whose leaves hold about
  // 16 or more collocation points on average
  int L = kFmaMinLevel;
  for (int l = kFmaMinLevel; l <= 20; ++l) {
    const double s = S / (double)(1 << l);
    if ((kFmaExpand - 1.0) * s / 2.0 < rho) break;
    std::unordered_map<Key3, int, Key3Hash> cnt;
    for (int i = 0; i < N; ++i)
      cnt[{(int)std::floor((Xi[3 * (size_t)i] - lo[0]) / s), (int)std::floor((Xi[3 * (size_t)i + 1] - lo[1]) / s),
           (int)std::floor((Xi[3 * (size_t)i + 2] - lo[2]) / s)}]++;
    if ((double)N / cnt.size() < 16.0 && l > kFmaMinLevel) break;
    L = l;
  }
  if ((kFmaExpand - 1.0) * (S / (double)(1 << L)) / 2.0 < rho)
    return fail(h, WBEM_ERR_ARG, "FMA: panels too large for an octree of at least two levels");
  F->L = L;
  const double sL = S / (double)(1 << L);
  auto keyL = [&](const double* p) {
    Key3 k{(int)std::floor((p[0] - lo[0]) / sL), (int)std::floor((p[1] - lo[1]) / sL),
           (int)std::floor((p[2] - lo[2]) / sL)};
    const int mx = (1 << L) - 1;
    k.x = std::min(std::max(k.x, 0), mx);
    k.y = std::min(std::max(k.y, 0), mx);
    k.z = std::min(std::max(k.z, 0), mx);
    return k;
  };
  // boxes per level (sorted keys), leaf = level L
  std::vector<std::vector<Key3>> keys(L + 1);
  std::vector<std::unordered_map<Key3, int, Key3Hash>> index(L + 1);
  std::vector<Key3> tk(N), pk(C);
  for (int i = 0; i < N; ++i) tk[i] = keyL(&Xi[3 * (size_t)i]);
  for (int c = 0; c < C; ++c) pk[c] = keyL(&pc[3 * (size_t)c]);
  {
    std::vector<Key3> all(tk);
    all.insert(all.end(), pk.begin(), pk.end());
    auto less = [](const Key3& a, const Key3& b) {
      return a.x != b.x ? a.x < b.x : a.y != b.y ? a.y < b.y : a.z < b.z;
    };
    for (int l = L; l >= 0; --l) {
      std::vector<Key3> v;
      v.reserve(all.size());
      for (const Key3& k : all) v.push_back({k.x >> (L - l), k.y >> (L - l), k.z >> (L - l)});
      std::sort(v.begin(), v.end(), less);
      v.erase(std::unique(v.begin(), v.end()), v.end());
      keys[l] = v;
      for (int b = 0; b < (int)v.size(); ++b) index[l][v[b]] = b;
    }
  }
  auto adjacent = [](const Key3& a, const Key3& b) {
    return std::abs(a.x - b.x) <= 1 && std::abs(a.y - b.y) <= 1 && std::abs(a.z - b.z) <= 1;
  };
  F->lev.assign(L + 1, FmaLevel{});
  const int n3 = F->n * F->n * F->n;
  for (int l = 0; l <= L; ++l) {
    FmaLevel& V = F->lev[l];
    const double s = S / (double)(1 << l);
    V.nbox = (int)keys[l].size();
    V.half = kFmaExpand * s / 2;
    std::vector<double> cen(3 * (size_t)V.nbox);
    for (int b = 0; b < V.nbox; ++b) {
      cen[3 * (size_t)b] = lo[0] + (keys[l][b].x + 0.5) * s;
      cen[3 * (size_t)b + 1] = lo[1] + (keys[l][b].y + 0.5) * s;
      cen[3 * (size_t)b + 2] = lo[2] + (keys[l][b].z + 0.5) * s;
    }
    WB_CHK(fma_upload(h, F, &V.d_cen, cen));
    WB_CHK(fma_alloc(h, F, &V.d_W, (size_t)V.nbox * n3));
    WB_CHK(fma_alloc(h, F, &V.d_L, (size_t)V.nbox * n3));
    if (l > 0) {
      V.parent.resize(V.nbox);
      V.oct.resize(V.nbox);
      for (int b = 0; b < V.nbox; ++b) {
        const Key3& k = keys[l][b];
        V.parent[b] = index[l - 1].at({k.x >> 1, k.y >> 1, k.z >> 1});
        V.oct[b] = (k.x & 1) * 4 + (k.y & 1) * 2 + (k.z & 1);
      }
      WB_CHK(fma_upload(h, F, &V.d_parent, V.parent));
      WB_CHK(fma_upload(h, F, &V.d_oct, V.oct));
      // children lists of the previous level
      FmaLevel& P = F->lev[l - 1];
      std::vector<int> cptr(P.nbox + 1, 0), ch, coct;
      for (int b = 0; b < V.nbox; ++b) cptr[V.parent[b] + 1]++;
      for (int p = 0; p < P.nbox; ++p) cptr[p + 1] += cptr[p];
      ch.resize(V.nbox);
      coct.resize(V.nbox);
      std::vector<int> fill(cptr.begin(), cptr.end() - 1);
      for (int b = 0; b < V.nbox; ++b) {
        const int e = fill[V.parent[b]]++;
        ch[e] = b;
        coct[e] = V.oct[b];
      }
      WB_CHK(fma_upload(h, F, &P.d_child_ptr, cptr));
      WB_CHK(fma_upload(h, F, &P.d_child, ch));
      WB_CHK(fma_upload(h, F, &P.d_child_oct, coct));
    }
    // interaction lists: children of the parent's neighbours (the parent
    // included) that are not adjacent to the box
    V.il_ptr.assign(V.nbox + 1, 0);
    std::vector<int> il;
    if (l >= kFmaMinLevel) {
      for (int b = 0; b < V.nbox; ++b) {
        const Key3& k = keys[l][b];
        const Key3 pk2{k.x >> 1, k.y >> 1, k.z >> 1};
        for (int dx = -1; dx <= 1; ++dx)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
              const Key3 pn{pk2.x + dx, pk2.y + dy, pk2.z + dz};
              if (!index[l - 1].count(pn)) continue;
              for (int o = 0; o < 8; ++o) {
                const Key3 c2{2 * pn.x + (o >> 2), 2 * pn.y + ((o >> 1) & 1), 2 * pn.z + (o & 1)};
                auto it = index[l].find(c2);
                if (it != index[l].end() && !adjacent(c2, k)) il.push_back(it->second);
              }
            }
        V.il_ptr[b + 1] = (int)il.size();
      }
    }
    WB_CHK(fma_upload(h, F, &V.d_il_ptr, V.il_ptr));
    if (il.empty()) il.push_back(0);
    WB_CHK(fma_upload(h, F, &V.d_il, il));
  }
  // leaves: panels per leaf, leaf of each target, near pairs per target
  const FmaLevel& LV = F->lev[L];
  F->nleaf = LV.nbox;
  std::vector<int> pptr(LV.nbox + 1, 0), pan(C), tl(N);
  for (int c = 0; c < C; ++c) pptr[index[L].at(pk[c]) + 1]++;
  for (int b = 0; b < LV.nbox; ++b) pptr[b + 1] += pptr[b];
  {
    std::vector<int> fill(pptr.begin(), pptr.end() - 1);
    for (int c = 0; c < C; ++c) pan[fill[index[L].at(pk[c])]++] = c;
  }
  for (int i = 0; i < N; ++i) tl[i] = index[L].at(tk[i]);
  WB_CHK(fma_upload(h, F, &F->d_leaf_pptr, pptr));
  WB_CHK(fma_upload(h, F, &F->d_leaf_pan, pan));
  WB_CHK(fma_upload(h, F, &F->d_tgt_leaf, tl));
  std::vector<std::vector<int>> near_leaves(LV.nbox);
  for (int b = 0; b < LV.nbox; ++b) {
    const Key3& k = keys[L][b];
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          auto it = index[L].find({k.x + dx, k.y + dy, k.z + dz});
          if (it != index[L].end()) near_leaves[b].push_back(it->second);
        }
  }
  std::vector<int> nptr(N + 1, 0);
  for (int i = 0; i < N; ++i) {
    size_t cnt = 0;
    for (int nb : near_leaves[tl[i]]) cnt += pptr[nb + 1] - pptr[nb];
    nptr[i + 1] = (int)cnt;
  }
  for (int i = 0; i < N; ++i) {
    if ((long long)nptr[i] + nptr[i + 1] > 2000000000LL)
      return fail(h, WBEM_ERR_ARG, "FMA: near field too large (more than 2e9 pairs)");
    nptr[i + 1] += nptr[i];
  }
  F->npairs = (size_t)nptr[N];
  std::vector<int> prow(F->npairs), ppan(F->npairs);
  for (int i = 0; i < N; ++i) {
    size_t e = nptr[i];
    for (int nb : near_leaves[tl[i]])
      for (int k = pptr[nb]; k < pptr[nb + 1]; ++k) {
        prow[e] = i;
        ppan[e] = pan[k];
        ++e;
      }
  }
  WB_CHK(fma_upload(h, F, &F->d_near_ptr, nptr));
  WB_CHK(fma_upload(h, F, &F->d_pair_row, prow));
  WB_CHK(fma_upload(h, F, &F->d_pair_pan, ppan));
  WB_CHK(fma_alloc(h, F, &F->d_near_val, 8 * std::max<size_t>(1, F->npairs)));
  // child -> parent interpolation matrices per octant (level-independent:
  // the interpolation cubes scale with the boxes)
  const int n = F->n;
  std::vector<double> t(n);
  for (int k = 0; k < n; ++k) t[k] = std::cos((2 * k + 1) * 3.14159265358979323846 / (2.0 * n));
  std::vector<float> T((size_t)8 * n3 * n3);
  std::vector<double> Sx(n), Sy(n), Sz(n);
  for (int o = 0; o < 8; ++o) {
    const int ox = o >> 2, oy = (o >> 1) & 1, oz = o & 1;
    for (int m = 0; m < n3; ++m) {
      const int mi = m / (n * n), mj = (m / n) % n, mk = m % n;
      // child node in parent cube coordinates: +-1/(2 e) + t / 2
      const double ux = (ox ? 1.0 : -1.0) / (2 * kFmaExpand) + t[mi] / 2;
      const double uy = (oy ? 1.0 : -1.0) / (2 * kFmaExpand) + t[mj] / 2;
      const double uz = (oz ? 1.0 : -1.0) / (2 * kFmaExpand) + t[mk] / 2;
      cheb_weights_host(n, ux, t, Sx.data());
      cheb_weights_host(n, uy, t, Sy.data());
      cheb_weights_host(n, uz, t, Sz.data());
      for (int M = 0; M < n3; ++M)
        T[((size_t)o * n3 + m) * n3 + M] =
            (float)(Sx[M / (n * n)] * Sy[(M / n) % n] * Sz[M % n]);
    }
  }
  WB_CHK(fma_upload(h, F, &F->d_T, T));
  const int nb = (N + kBJ - 1) / kBJ;
  WB_CHK(fma_alloc(h, F, &F->d_blocks, (size_t)nb * kBJ * kBJ));
  WB_CHK(fma_alloc(h, F, &F->d_a, (size_t)N));
  WB_CHK(fma_alloc(h, F, &F->d_b, (size_t)N));
  std::vector<QuadTables> qv(1, qt);
  WB_CHK(fma_upload(h, F, &F->d_qt, qv));
  // constants
  FmaConst& fc = F->cst;
  fc = FmaConst{};
  fc.n = n;
  fc.inv_n = 1.f / (float)n;
  fc.n3 = n3;
  fc.nq = qt.q1 * qt.q1;
  for (int k = 0; k < n; ++k) {
    fc.t[k] = (float)t[k];
    double T0 = 1, T1 = t[k];
    for (int j = 0; j < kFmaMaxOrder; ++j) {
      const double v = j == 0 ? 1.0 : (j == 1 ? t[k] : 2 * t[k] * T1 - T0);
      if (j >= 2) {
        T0 = T1;
        T1 = v;
      }
      fc.Tt[j][k] = j < n ? (float)v : 0.f;
    }
  }
  for (int q = 0; q < qt.q1 * qt.q1; ++q)
    for (int j = 0; j < 4; ++j) fc.phi[q][j] = (float)qt.phi[q][j];
  return WBEM_OK;
}

// y = N a + D b with the FMA (a, b, y device vectors, internal order).
static int fma_product(wbem_context* h, const double* a, const double* b, double* y) {
  FmaState* F = static_cast<FmaState*>(h->fma_state);
  const int N = h->N, L = F->L, n3 = F->n * F->n * F->n;
  const int nt = (n3 + 31) / 32 * 32;
  cudaStream_t s = h->stream;
  FmaLevel& LV = F->lev[L];
  k_fma_p2m<<<LV.nbox, std::max(nt, kP2MChunk), 0, s>>>(F->d_leaf_pptr, F->d_leaf_pan, h->d_rec,
                                                         h->d_cell_dofs, a, b, LV.d_cen, LV.half,
                                                         LV.d_W, F->cst);
  for (int l = L; l > kFmaMinLevel; --l) {
    FmaLevel& P = F->lev[l - 1];
    k_fma_m2m<<<P.nbox, nt, 0, s>>>(P.d_child_ptr, P.d_child, P.d_child_oct, F->d_T,
                                    F->lev[l].d_W, P.d_W, F->cst);
  }
  for (int l = kFmaMinLevel; l <= L; ++l) {
    FmaLevel& V = F->lev[l];
    k_fma_m2l<<<V.nbox, nt, 0, s>>>(V.d_il_ptr, V.d_il, V.d_cen, V.half, V.d_W, V.d_L,
                                     F->cst);
  }
  for (int l = kFmaMinLevel + 1; l <= L; ++l) {
    FmaLevel& V = F->lev[l];
    k_fma_l2l<<<V.nbox, nt, 0, s>>>(V.d_parent, V.d_oct, F->d_T, F->lev[l - 1].d_L, V.d_L,
                                     F->cst);
  }
  k_fma_eval<<<(N + 127) / 128, 128, 0, s>>>(N, h->d_X, F->d_tgt_leaf, LV.d_cen, LV.half,
                                             L >= kFmaMinLevel ? LV.d_L : nullptr, F->d_near_ptr,
                                             F->d_pair_pan, F->d_near_val, h->d_cell_dofs, a, b, y,
                                             F->cst);
  h->launches += 2 + 2 * (L - kFmaMinLevel) + (L - kFmaMinLevel + 1);
  WB_CU(cudaGetLastError());
  return WBEM_OK;
}

// The FMA operators of the collocation system: mode 0 = vmult's operator
// (-D (x s) + N (x o) + alpha x o), 1 = compute_rhs's
// (-(N (x s) + alpha x s) + D (x o)), 2 = alpha = -N 1 (x unused, y = alpha).
int fma_apply(wbem_context* h, int mode, const double* x, double* y) {
  FmaState* F = static_cast<FmaState*>(h->fma_state);
  if (!F) return fail(h, WBEM_ERR_STATE, "FMA: not assembled");
  const int N = h->N, bs = 256, nb = (N + bs - 1) / bs;
  k_fma_inputs<<<nb, bs, 0, h->stream>>>(N, mode, h->d_mask, x, F->d_a, F->d_b);
  WB_CHK(fma_product(h, F->d_a, F->d_b, y));
  k_fma_finish<<<nb, bs, 0, h->stream>>>(N, mode, h->d_mask, h->d_alpha, x, y);
  h->launches += 2;
  WB_CU(cudaGetLastError());
  return WBEM_OK;
}

// The near-field diagonal blocks of the system (for the block-Jacobi
// preconditioner of the FMA solve), for the current mask.
int fma_near_blocks(wbem_context* h, double** blocks) {
  FmaState* F = static_cast<FmaState*>(h->fma_state);
  if (!F) return fail(h, WBEM_ERR_STATE, "FMA: not assembled");
  const int N = h->N, nb = (N + kBJ - 1) / kBJ;
  WB_CU(cudaMemsetAsync(F->d_blocks, 0, sizeof(double) * (size_t)nb * kBJ * kBJ, h->stream));
  k_fma_near_blocks<<<(N + 127) / 128, 128, 0, h->stream>>>(N, F->d_near_ptr, F->d_pair_pan,
                                                            F->d_near_val, h->d_cell_dofs, h->d_mask,
                                                            h->d_alpha, F->d_blocks);
  WB_CU(cudaGetLastError());
  h->launches++;
  *blocks = F->d_blocks;
  return WBEM_OK;
}

// "Solution method = FMA": octree (once per geometry and order), FP64 panel
// records, near field, and alpha = -N 1 through the FMA.
int assemble_fma(wbem_context* h, const QuadTables& qt) {
  const int N = h->N, C = h->C;
  const int n = h->opt.fma_order;
  if (n < 3 || n > kFmaMaxOrder) return fail(h, WBEM_ERR_ARG, "fma_order must be in [3, 8]");
  FmaState* F = static_cast<FmaState*>(h->fma_state);
  if (!F || F->n != n || h->fma_geometry_stale) {
    free_fma(h);
    F = new FmaState();
    F->n = n;
    h->fma_state = F;
    const int st = fma_build(h, F, qt);
    if (st != WBEM_OK) {
      free_fma(h);
      return st;
    }
    h->fma_geometry_stale = false;
  }
  const int nq = qt.q1 * qt.q1;
  if (h->rec_cells != (size_t)C * nq || !h->d_rec) {
    WB_CHK(dev_alloc(h, &h->d_rec, (size_t)C * nq * 8));
    h->rec_cells = (size_t)C * nq;
  }
  if (!h->d_alpha) WB_CHK(dev_alloc(h, &h->d_alpha, (size_t)N));
  EvTimer tm(h->stream);
  WB_CU(launch_cell_records_fp64(C, h->d_X, h->d_cell_dofs, h->d_rec, qt.q1, h->stream));
  h->stats.t_geometry_ms = tm.ms();
  if (F->npairs > 0) {
    const unsigned grid = (unsigned)((F->npairs + 127) / 128);
    k_fma_near<<<grid, 128, 0, h->stream>>>((int)F->npairs, F->d_pair_row, F->d_pair_pan, h->d_X,
                                             h->d_dnset, h->d_cell_dofs, h->d_rec, F->d_near_val,
                                             F->d_qt);
    WB_CU(cudaGetLastError());
  }
  h->stats.t_singular_ms = tm.ms();
  WB_CHK(fma_apply(h, 2, nullptr, h->d_alpha));
  h->stats.t_alpha_ms = tm.ms();
  h->launches += 2;
  return check_device_error(h, "assemble (FMA)");
}

}  // namespace wbem
