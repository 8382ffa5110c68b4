// Fast multipole alternative of the dense collocation operators: the role of
// the reference's BEMFMA (source/bem_fma.cc:56-1196, the mat-vec at :886-1097,
// selected by "Solution method = FMA" in source/bem_problem.cc:87, :646-664,
// :700-712, :974-987). An O(N) mat-vec
//     y = N a + D b      (N = dG/dn, D = G of the collocation system)
// for meshes too large for dense N x N storage, with
//   - an octree over the collocation points and the panel centres; panels
//     are attached to the leaf of their centre;
//   - a near field: every panel of the leaves adjacent to a row's leaf,
//     evaluated on the fly in every product with the regular Gauss rule in
//     FP32 (leaf-local coordinates, two rows per packed FP32x2 instruction),
//     plus stored FP64 corrections for the close pairs (a double-node partner
//     of the row on the panel: the vertex-singular rule; centre within two
//     panel diameters: the regular rule in FP64), so that those pairs carry
//     the dense assembly's values;
//   - the far field through Chebyshev-interpolation expansions of order n
//     per direction (the kernel-independent form of the multipole / local
//     expansions): P2M at the leaves into four sets of n^3 coefficients per
//     box (the charges JxW phi_j b_j and the three components of the dipoles
//     n JxW phi_j a_j of the quadrature points, each interpolated by value),
//     M2M up the tree and L2L down it as three 1-D passes, M2L over the
//     interaction lists as FP32 GEMMs with the operators between Chebyshev
//     nodes (1/r and its gradient for the dipoles) precomputed per box
//     offset, and L2P at the collocation points.
//     Boxes are interpolated over their cube enlarged by kFmaExpand, so that a
//     panel attached by its centre lies inside its leaf's box.
// Every sum runs in a fixed order: the product is deterministic.
// The reference expands in spherical harmonics (its truncation order 3 by
// default); this form trades that for dense n^3 x n^3 translations, which
// map onto the GPU as GEMMs and plain loops. The preconditioner of the GMRES
// solve is block-Jacobi on the near field (the reference: UMFPACK on its
// near-field matrix, source/bem_fma.cc:1099-1196).
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <cstdint>
#include <vector>
#include "context.h"
#include "host_util.h"
#include "fma_tree.h"
#include "kernels.h"

namespace wbem {

using namespace fma_tree;

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
  float S1[2][kFmaMaxOrder][kFmaMaxOrder]; // [child half][child node][parent node] 1-D weights
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

// 1 / sqrt(x) by the hardware approximation with flush-to-zero (one
// instruction; the squared distances here are never subnormal).
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ bool fma_in_set(const int* set, int v) {
  bool r = false;
#pragma unroll
  for (int k = 0; k < kMaxSet; ++k) r |= (set[k] == v);
  return r;
}

// ------------------------------------------------------------ near field
// The near field of a row is every panel attached to a leaf adjacent to the
// row's leaf (the leaf included). The product evaluates all of them on the
// fly in FP32 with the regular Gauss rule, in coordinates local to the leaf
// centres; for the close pairs (panels that hold a double-node partner of the
// row, or whose centre is within two diameters of it) a stored FP64
// correction replaces that FP32 value by the dense assembly's: the
// vertex-singular rule (source/bem_problem.cc:478-522) or the regular rule in
// FP64.

// Panel centre and the larger component of its two diagonals (the measure of
// the close test), FP64, one thread per panel.
__global__ void k_fma_panel_geo(int C, const double* __restrict__ X,
                                const int4* __restrict__ cell_dofs, double* __restrict__ geo) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int4 d = cell_dofs[c];
  const int id[4] = {d.x, d.y, d.z, d.w};
  double P[4][3];
  for (int j = 0; j < 4; ++j)
    for (int e = 0; e < 3; ++e) P[j][e] = X[3 * (size_t)id[j] + e];
  double dia = 0;
  for (int e = 0; e < 3; ++e) {
    geo[4 * (size_t)c + e] = 0.25 * (P[0][e] + P[1][e] + P[2][e] + P[3][e]);
    dia = fmax(dia, fabs(P[3][e] - P[0][e]));
    dia = fmax(dia, fabs(P[2][e] - P[1][e]));
  }
  geo[4 * (size_t)c + 3] = dia;
}

// Close pairs of each row, in the order of the row's neighbour leaves and
// their panels; one thread per row, the rows taken in leaf order (tidx) so
// that a warp walks the same neighbour panels. Count pass (ptr == nullptr):
// cnt[i] = (pairs, singular pairs). List pass: the pairs as (row, panel) from ptr[i]
// on, and their indices in the correction list, the regular pairs from
// lptr[i].x on and the singular ones from lptr[i].y on.
__global__ void k_fma_close(int N, const int* __restrict__ tidx, const int* __restrict__ tgt_leaf,
                            const int* __restrict__ nb_ptr,
                            const int* __restrict__ nb, const int* __restrict__ leaf_pptr,
                            const int* __restrict__ leaf_pan, const double* __restrict__ X,
                            const double* __restrict__ geo, const int* __restrict__ sptr,
                            const int* __restrict__ scell, const int* __restrict__ ptr,
                            const int2* __restrict__ lptr, int2* __restrict__ cnt,
                            int* __restrict__ prow, int* __restrict__ ppan,
                            int* __restrict__ plist) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const int i = tidx[j];
  const double xi = X[3 * (size_t)i], yi = X[3 * (size_t)i + 1], zi = X[3 * (size_t)i + 2];
  const int t = tgt_leaf[i];
  const int base = ptr ? ptr[i] : 0;
  const int2 lp = ptr ? lptr[i] : make_int2(0, 0);
  // the row's singular cells, in registers when there are at most 16
  const int s0 = sptr[i], nsr = sptr[i + 1] - s0;
  int sc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) sc[q] = q < nsr ? scell[s0 + q] : -1;
  int c = 0, ns = 0;
  for (int e = nb_ptr[t]; e < nb_ptr[t + 1]; ++e) {
    const int s = nb[e];
    for (int k = leaf_pptr[s]; k < leaf_pptr[s + 1]; ++k) {
      const int cell = leaf_pan[k];
      const double* g = geo + 4 * (size_t)cell;
      const double dx = g[0] - xi, dy = g[1] - yi, dz = g[2] - zi;
      bool sing = false;  // a double-node partner of the row is a vertex of the panel
      if (nsr <= 16) {
#pragma unroll
        for (int q = 0; q < 16; ++q) sing |= sc[q] == cell;
      } else {
        for (int m = s0; m < s0 + nsr && !sing; ++m) sing = scell[m] == cell;
      }
      const bool close = sing || dx * dx + dy * dy + dz * dz < 12.0 * g[3] * g[3];
      if (!close) continue;
      if (ptr) {
        prow[base + c] = i;
        ppan[base + c] = cell;
        if (sing) plist[lp.y + ns] = base + c;
        else plist[lp.x + c - ns] = base + c;
      }
      ns += sing ? 1 : 0;
      ++c;
    }
  }
  if (!ptr) cnt[i] = make_int2(c, ns);
}

// The FP32 value the product computes for one (row, panel) pair, as the 4 N
// and 4 D coefficients of the panel's vertex values: P = the panel's nq
// points local to their leaf centre, (cx, cy, cz) = that centre minus the
// row's position.
__device__ __forceinline__ void fma_pair_approx(const float4* __restrict__ P,
                                                const double* __restrict__ r, float cx, float cy,
                                                float cz, const FmaConst& c_fma, float ln[4],
                                                float ld[4]) {
  for (int j = 0; j < 4; ++j) ln[j] = ld[j] = 0.f;
  for (int q = 0; q < c_fma.nq; ++q) {
    const float4 y = P[q];
    const float rx = y.x + cx, ry = y.y + cy, rz = y.z + cz;
    const float ri = rsqrt_approx(fmaf(rx, rx, fmaf(ry, ry, rz * rz)));
    const double* rq = r + 8 * q;
    const float sq = (float)rq[3] * ri;
    const float dq = -fmaf(rx, (float)rq[4], fmaf(ry, (float)rq[5], rz * (float)rq[6])) * (ri * ri * ri);
    for (int j = 0; j < 4; ++j) {
      ln[j] = fmaf(dq, c_fma.phi[q][j], ln[j]);
      ld[j] = fmaf(sq, c_fma.phi[q][j], ld[j]);
    }
  }
}

// Corrections of the close pairs, one thread per pair of a list (the
// regular and the singular pairs are launched as separate lists, so that the
// warps do not diverge between the 16-point and the vertex-singular rules):
// the dense assembly's FP64 value (4 N and 4 D entries) minus the product's
// FP32 value, stored as val[8 * pair + 0..3] = N, [4..7] = D.
__global__ void k_fma_close_val(long long npairs, const int* __restrict__ plist,
                                const int* __restrict__ pair_row,
                                const int* __restrict__ pair_pan, const double* __restrict__ X,
                                const int* __restrict__ dnset, const int4* __restrict__ cell_dofs,
                                const double* __restrict__ rec, const int* __restrict__ tgt_leaf,
                                const int* __restrict__ pan_pos, const int* __restrict__ pos_leaf,
                                const double* __restrict__ cen, const float4* __restrict__ xloc,
                                const float4* __restrict__ ppos, double* __restrict__ val,
                                const QuadTables* __restrict__ qt, const __grid_constant__ FmaConst c_fma) {
  const long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (li >= npairs) return;
  const int k = plist[li];
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
  const int nq = qt->q1 * qt->q1;
  const double* r = rec + (size_t)cell * nq * 8;
  if (v >= 0) {
    // vertex-singular rule at local vertex v
    double P[4][3];
    for (int j = 0; j < 4; ++j)
      for (int e = 0; e < 3; ++e) P[j][e] = X[3 * (size_t)id[j] + e];
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
    // the regular rule in FP64
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
  }
  // minus what the product evaluates for this pair
  const int kp = pan_pos[cell], s = pos_leaf[kp], t = tgt_leaf[row];
  const float4 xl = xloc[row];
  float lnf[4], ldf[4];
  fma_pair_approx(ppos + (size_t)kp * nq, r, (float)(cen[3 * s] - cen[3 * t]) - xl.x,
                  (float)(cen[3 * s + 1] - cen[3 * t + 1]) - xl.y,
                  (float)(cen[3 * s + 2] - cen[3 * t + 2]) - xl.z, c_fma, lnf, ldf);
  double* o = val + 8 * (size_t)k;
  for (int j = 0; j < 4; ++j) {
    o[j] = ln[j] - (double)lnf[j];
    o[4 + j] = ld[j] - (double)ldf[j];
  }
}

// The near-field entries of the diagonal 128-blocks of the system operator
// (sel_j ? -D_ij : N_ij, plus alpha on Neumann diagonals), for the
// block-Jacobi preconditioner of the FMA solve: the FP32 values of the
// neighbour panels with a vertex in the row's block plus the close-pair
// corrections. One thread per row writes its own block row (blocks zeroed
// before).
__global__ void k_fma_near_blocks(int N, const int* __restrict__ tgt_leaf,
                                  const int* __restrict__ nb_ptr, const int* __restrict__ nb,
                                  const int* __restrict__ leaf_pptr, const int* __restrict__ leaf_pan,
                                  const double* __restrict__ cen, const float4* __restrict__ xloc,
                                  const float4* __restrict__ ppos, const double* __restrict__ rec,
                                  const int* __restrict__ close_ptr, const int* __restrict__ pair_pan,
                                  const double* __restrict__ val, const int4* __restrict__ cell_dofs,
                                  const uint8_t* __restrict__ mask, const double* __restrict__ alpha,
                                  double* __restrict__ blocks, const __grid_constant__ FmaConst c_fma) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int b = i / kBJ, r = i % kBJ, t = tgt_leaf[i], nq = c_fma.nq;
  const float4 xl = xloc[i];
  double* row = blocks + ((size_t)b * kBJ + r) * kBJ;
  for (int e = nb_ptr[t]; e < nb_ptr[t + 1]; ++e) {
    const int s = nb[e];
    const float cx = (float)(cen[3 * s] - cen[3 * t]) - xl.x;
    const float cy = (float)(cen[3 * s + 1] - cen[3 * t + 1]) - xl.y;
    const float cz = (float)(cen[3 * s + 2] - cen[3 * t + 2]) - xl.z;
    for (int k = leaf_pptr[s]; k < leaf_pptr[s + 1]; ++k) {
      const int cell = leaf_pan[k];
      const int4 d = cell_dofs[cell];
      const int id[4] = {d.x, d.y, d.z, d.w};
      if (id[0] / kBJ != b && id[1] / kBJ != b && id[2] / kBJ != b && id[3] / kBJ != b) continue;
      float lnf[4], ldf[4];
      fma_pair_approx(ppos + (size_t)k * nq, rec + (size_t)cell * nq * 8, cx, cy, cz, c_fma, lnf, ldf);
      for (int j = 0; j < 4; ++j)
        if (id[j] / kBJ == b) row[id[j] % kBJ] += mask[id[j]] ? -(double)ldf[j] : (double)lnf[j];
    }
  }
  for (int k = close_ptr[i]; k < close_ptr[i + 1]; ++k) {
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
// Per-point data of the panels in leaf order (point f = k nq + q of the
// panel at position k of the leaf lists): its position local to the centre
// of the panel's leaf (once per assembly) and its strengths, the charge
// JxW phi.b and the dipole n JxW phi.a (once per product; the record weights
// carry the 1 / (4 pi)).
__global__ void k_fma_points(int npts, int nq, const int* __restrict__ leaf_pan,
                             const int* __restrict__ pos_leaf, const double* __restrict__ rec,
                             const double* __restrict__ cen, float4* __restrict__ ppos) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= npts) return;
  const int k = f / nq, q = f % nq, cell = leaf_pan[k], s = pos_leaf[k];
  const double* r = rec + ((size_t)cell * nq + q) * 8;
  ppos[f] = make_float4((float)(r[0] - cen[3 * s]), (float)(r[1] - cen[3 * s + 1]),
                        (float)(r[2] - cen[3 * s + 2]), 0.f);
}

__global__ void k_fma_strengths(int npts, const int* __restrict__ leaf_pan,
                                const double* __restrict__ rec, const int4* __restrict__ cell_dofs,
                                const double* __restrict__ a, const double* __restrict__ b,
                                float4* __restrict__ pstr, const __grid_constant__ FmaConst c_fma) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= npts) return;
  const int nq = c_fma.nq, k = f / nq, q = f % nq, cell = leaf_pan[k];
  const double* r = rec + ((size_t)cell * nq + q) * 8;
  const int4 d = cell_dofs[cell];
  const double sb = c_fma.phi[q][0] * b[d.x] + c_fma.phi[q][1] * b[d.y] + c_fma.phi[q][2] * b[d.z] +
                    c_fma.phi[q][3] * b[d.w];
  const double sa = c_fma.phi[q][0] * a[d.x] + c_fma.phi[q][1] * a[d.y] + c_fma.phi[q][2] * a[d.z] +
                    c_fma.phi[q][3] * a[d.w];
  pstr[f] = make_float4((float)(r[3] * sb), (float)(r[4] * sa), (float)(r[5] * sa), (float)(r[6] * sa));
}

// P2M in work items of up to kP2MPanels panels of one leaf (so that large
// leaves spread over several CTAs), kP2MGroups groups of kP2MGroupThreads
// threads per item. A box's multipole expansion has four sets of n^3
// coefficients: the charges and the three dipole components, each
// interpolated by value (the dipoles' kernel derivative is applied exactly
// in the M2L, which keeps the double layer as accurate as the single
// layer). Thread (i, j) < n^2 of a group holds coefficients (i, j, 0..n-1)
// of the four sets over the group's chunks of kP2MChunk points (chunks g,
// g + G, ...), whose 1-D interpolation weights the group computes first (one
// thread per point and axis). The groups' sums are added in a fixed order
// into the item's partial expansion; k_fma_p2m_sum adds a leaf's items in
// order.
constexpr int kP2MPanels = 32;
constexpr int kP2MChunk = 32;
constexpr int kP2MGroups = 4;
constexpr int kP2MGroupThreads = 64;
constexpr int kMpSets = 4;  // charge, dipole x, y, z
template <int NO>
__global__ void __launch_bounds__(kP2MGroups* kP2MGroupThreads)
k_fma_p2m(const int4* __restrict__ items, const float4* __restrict__ ppos,
          const float4* __restrict__ pstr, double half, float* __restrict__ Wpart,
          const __grid_constant__ FmaConst c_fma) {
  constexpr int n3 = NO * NO * NO;
  const int nq = c_fma.nq, g = threadIdx.y, tid = threadIdx.x;
  __shared__ float4 sg[kP2MGroups][kP2MChunk];
  __shared__ __align__(16) float Sw[kP2MGroups][kP2MChunk][3][kFmaMaxOrder];
  __shared__ float red[kP2MGroups][kMpSets * n3];
  const int4 it = items[blockIdx.x];
  const int p0 = it.y * nq, p1 = it.z * nq;
  const int nchunk = (p1 - p0 + kP2MChunk - 1) / kP2MChunk;
  const int rounds = (nchunk + kP2MGroups - 1) / kP2MGroups;
  const int mi = tid / NO, mj = tid % NO;
  const float ih = (float)(1.0 / half);
  float acc[kMpSets][NO];
#pragma unroll
  for (int q = 0; q < kMpSets; ++q)
#pragma unroll
    for (int k = 0; k < NO; ++k) acc[q][k] = 0.f;
  for (int r = 0; r < rounds; ++r) {
    const int base = p0 + (r * kP2MGroups + g) * kP2MChunk;
    const int cnt = max(0, min(kP2MChunk, p1 - base));
    for (int x = tid; x < 3 * cnt; x += kP2MGroupThreads) {
      const int pt = x / 3, dir = x % 3;
      const float4 y = ppos[base + pt];
      cheb_weights(c_fma, (dir == 0 ? y.x : dir == 1 ? y.y : y.z) * ih, Sw[g][pt][dir], nullptr);
      if (dir == 0) sg[g][pt] = pstr[base + pt];
    }
    __syncthreads();
    if (tid < NO * NO) {
      for (int p = 0; p < cnt; ++p) {
        const float4 q4 = sg[g][p];
        const float sxy = Sw[g][p][0][mi] * Sw[g][p][1][mj];
        const float c0 = q4.x * sxy, c1 = q4.y * sxy, c2 = q4.z * sxy, c3 = q4.w * sxy;
        const float* sz = Sw[g][p][2];
#pragma unroll
        for (int k = 0; k < NO; ++k) {
          acc[0][k] = fmaf(c0, sz[k], acc[0][k]);
          acc[1][k] = fmaf(c1, sz[k], acc[1][k]);
          acc[2][k] = fmaf(c2, sz[k], acc[2][k]);
          acc[3][k] = fmaf(c3, sz[k], acc[3][k]);
        }
      }
    }
    __syncthreads();
  }
  if (tid < NO * NO)
#pragma unroll
    for (int q = 0; q < kMpSets; ++q)
#pragma unroll
      for (int k = 0; k < NO; ++k) red[g][q * n3 + tid * NO + k] = acc[q][k];
  __syncthreads();
  for (int m = g * kP2MGroupThreads + tid; m < kMpSets * n3; m += kP2MGroups * kP2MGroupThreads) {
    float v = red[0][m];
#pragma unroll
    for (int k = 1; k < kP2MGroups; ++k) v += red[k][m];
    Wpart[(size_t)blockIdx.x * kMpSets * n3 + m] = v;
  }
}

// W_leaf = sum of the leaf's P2M items in order; one CTA per leaf.
__global__ void k_fma_p2m_sum(const int* __restrict__ iptr, const float* __restrict__ Wpart,
                              float* __restrict__ W, int n3) {
  const int leaf = blockIdx.x;
  for (int m = threadIdx.x; m < n3; m += blockDim.x) {
    float v = 0.f;
    for (int k = iptr[leaf]; k < iptr[leaf + 1]; ++k) v += Wpart[(size_t)k * n3 + m];
    W[(size_t)leaf * n3 + m] = v;
  }
}

// M2M and L2L through the 1-D child -> parent interpolation matrices
// S1[h][c][P] (the parent's weight of node P at child node c, h = the
// child's half along the axis): the n^3 x n^3 translation is their tensor
// product, applied as three passes of n^4 multiply-adds.
// M2M: one CTA per parent box; W_P[P] = sum_children sum_c T[c][P] W_c[c],
// for each of the kMpSets coefficient sets (stride kMpSets n^3 per box).
__global__ void k_fma_m2m(const int* __restrict__ child_ptr, const int* __restrict__ child,
                          const int* __restrict__ child_oct, const float* __restrict__ Wc,
                          float* __restrict__ Wp, const __grid_constant__ FmaConst c_fma) {
  const int p = blockIdx.x, tid = threadIdx.x, n = c_fma.n, n3 = c_fma.n3;
  __shared__ float w[kFmaMaxOrder * kFmaMaxOrder * kFmaMaxOrder];
  __shared__ float t1[kFmaMaxOrder * kFmaMaxOrder * kFmaMaxOrder];
  const int i0 = tid / (n * n), i1 = (tid / n) % n, i2 = tid % n;
  for (int set = 0; set < kMpSets; ++set) {
    float acc = 0.f;
    for (int e = child_ptr[p]; e < child_ptr[p + 1]; ++e) {
      const int o = child_oct[e];
      const float(*Sx)[kFmaMaxOrder] = c_fma.S1[o >> 2];
      const float(*Sy)[kFmaMaxOrder] = c_fma.S1[(o >> 1) & 1];
      const float(*Sz)[kFmaMaxOrder] = c_fma.S1[o & 1];
      __syncthreads();
      if (tid < n3) w[tid] = Wc[((size_t)child[e] * kMpSets + set) * n3 + tid];
      __syncthreads();
      if (tid < n3) {  // t1[cx][cy][Pz]
        float v = 0.f;
        for (int c = 0; c < n; ++c) v = fmaf(Sz[c][i2], w[(i0 * n + i1) * n + c], v);
        t1[tid] = v;
      }
      __syncthreads();
      if (tid < n3) {  // w[cx][Py][Pz]
        float v = 0.f;
        for (int c = 0; c < n; ++c) v = fmaf(Sy[c][i1], t1[(i0 * n + c) * n + i2], v);
        w[tid] = v;
      }
      __syncthreads();
      if (tid < n3)  // W_P[Px][Py][Pz]
        for (int c = 0; c < n; ++c) acc = fmaf(Sx[c][i0], w[(c * n + i1) * n + i2], acc);
    }
    if (tid < n3) Wp[((size_t)p * kMpSets + set) * n3 + tid] = acc;
  }
}

// M2L. The kernel 1/r is homogeneous and the interpolation cubes scale with
// the boxes, so the operator between the nodes of two boxes of one level
// depends only on their offset d = key_target - key_source in [-3, 3]^3 (in
// box units). With R = d + (e / 2)(t_a - t_m) it has four blocks of n^3
// columns, one per multipole set: 1 / |R| for the charges and R_k / |R|^3
// (the gradient of 1/|x - y| in y) for the dipole components, divided by the
// box size of the level and by its square. The operators are computed once
// per order and the M2L of a product runs as FP32 GEMMs (K = 4 n^3), one per
// (level, offset) group of up to kM2LPairs (target, source) pairs:
// C[a][p] = sum_m' K[d][a][m'] W_{s_p}[m'], written per pair; k_fma_m2l_sum
// adds a box's pairs in its list order.
constexpr int kM2LOffsets = 343;  // ((dx + 3) 7 + dy + 3) 7 + dz + 3
constexpr int kM2LPairs = 64;
constexpr int kM2LRows = 128;
constexpr int kM2LK = 32;
__global__ void k_fma_m2l_ops(int n, double e2, float* __restrict__ K) {
  const int oi = blockIdx.x, a = blockIdx.y, n3 = n * n * n, kd = kMpSets * n3;
  const int dx = oi / 49 - 3, dy = (oi / 7) % 7 - 3, dz = oi % 7 - 3;
  const bool used = max(abs(dx), max(abs(dy), abs(dz))) >= 2;
  __shared__ double tn[kFmaMaxOrder];  // Chebyshev nodes, scaled by e / 2
  if (threadIdx.x < n)
    tn[threadIdx.x] = e2 * cos((2 * threadIdx.x + 1) * 3.14159265358979323846 / (2.0 * n));
  __syncthreads();
  const double ax = dx + tn[a / (n * n)], ay = dy + tn[(a / n) % n], az = dz + tn[a % n];
  float* row = K + ((size_t)oi * n3 + a) * kd;
  for (int m = threadIdx.x; m < n3; m += blockDim.x) {
    float k0 = 0.f, k1 = 0.f, k2 = 0.f, k3 = 0.f;
    if (used) {
      const double rx = ax - tn[m / (n * n)], ry = ay - tn[(m / n) % n], rz = az - tn[m % n];
      const double ri = 1.0 / sqrt(rx * rx + ry * ry + rz * rz), ri3 = ri * ri * ri;
      k0 = (float)ri;
      k1 = (float)(rx * ri3);
      k2 = (float)(ry * ri3);
      k3 = (float)(rz * ri3);
    }
    row[m] = k0;
    row[n3 + m] = k1;
    row[2 * n3 + m] = k2;
    row[3 * n3 + m] = k3;
  }
}

// items: (offset, first entry, entries, level); entries: source box and
// output row (global over the levels); one CTA of 256 threads per item, each
// thread an 8 x 4 block of C per pass of kM2LRows target nodes. The dipole
// columns (m' >= n3) carry one more factor 1 / s, applied when staged.
__global__ void __launch_bounds__(256)
k_fma_m2l_gemm(const int4* __restrict__ items, const int* __restrict__ ent_src,
               const int* __restrict__ ent_out, const float* __restrict__ K,
               const float* __restrict__ Wall, const float* __restrict__ lvl_scale,
               float* __restrict__ part, int n3) {
  __shared__ __align__(16) float Ks[kM2LK][kM2LRows + 4];
  __shared__ __align__(16) float Ws[kM2LK][kM2LPairs + 4];
  const int kd = kMpSets * n3;
  const int4 it = items[blockIdx.x];
  const int begin = it.y, cnt = it.z;
  const float sc = lvl_scale[it.w];
  const float* Ko = K + (size_t)it.x * n3 * kd;
  const int tid = threadIdx.x, ty = tid / 16, tx = tid % 16;
  for (int a0 = 0; a0 < n3; a0 += kM2LRows) {
    float acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int m0 = 0; m0 < kd; m0 += kM2LK) {
      __syncthreads();
      for (int x = tid; x < kM2LRows * kM2LK; x += 256) {
        const int r = x / kM2LK, c = x % kM2LK, a = a0 + r, m = m0 + c;
        Ks[c][r] = (a < n3 && m < kd) ? Ko[(size_t)a * kd + m] : 0.f;
      }
      for (int x = tid; x < kM2LPairs * kM2LK; x += 256) {
        const int p = x / kM2LK, c = x % kM2LK, m = m0 + c;
        float w = (p < cnt && m < kd) ? Wall[(size_t)ent_src[begin + p] * kd + m] : 0.f;
        Ws[c][p] = m >= n3 ? w * sc : w;
      }
      __syncthreads();
#pragma unroll 8
      for (int c = 0; c < kM2LK; ++c) {
        const float4 k0 = *reinterpret_cast<const float4*>(&Ks[c][ty * 8]);
        const float4 k1 = *reinterpret_cast<const float4*>(&Ks[c][ty * 8 + 4]);
        const float4 w = *reinterpret_cast<const float4*>(&Ws[c][tx * 4]);
        const float av[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
        const float wv[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], wv[j], acc[i][j]);
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int a = a0 + ty * 8 + i;
      if (a >= n3) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int p = tx * 4 + j;
        if (p < cnt) part[(size_t)ent_out[begin + p] * n3 + a] = acc[i][j] * sc;
      }
    }
  }
}

// L_box = sum of the box's M2L pairs in list order (all levels at once; the
// boxes of levels without lists get zero).
__global__ void k_fma_m2l_sum(const int* __restrict__ gptr, const float* __restrict__ part,
                              float* __restrict__ Lall, int n3) {
  const int bx = blockIdx.x;
  for (int a = threadIdx.x; a < n3; a += blockDim.x) {
    float v = 0.f;
    for (int e = gptr[bx]; e < gptr[bx + 1]; ++e) v += part[(size_t)e * n3 + a];
    Lall[(size_t)bx * n3 + a] = v;
  }
}

// L2L: one CTA per child box; L_c[c] += sum_P T[c][P] L_P[P].
__global__ void k_fma_l2l(const int* __restrict__ parent, const int* __restrict__ oct,
                          const float* __restrict__ Lp, float* __restrict__ Lc,
                          const __grid_constant__ FmaConst c_fma) {
  const int cb = blockIdx.x, tid = threadIdx.x, n = c_fma.n, n3 = c_fma.n3;
  __shared__ float l[kFmaMaxOrder * kFmaMaxOrder * kFmaMaxOrder];
  __shared__ float t1[kFmaMaxOrder * kFmaMaxOrder * kFmaMaxOrder];
  const int o = oct[cb];
  const float(*Sx)[kFmaMaxOrder] = c_fma.S1[o >> 2];
  const float(*Sy)[kFmaMaxOrder] = c_fma.S1[(o >> 1) & 1];
  const float(*Sz)[kFmaMaxOrder] = c_fma.S1[o & 1];
  const int i0 = tid / (n * n), i1 = (tid / n) % n, i2 = tid % n;
  if (tid < n3) l[tid] = Lp[(size_t)parent[cb] * n3 + tid];
  __syncthreads();
  if (tid < n3) {  // t1[Px][Py][cz]
    float v = 0.f;
    for (int P = 0; P < n; ++P) v = fmaf(Sz[i2][P], l[(i0 * n + i1) * n + P], v);
    t1[tid] = v;
  }
  __syncthreads();
  float v = 0.f;
  if (tid < n3)  // [Px][cy][cz]
    for (int P = 0; P < n; ++P) v = fmaf(Sy[i1][P], t1[(i0 * n + P) * n + i2], v);
  __syncthreads();
  if (tid < n3) l[tid] = v;
  __syncthreads();
  if (tid < n3) {  // [cx][cy][cz]
    float acc = Lc[(size_t)cb * n3 + tid];
    for (int P = 0; P < n; ++P) acc = fmaf(Sx[i0][P], l[(P * n + i1) * n + i2], acc);
    Lc[(size_t)cb * n3 + tid] = acc;
  }
}

// The product's evaluation at the collocation points, one CTA per chunk of
// up to kEvalTargets rows of one leaf, each thread holding four rows (two
// packed pairs) and kEvalLanes threads sharing a quad: the far field (L2P of
// the leaf's local expansion), the near field evaluated on the fly over the
// points of the neighbour leaves (FP32 in coordinates local to this leaf's
// centre, two rows per packed FP32x2 instruction, points staged in shared
// memory with each value duplicated for the packed operands and the next
// chunk loaded into registers meanwhile; FP64 sum of FP32 partials) and the
// close-pair corrections (FP64). The lanes of a quad split every sum the same
// way on every call and are combined by shuffles: the product is
// deterministic.
constexpr int kEvalTargets = 64;
constexpr int kEvalLanes = 8;
constexpr int kEvalRows = 4;  // rows per thread
constexpr int kEvalThreads = kEvalTargets / kEvalRows * kEvalLanes;
constexpr int kEvalChunk = 256;
// Packed FP32x2 arithmetic on 64-bit registers (two rows per instruction).
__device__ __forceinline__ unsigned long long pk2(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void upk2(unsigned long long v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long add2(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b,
                                                   unsigned long long c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__global__ void __launch_bounds__(kEvalThreads)
k_fma_eval(const int2* __restrict__ items, const int* __restrict__ tptr, const int* __restrict__ tidx,
           const float4* __restrict__ xloc, const int* __restrict__ nb_ptr, const int* __restrict__ nb,
           const int* __restrict__ leaf_pptr, const double* __restrict__ cen, double half,
           const float* __restrict__ Lx, const float4* __restrict__ ppos,
           const float4* __restrict__ pstr, const int* __restrict__ close_ptr,
           const int* __restrict__ pair_pan, const double* __restrict__ val,
           const int4* __restrict__ cell_dofs, const double* __restrict__ a,
           const double* __restrict__ b, double* __restrict__ y,
           const __grid_constant__ FmaConst c_fma) {
  // point k, each value duplicated for the packed operands:
  // sA = ((x, x), (y, y)), sB = ((z, z), (q, q)), sC = ((-mx, -mx), (-my, -my)), sD = (-mz, -mz)
  __shared__ ulonglong2 sA[kEvalChunk], sB[kEvalChunk], sC[kEvalChunk];
  __shared__ unsigned long long sD[kEvalChunk];
  __shared__ float sL[kFmaMaxOrder * kFmaMaxOrder * kFmaMaxOrder];
  __shared__ float sw[kEvalTargets][3][kFmaMaxOrder];
  __shared__ int snp[28];
  __shared__ float soff[27][3];
  const int2 it = items[blockIdx.x];
  const int leaf = it.x, t0 = it.y;
  const int nt = min(kEvalTargets, tptr[leaf + 1] - t0);
  const int tid = threadIdx.x, qd = tid / kEvalLanes, lane = tid % kEvalLanes;
  int ix[kEvalRows];
  float4 xr[kEvalRows];
#pragma unroll
  for (int h = 0; h < kEvalRows; ++h) {
    const int r = kEvalRows * qd + h;
    ix[h] = r < nt ? tidx[t0 + r] : -1;
    xr[h] = ix[h] >= 0 ? xloc[ix[h]] : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  const int n = c_fma.n, n3 = c_fma.n3, nq = c_fma.nq;
  double acc[kEvalRows] = {0.0, 0.0, 0.0, 0.0};
  if (Lx) {
    for (int k = tid; k < n3; k += kEvalThreads) sL[k] = Lx[(size_t)leaf * n3 + k];
    // the quad's 3 x kEvalRows (row, axis) weight sets over its kEvalLanes lanes
    for (int x = lane; x < 3 * kEvalRows; x += kEvalLanes) {
      const int hh = x / 3, dir = x % 3;
      float u = 0.f;  // the coordinate by unrolled selection (no indexed register array)
#pragma unroll
      for (int h = 0; h < kEvalRows; ++h)
        if (h == hh) u = dir == 0 ? xr[h].x : dir == 1 ? xr[h].y : xr[h].z;
      cheb_weights(c_fma, u * (float)(1.0 / half), sw[kEvalRows * qd + hh][dir], nullptr);
    }
    __syncthreads();
#pragma unroll
    for (int h = 0; h < kEvalRows; ++h) {
      const int r = kEvalRows * qd + h;
      float f = 0.f;
      for (int uv = lane; uv < n * n; uv += kEvalLanes) {
        const float sxy = sw[r][0][uv / n] * sw[r][1][uv % n];
        const float* Lr = sL + uv * n;
        for (int w = 0; w < n; ++w) f = fmaf(sxy * sw[r][2][w], Lr[w], f);
      }
      acc[h] = (double)f;
    }
  }
  const int ne = nb_ptr[leaf + 1] - nb_ptr[leaf];
  if (tid == 0) {
    int c = 0;
    for (int e = 0; e < ne; ++e) {
      const int sl = nb[nb_ptr[leaf] + e];
      snp[e] = c;
      c += (leaf_pptr[sl + 1] - leaf_pptr[sl]) * nq;
      for (int d = 0; d < 3; ++d) soff[e][d] = (float)(cen[3 * sl + d] - cen[3 * leaf + d]);
    }
    snp[ne] = c;
  }
  __syncthreads();
  const int total = snp[ne];
  const unsigned long long cx0 = pk2(-xr[0].x, -xr[1].x), cy0 = pk2(-xr[0].y, -xr[1].y),
                           cz0 = pk2(-xr[0].z, -xr[1].z);
  const unsigned long long cx1 = pk2(-xr[2].x, -xr[3].x), cy1 = pk2(-xr[2].y, -xr[3].y),
                           cz1 = pk2(-xr[2].z, -xr[3].z);
  // point g of the sequence: leaf-local position plus its leaf's offset
  auto fetch = [&](int g, float4& P, float4& Q) {
    int e = 0;
    while (g >= snp[e + 1]) ++e;
    const int f = leaf_pptr[nb[nb_ptr[leaf] + e]] * nq + (g - snp[e]);
    P = ppos[f];
    Q = pstr[f];
    P.x += soff[e][0];
    P.y += soff[e][1];
    P.z += soff[e][2];
  };
  constexpr int kPer = kEvalChunk / kEvalThreads;  // staged points per thread
  float4 nP[kPer], nQ[kPer];
#pragma unroll
  for (int u = 0; u < kPer; ++u)
    if (u * kEvalThreads + tid < total) fetch(u * kEvalThreads + tid, nP[u], nQ[u]);
  unsigned long long pa0 = 0ull, pa1 = 0ull;
  int nchunk = 0;
  for (int base = 0; base < total; base += kEvalChunk) {
    const int cnt = min(kEvalChunk, total - base);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int j = u * kEvalThreads + tid;
      if (j < cnt) {
        const float4 P = nP[u], Q = nQ[u];
        sA[j] = make_ulonglong2(pk2(P.x, P.x), pk2(P.y, P.y));
        sB[j] = make_ulonglong2(pk2(P.z, P.z), pk2(Q.x, Q.x));
        sC[j] = make_ulonglong2(pk2(-Q.y, -Q.y), pk2(-Q.z, -Q.z));
        sD[j] = pk2(-Q.w, -Q.w);
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int g = base + kEvalChunk + u * kEvalThreads + tid;
      if (g < total) fetch(g, nP[u], nQ[u]);
    }
    // q / r - (R . m) / r^3 = (q - (R . m) / r^2) / r for two row pairs
    auto term = [&](int k, unsigned long long& p0, unsigned long long& p1) {
      const ulonglong2 A = sA[k], B = sB[k], C = sC[k];
      const unsigned long long D = sD[k];
      {
        const unsigned long long rx = add2(A.x, cx0), ry = add2(A.y, cy0), rz = add2(B.x, cz0);
        const unsigned long long r2 = fma2(rx, rx, fma2(ry, ry, mul2(rz, rz)));
        float q0, q1;
        upk2(r2, q0, q1);
        const unsigned long long ri = pk2(rsqrt_approx(q0), rsqrt_approx(q1));
        const unsigned long long dn = fma2(rx, C.x, fma2(ry, C.y, mul2(rz, D)));
        p0 = fma2(fma2(dn, mul2(ri, ri), B.y), ri, p0);
      }
      {
        const unsigned long long rx = add2(A.x, cx1), ry = add2(A.y, cy1), rz = add2(B.x, cz1);
        const unsigned long long r2 = fma2(rx, rx, fma2(ry, ry, mul2(rz, rz)));
        float q0, q1;
        upk2(r2, q0, q1);
        const unsigned long long ri = pk2(rsqrt_approx(q0), rsqrt_approx(q1));
        const unsigned long long dn = fma2(rx, C.x, fma2(ry, C.y, mul2(rz, D)));
        p1 = fma2(fma2(dn, mul2(ri, ri), B.y), ri, p1);
      }
    };
    for (int k = lane; k < cnt; k += kEvalLanes) term(k, pa0, pa1);
    // FP64 sum of FP32 partials every eight chunks
    if ((++nchunk & 7) == 0 || base + kEvalChunk >= total) {
      float l0, h0, l1, h1;
      upk2(pa0, l0, h0);
      upk2(pa1, l1, h1);
      acc[0] += (double)l0;
      acc[1] += (double)h0;
      acc[2] += (double)l1;
      acc[3] += (double)h1;
      pa0 = pa1 = 0ull;
    }
  }
#pragma unroll
  for (int h = 0; h < kEvalRows; ++h) {
    const int i = ix[h];
    if (i < 0) continue;
    double c = 0.0;
    for (int k = close_ptr[i] + lane; k < close_ptr[i + 1]; k += kEvalLanes) {
      const int4 d = cell_dofs[pair_pan[k]];
      const double* v = val + 8 * (size_t)k;
      c += v[0] * a[d.x] + v[1] * a[d.y] + v[2] * a[d.z] + v[3] * a[d.w] + v[4] * b[d.x] +
           v[5] * b[d.y] + v[6] * b[d.z] + v[7] * b[d.w];
    }
    acc[h] += c;
  }
#pragma unroll
  for (int h = 0; h < kEvalRows; ++h)
#pragma unroll
    for (int o = 1; o < kEvalLanes; o <<= 1) acc[h] += __shfl_xor_sync(0xffffffffu, acc[h], o);
  if (lane == 0)
#pragma unroll
    for (int h = 0; h < kEvalRows; ++h)
      if (ix[h] >= 0) y[ix[h]] = acc[h];
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
  int* d_child_ptr = nullptr;    // children at the next level, CSR
  int* d_child = nullptr;
  int* d_child_oct = nullptr;
  int* d_parent = nullptr;       // parent at the previous level
  int* d_oct = nullptr;          // octant in the parent
  float* d_W = nullptr;          // nbox x n^3
  float* d_L = nullptr;
  std::vector<int> parent, oct, il_ptr;  // host copies
};

struct FmaState {
  int L = 0, n = 0, nq = 0;
  std::vector<FmaLevel> lev;
  int nleaf = 0;
  int* d_leaf_pptr = nullptr;    // panels per leaf (CSR over positions k)
  int* d_leaf_pan = nullptr;     // panel at position k
  int* d_pos_leaf = nullptr;     // leaf of position k
  int* d_pan_pos = nullptr;      // position of each panel
  int* d_tgt_leaf = nullptr;     // leaf of each row
  int* d_tptr = nullptr;         // rows per leaf (CSR), rows sorted by leaf
  int* d_tidx = nullptr;
  int* d_nb_ptr = nullptr;       // neighbour leaves of each leaf (itself included), CSR
  int* d_nb = nullptr;
  int2* d_items = nullptr;       // evaluation work items: (leaf, first row in tidx)
  int n_items = 0;
  int4* d_p2m_items = nullptr;   // P2M work items: (leaf, first and end panel position)
  int* d_p2m_iptr = nullptr;     // P2M items per leaf (CSR)
  float* d_Wpart = nullptr;      // partial expansions of the P2M items
  int n_p2m_items = 0;
  int total_boxes = 0;
  float* d_Wall = nullptr;       // multipole / local coefficients of every box, levels
  float* d_Lall = nullptr;       // concatenated (the levels' d_W / d_L point into these)
  float* d_K = nullptr;          // M2L operators per box offset (343 x n^3 x 4 n^3)
  int4* d_m2l_items = nullptr;   // (offset, first entry, entries, level)
  int n_m2l_items = 0;
  int* d_ent_src = nullptr;      // M2L entries: global source box
  int* d_ent_out = nullptr;      //   and output row (global list position)
  float* d_part = nullptr;       // per-pair M2L results
  int* d_gptr = nullptr;         // list positions of every box (CSR over all levels)
  float* d_lvl_scale = nullptr;  // 1 / box size per level
  float4* d_xloc = nullptr;      // rows local to their leaf centre
  float4* d_ppos = nullptr;      // points local to their leaf centre (C nq)
  float4* d_pstr = nullptr;      // point strengths of the current product (C nq)
  double* d_geo = nullptr;       // panel centre and diameter (C x 4)
  int* d_close_ptr = nullptr;    // close pairs per row (CSR)
  int* d_pair_row = nullptr;
  int* d_pair_pan = nullptr;
  double* d_close_val = nullptr; // FP64 corrections, 8 per close pair
  size_t npairs = 0;
  int* d_plist = nullptr;        // close pairs, the regular ones first, then the singular ones
  size_t n_regular = 0;
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
  // (the margin only shrinks with depth: lm is the deepest level it allows)
  int lm = kFmaMinLevel - 1;
  for (int l = kFmaMinLevel; l <= 20; ++l) {
    if ((kFmaExpand - 1.0) * (S / (double)(1 << l)) / 2.0 < rho) break;
    lm = l;
  }
  if (lm < kFmaMinLevel)
    return fail(h, WBEM_ERR_ARG, "FMA: panels too large for an octree of at least two levels");
  // Morton codes at level lm of the rows (ids 0..N-1) and panel centres
  // (ids N + c); the key of a level l <= lm is the code shifted by 3 (lm - l)
  // (floor(q 2^l) = floor(floor(q 2^lm) / 2^(lm - l)))
  const double sm = S / (double)(1 << lm);
  auto code_lm = [&](const double* p) {
    const int mx = (1 << lm) - 1;
    Key3 k{(int)std::floor((p[0] - lo[0]) / sm), (int)std::floor((p[1] - lo[1]) / sm),
           (int)std::floor((p[2] - lo[2]) / sm)};
    k.x = std::min(std::max(k.x, 0), mx);
    k.y = std::min(std::max(k.y, 0), mx);
    k.z = std::min(std::max(k.z, 0), mx);
    return morton(k);
  };
  std::vector<uint64_t> code(N + (size_t)C);
  std::vector<int> cid(N + (size_t)C);
  for (int i = 0; i < N; ++i) {
    code[i] = code_lm(&Xi[3 * (size_t)i]);
    cid[i] = i;
  }
  for (int c = 0; c < C; ++c) {
    code[N + (size_t)c] = code_lm(&pc[3 * (size_t)c]);
    cid[N + (size_t)c] = N + c;
  }
  int L = kFmaMinLevel;
  {
    std::vector<uint64_t> tc(code.begin(), code.begin() + N);
    std::vector<int> ti(cid.begin(), cid.begin() + N);
    radix_sort_pairs(tc, ti, 3 * lm);
    for (int l = kFmaMinLevel; l <= lm; ++l) {
      const int sh = 3 * (lm - l);
      size_t boxes = N > 0 ? 1 : 0;
      for (int i = 1; i < N; ++i) boxes += (tc[i] >> sh) != (tc[i - 1] >> sh);
      if ((double)N / (double)boxes < 16.0 && l > kFmaMinLevel) break;
      L = l;
    }
  }
  F->L = L;
  const double sL = S / (double)(1 << L);
  // leaves: the distinct codes of rows and panels at level L, in code order;
  // rows and panels of a leaf keep their index order (the sort is stable)
  std::vector<int> tl(N), plf(C);
  std::vector<std::vector<uint64_t>> codes(L + 1);
  for (auto& c : code) c >>= 3 * (lm - L);
  radix_sort_pairs(code, cid, 3 * L);
  for (size_t e = 0; e < code.size(); ++e) {
    if (e == 0 || code[e] != code[e - 1]) codes[L].push_back(code[e]);
    const int b = (int)codes[L].size() - 1;
    if (cid[e] < N) tl[cid[e]] = b;
    else plf[cid[e] - N] = b;
  }
  for (int l = L - 1; l >= 0; --l) codes[l] = coarser_codes(codes[l + 1]);
  std::vector<std::vector<Key3>> keys(L + 1);
  std::vector<BoxIndex> index(L + 1);
  for (int l = 0; l <= L; ++l) {
    keys[l].resize(codes[l].size());
    for (size_t b = 0; b < codes[l].size(); ++b) keys[l][b] = unmorton(codes[l][b]);
    index[l].build(codes[l]);
  }
  F->lev.assign(L + 1, FmaLevel{});
  const int n3 = F->n * F->n * F->n;
  std::vector<int> box_off(L + 2, 0);
  for (int l = 0; l <= L; ++l) box_off[l + 1] = box_off[l] + (int)keys[l].size();
  F->total_boxes = box_off[L + 1];
  WB_CHK(fma_alloc(h, F, &F->d_Wall, (size_t)F->total_boxes * kMpSets * n3));
  WB_CHK(fma_alloc(h, F, &F->d_Lall, (size_t)F->total_boxes * n3));
  // M2L entries of all levels: (level, offset index, source box, list position)
  struct M2LEnt {
    int level, oi, src, out;
  };
  std::vector<M2LEnt> ents;
  std::vector<int> gptr(F->total_boxes + 1, 0);
  std::vector<float> lvl_scale(L + 1);
  int il_off = 0;
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
    V.d_W = F->d_Wall + (size_t)box_off[l] * kMpSets * n3;
    V.d_L = F->d_Lall + (size_t)box_off[l] * n3;
    LevelLinks lk;
    link_level(l, kFmaMinLevel, codes[l], keys[l], l > 0 ? codes[l - 1] : codes[l],
               l > 0 ? &index[l - 1] : nullptr, lk);
    if (l > 0) {
      V.parent = lk.parent;
      V.oct = lk.oct;
      WB_CHK(fma_upload(h, F, &V.d_parent, V.parent));
      WB_CHK(fma_upload(h, F, &V.d_oct, V.oct));
      FmaLevel& P = F->lev[l - 1];
      WB_CHK(fma_upload(h, F, &P.d_child_ptr, lk.cptr));
      WB_CHK(fma_upload(h, F, &P.d_child, lk.ch));
      WB_CHK(fma_upload(h, F, &P.d_child_oct, lk.coct));
    }
    V.il_ptr = lk.il_ptr;
    const std::vector<int>& il = lk.il;
    lvl_scale[l] = (float)(1.0 / s);
    for (int b = 0; b < V.nbox; ++b) {
      const Key3& kt = keys[l][b];
      for (int e = V.il_ptr[b]; e < V.il_ptr[b + 1]; ++e) {
        const Key3& ks = keys[l][il[e]];
        const int oi = ((kt.x - ks.x + 3) * 7 + (kt.y - ks.y + 3)) * 7 + (kt.z - ks.z + 3);
        ents.push_back({l, oi, box_off[l] + il[e], il_off + e});
      }
      gptr[box_off[l] + b + 1] = il_off + V.il_ptr[b + 1];
    }
    il_off += V.il_ptr[V.nbox];
  }
  // M2L work: entries grouped by (level, offset), items of up to kM2LPairs
  std::stable_sort(ents.begin(), ents.end(), [](const M2LEnt& x, const M2LEnt& y) {
    return x.level != y.level ? x.level < y.level : x.oi < y.oi;
  });
  {
    std::vector<int> es(ents.size()), eo(ents.size());
    std::vector<int4> mi;
    for (size_t e = 0; e < ents.size(); ++e) {
      es[e] = ents[e].src;
      eo[e] = ents[e].out;
      const bool head = e == 0 || ents[e].level != ents[e - 1].level || ents[e].oi != ents[e - 1].oi ||
                        mi.back().z == kM2LPairs;
      if (head) mi.push_back(make_int4(ents[e].oi, (int)e, 0, ents[e].level));
      mi.back().z++;
    }
    F->n_m2l_items = (int)mi.size();
    if (mi.empty()) mi.push_back(make_int4(0, 0, 0, 0));
    if (es.empty()) es.push_back(0), eo.push_back(0);
    WB_CHK(fma_upload(h, F, &F->d_m2l_items, mi));
    WB_CHK(fma_upload(h, F, &F->d_ent_src, es));
    WB_CHK(fma_upload(h, F, &F->d_ent_out, eo));
    WB_CHK(fma_upload(h, F, &F->d_gptr, gptr));
    WB_CHK(fma_upload(h, F, &F->d_lvl_scale, lvl_scale));
    WB_CHK(fma_alloc(h, F, &F->d_part, (size_t)std::max(1, il_off) * n3));
    if (!F->d_K) {
      WB_CHK(fma_alloc(h, F, &F->d_K, (size_t)kM2LOffsets * n3 * kMpSets * n3));
      k_fma_m2l_ops<<<dim3(kM2LOffsets, n3), 128, 0, h->stream>>>(F->n, kFmaExpand / 2, F->d_K);
      WB_CU(cudaGetLastError());
    }
  }
  // leaves: panels per leaf, rows per leaf, neighbour leaves
  const FmaLevel& LV = F->lev[L];
  F->nleaf = LV.nbox;
  std::vector<int> pptr(LV.nbox + 1, 0), pan(C), kleaf(C), ppos_of(C);
  for (int c = 0; c < C; ++c) pptr[plf[c] + 1]++;
  for (int b = 0; b < LV.nbox; ++b) pptr[b + 1] += pptr[b];
  {
    std::vector<int> fill(pptr.begin(), pptr.end() - 1);
    for (int c = 0; c < C; ++c) {
      const int lf = plf[c], k = fill[lf]++;
      pan[k] = c;
      kleaf[k] = lf;
      ppos_of[c] = k;
    }
  }
  std::vector<int> tptr(LV.nbox + 1, 0), tidx(N);
  for (int i = 0; i < N; ++i) tptr[tl[i] + 1]++;
  for (int b = 0; b < LV.nbox; ++b) tptr[b + 1] += tptr[b];
  {
    std::vector<int> fill(tptr.begin(), tptr.end() - 1);
    for (int i = 0; i < N; ++i) tidx[fill[tl[i]]++] = i;
  }
  std::vector<int> nbp(LV.nbox + 1, 0), nbl;
  for (int b = 0; b < LV.nbox; ++b) {
    const Key3& k = keys[L][b];
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          const int nbr = index[L].find({k.x + dx, k.y + dy, k.z + dz}, L);
          if (nbr >= 0) nbl.push_back(nbr);
        }
    nbp[b + 1] = (int)nbl.size();
  }
  // evaluation items, the most expensive first: blocks are dispatched in
  // index order as SMs free up, which makes this a longest-first schedule
  std::vector<std::pair<long long, int2>> it_cost;
  for (int b = 0; b < LV.nbox; ++b) {
    long long np = 0;
    for (int e = nbp[b]; e < nbp[b + 1]; ++e) np += pptr[nbl[e] + 1] - pptr[nbl[e]];
    for (int t0 = tptr[b]; t0 < tptr[b + 1]; t0 += kEvalTargets)
      it_cost.push_back({np * std::min(kEvalTargets, tptr[b + 1] - t0), make_int2(b, t0)});
  }
  std::stable_sort(it_cost.begin(), it_cost.end(),
                   [](const auto& x, const auto& y) { return x.first > y.first; });
  std::vector<int2> items;
  for (const auto& c : it_cost) items.push_back(c.second);
  F->n_items = (int)items.size();
  std::vector<int4> p2m_items;
  std::vector<int> p2m_iptr(LV.nbox + 1, 0);
  for (int b = 0; b < LV.nbox; ++b) {
    for (int k0 = pptr[b]; k0 < pptr[b + 1]; k0 += kP2MPanels)
      p2m_items.push_back(make_int4(b, k0, std::min(k0 + kP2MPanels, pptr[b + 1]), 0));
    p2m_iptr[b + 1] = (int)p2m_items.size();
  }
  F->n_p2m_items = (int)p2m_items.size();
  if (p2m_items.empty()) p2m_items.push_back(make_int4(0, 0, 0, 0));
  WB_CHK(fma_upload(h, F, &F->d_p2m_items, p2m_items));
  WB_CHK(fma_upload(h, F, &F->d_p2m_iptr, p2m_iptr));
  WB_CHK(fma_alloc(h, F, &F->d_Wpart,
                   (size_t)std::max(1, F->n_p2m_items) * kMpSets * F->n * F->n * F->n));
  std::vector<float4> xloc(N);
  for (int i = 0; i < N; ++i) {
    const Key3& k = keys[L][tl[i]];
    xloc[i] = make_float4((float)(Xi[3 * (size_t)i] - (lo[0] + (k.x + 0.5) * sL)),
                          (float)(Xi[3 * (size_t)i + 1] - (lo[1] + (k.y + 0.5) * sL)),
                          (float)(Xi[3 * (size_t)i + 2] - (lo[2] + (k.z + 0.5) * sL)), 0.f);
  }
  WB_CHK(fma_upload(h, F, &F->d_leaf_pptr, pptr));
  WB_CHK(fma_upload(h, F, &F->d_leaf_pan, pan));
  WB_CHK(fma_upload(h, F, &F->d_pos_leaf, kleaf));
  WB_CHK(fma_upload(h, F, &F->d_pan_pos, ppos_of));
  WB_CHK(fma_upload(h, F, &F->d_tgt_leaf, tl));
  WB_CHK(fma_upload(h, F, &F->d_tptr, tptr));
  WB_CHK(fma_upload(h, F, &F->d_tidx, tidx));
  WB_CHK(fma_upload(h, F, &F->d_items, items));
  WB_CHK(fma_upload(h, F, &F->d_nb_ptr, nbp));
  if (nbl.empty()) nbl.push_back(0);
  WB_CHK(fma_upload(h, F, &F->d_nb, nbl));
  WB_CHK(fma_upload(h, F, &F->d_xloc, xloc));
  const size_t npts = (size_t)C * F->nq;
  if (npts > 2000000000ull) return fail(h, WBEM_ERR_ARG, "FMA: too many quadrature points");
  WB_CHK(fma_alloc(h, F, &F->d_ppos, npts));
  WB_CHK(fma_alloc(h, F, &F->d_pstr, npts));
  // close pairs: counted and listed on the device
  WB_CHK(fma_alloc(h, F, &F->d_geo, 4 * (size_t)C));
  k_fma_panel_geo<<<(C + 127) / 128, 128, 0, h->stream>>>(C, h->d_X, h->d_cell_dofs, F->d_geo);
  {
    int2 *d_cnt = nullptr, *d_lptr = nullptr;
    DeviceFreeGuard guard{{(void**)&d_cnt, (void**)&d_lptr}};
    WB_CHK(dev_alloc(h, &d_cnt, (size_t)N));
    k_fma_close<<<(N + 127) / 128, 128, 0, h->stream>>>(
        N, F->d_tidx, F->d_tgt_leaf, F->d_nb_ptr, F->d_nb, F->d_leaf_pptr, F->d_leaf_pan, h->d_X, F->d_geo,
        h->d_sptr, h->d_scell, nullptr, nullptr, d_cnt, nullptr, nullptr, nullptr);
    std::vector<int2> cnt(N), lptr(N);
    std::vector<int> cptr(N + 1, 0);
    WB_CU(cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int2) * N, cudaMemcpyDeviceToHost, h->stream));
    WB_CU(cudaStreamSynchronize(h->stream));
    // row offsets of the pairs, and of the correction list: the regular
    // pairs (in pair order) first, then the singular ones (in pair order)
    long long tot = 0, nreg = 0;
    for (int i = 0; i < N; ++i) {
      tot += cnt[i].x;
      if (tot > 2000000000LL) return fail(h, WBEM_ERR_ARG, "FMA: more than 2e9 close pairs");
      cptr[i + 1] = (int)tot;
      lptr[i].x = (int)nreg;
      nreg += cnt[i].x - cnt[i].y;
    }
    for (int i = 0, ns = 0; i < N; ++i) {
      lptr[i].y = (int)nreg + ns;
      ns += cnt[i].y;
    }
    F->npairs = (size_t)tot;
    F->n_regular = (size_t)nreg;
    WB_CHK(fma_upload(h, F, &F->d_close_ptr, cptr));
    WB_CHK(upload(h, &d_lptr, lptr));
    WB_CHK(fma_alloc(h, F, &F->d_pair_row, std::max<size_t>(1, F->npairs)));
    WB_CHK(fma_alloc(h, F, &F->d_pair_pan, std::max<size_t>(1, F->npairs)));
    WB_CHK(fma_alloc(h, F, &F->d_close_val, 8 * std::max<size_t>(1, F->npairs)));
    WB_CHK(fma_alloc(h, F, &F->d_plist, std::max<size_t>(1, F->npairs)));
    k_fma_close<<<(N + 127) / 128, 128, 0, h->stream>>>(
        N, F->d_tidx, F->d_tgt_leaf, F->d_nb_ptr, F->d_nb, F->d_leaf_pptr, F->d_leaf_pan, h->d_X, F->d_geo,
        h->d_sptr, h->d_scell, F->d_close_ptr, d_lptr, nullptr, F->d_pair_row, F->d_pair_pan,
        F->d_plist);
    WB_CU(cudaGetLastError());
    // d_lptr is freed on return: the list pass must have read it
    WB_CU(cudaStreamSynchronize(h->stream));
  }
  const int n = F->n;
  std::vector<double> t(n);
  for (int k = 0; k < n; ++k) t[k] = std::cos((2 * k + 1) * 3.14159265358979323846 / (2.0 * n));
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
  // child -> parent interpolation (level-independent: the interpolation
  // cubes scale with the boxes): child node c of the lower / upper half in
  // parent cube coordinates is -+1/(2 e) + t_c / 2
  std::vector<double> S1(n);
  for (int hf = 0; hf < 2; ++hf)
    for (int c = 0; c < n; ++c) {
      cheb_weights_host(n, (hf ? 1.0 : -1.0) / (2 * kFmaExpand) + t[c] / 2, t, S1.data());
      for (int P = 0; P < n; ++P) fc.S1[hf][c][P] = (float)S1[P];
    }
  return WBEM_OK;
}

// y = N a + D b with the FMA (a, b, y device vectors, internal order).
static int fma_product(wbem_context* h, const double* a, const double* b, double* y) {
  FmaState* F = static_cast<FmaState*>(h->fma_state);
  const int C = h->C, L = F->L, n3 = F->n * F->n * F->n;
  const int nt = (n3 + 31) / 32 * 32;
  cudaStream_t s = h->stream;
  FmaLevel& LV = F->lev[L];
  const int npts = C * F->nq;
  k_fma_strengths<<<(npts + 255) / 256, 256, 0, s>>>(npts, F->d_leaf_pan, h->d_rec, h->d_cell_dofs,
                                                    a, b, F->d_pstr, F->cst);
  if (F->n_p2m_items > 0) {
    const dim3 pb(kP2MGroupThreads, kP2MGroups);
    const int ni = F->n_p2m_items;
    switch (F->n) {
      case 3: k_fma_p2m<3><<<ni, pb, 0, s>>>(F->d_p2m_items, F->d_ppos, F->d_pstr, LV.half, F->d_Wpart, F->cst); break;
      case 4: k_fma_p2m<4><<<ni, pb, 0, s>>>(F->d_p2m_items, F->d_ppos, F->d_pstr, LV.half, F->d_Wpart, F->cst); break;
      case 5: k_fma_p2m<5><<<ni, pb, 0, s>>>(F->d_p2m_items, F->d_ppos, F->d_pstr, LV.half, F->d_Wpart, F->cst); break;
      case 6: k_fma_p2m<6><<<ni, pb, 0, s>>>(F->d_p2m_items, F->d_ppos, F->d_pstr, LV.half, F->d_Wpart, F->cst); break;
      case 7: k_fma_p2m<7><<<ni, pb, 0, s>>>(F->d_p2m_items, F->d_ppos, F->d_pstr, LV.half, F->d_Wpart, F->cst); break;
      default: k_fma_p2m<8><<<ni, pb, 0, s>>>(F->d_p2m_items, F->d_ppos, F->d_pstr, LV.half, F->d_Wpart, F->cst); break;
    }
  }
  k_fma_p2m_sum<<<LV.nbox, 256, 0, s>>>(F->d_p2m_iptr, F->d_Wpart, LV.d_W, kMpSets * n3);
  for (int l = L; l > kFmaMinLevel; --l) {
    FmaLevel& P = F->lev[l - 1];
    k_fma_m2m<<<P.nbox, nt, 0, s>>>(P.d_child_ptr, P.d_child, P.d_child_oct, F->lev[l].d_W, P.d_W,
                                    F->cst);
  }
  if (F->n_m2l_items > 0)
    k_fma_m2l_gemm<<<F->n_m2l_items, 256, 0, s>>>(F->d_m2l_items, F->d_ent_src, F->d_ent_out, F->d_K,
                                                  F->d_Wall, F->d_lvl_scale, F->d_part, n3);
  k_fma_m2l_sum<<<F->total_boxes, nt, 0, s>>>(F->d_gptr, F->d_part, F->d_Lall, n3);
  for (int l = kFmaMinLevel + 1; l <= L; ++l) {
    FmaLevel& V = F->lev[l];
    k_fma_l2l<<<V.nbox, nt, 0, s>>>(V.d_parent, V.d_oct, F->lev[l - 1].d_L, V.d_L, F->cst);
  }
  k_fma_eval<<<F->n_items, kEvalThreads, 0, s>>>(
      F->d_items, F->d_tptr, F->d_tidx, F->d_xloc, F->d_nb_ptr, F->d_nb, F->d_leaf_pptr, LV.d_cen,
      LV.half, L >= kFmaMinLevel ? LV.d_L : nullptr, F->d_ppos, F->d_pstr, F->d_close_ptr,
      F->d_pair_pan, F->d_close_val, h->d_cell_dofs, a, b, y, F->cst);
  h->launches += 6 + 2 * (L - kFmaMinLevel);
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
  k_fma_near_blocks<<<(N + 127) / 128, 128, 0, h->stream>>>(
      N, F->d_tgt_leaf, F->d_nb_ptr, F->d_nb, F->d_leaf_pptr, F->d_leaf_pan, F->lev[F->L].d_cen,
      F->d_xloc, F->d_ppos, h->d_rec, F->d_close_ptr, F->d_pair_pan, F->d_close_val,
      h->d_cell_dofs, h->d_mask, h->d_alpha, F->d_blocks, F->cst);
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
  const int nq = qt.q1 * qt.q1;
  FmaState* F = static_cast<FmaState*>(h->fma_state);
  if (!F || F->n != n || F->nq != nq || h->fma_geometry_stale) {
    // the M2L operators depend on the order alone: a rebuild for moved
    // nodes keeps them
    float* keep_K = nullptr;
    if (F && F->n == n && F->d_K) {
      const auto it = std::find(F->owned.begin(), F->owned.end(), (void*)F->d_K);
      if (it != F->owned.end()) {
        keep_K = F->d_K;
        F->owned.erase(it);
      }
    }
    free_fma(h);
    F = new FmaState();
    F->n = n;
    F->nq = nq;
    if (keep_K) {
      F->d_K = keep_K;
      F->owned.push_back(keep_K);
    }
    h->fma_state = F;
    const auto t0 = std::chrono::steady_clock::now();
    const int st = fma_build(h, F, qt);
    if (st != WBEM_OK) {
      free_fma(h);
      return st;
    }
    h->stats.t_assemble_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    h->fma_geometry_stale = false;
  } else {
    h->stats.t_assemble_ms = 0.0;  // the tree and lists of the last build still hold
  }
  if (h->rec_cells != (size_t)C * nq || !h->d_rec) {
    WB_CHK(dev_alloc(h, &h->d_rec, (size_t)C * nq * 8));
    h->rec_cells = (size_t)C * nq;
  }
  if (!h->d_alpha) WB_CHK(dev_alloc(h, &h->d_alpha, (size_t)N));
  EvTimer tm(h->stream);
  WB_CU(launch_cell_records_fp64(C, h->d_X, h->d_cell_dofs, h->d_rec, qt.q1, h->stream));
  h->stats.t_geometry_ms = tm.ms();
  const int npts = C * nq;
  k_fma_points<<<(npts + 255) / 256, 256, 0, h->stream>>>(npts, nq, F->d_leaf_pan, F->d_pos_leaf,
                                                          h->d_rec, F->lev[F->L].d_cen, F->d_ppos);
  // the regular pairs, then the singular ones (each list warp-uniform)
  for (int part = 0; part < 2; ++part) {
    const size_t off = part ? F->n_regular : 0;
    const size_t cnt = part ? F->npairs - F->n_regular : F->n_regular;
    if (cnt == 0) continue;
    k_fma_close_val<<<(unsigned)((cnt + 127) / 128), 128, 0, h->stream>>>(
        (long long)cnt, F->d_plist + off, F->d_pair_row, F->d_pair_pan, h->d_X, h->d_dnset,
        h->d_cell_dofs, h->d_rec, F->d_tgt_leaf, F->d_pan_pos, F->d_pos_leaf, F->lev[F->L].d_cen,
        F->d_xloc, F->d_ppos, F->d_close_val, F->d_qt, F->cst);
    WB_CU(cudaGetLastError());
    h->launches++;
  }
  h->stats.t_singular_ms = tm.ms();
  WB_CHK(fma_apply(h, 2, nullptr, h->d_alpha));
  h->stats.t_alpha_ms = tm.ms();
  h->launches += 2;
  return check_device_error(h, "assemble (FMA)");
}

}  // namespace wbem
