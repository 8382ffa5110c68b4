// Hull force evaluation and the hand-written adjoint of
// assemble_system + solve_system + hull force.
//
// With x the unknowns (phi on Neumann nodes, dphi/dn on Dirichlet nodes), b
// the known data (tmp_rhs) and G(x, b, X) = 0 the constrained collocation
// system, the force F(X, phi, dphi/dn) has
//     dF/dX = dF/dX|direct - lambda^T dG/dX,     A^T lambda = dF/dx,
//     dF/db = dF/db|direct - lambda^T dG/db.
// Row i of the unconstrained system is (source/bem_problem.cc:620-706 with
// alpha_i = -sum_j N_ij, :594-618)
//     R_i = sum_panels sum_q w_q [ DL(x_q - x_i, c_q) (phi(q) - phi_i) - SL(x_q - x_i) |c_q| dphi(q) ]
// with c_q the (unnormalised) cross product of the Q1 map, so lambda^T dR/dX
// is obtained by recomputing every (row, panel, point) term with its
// derivatives with respect to the collocation point and the 4 panel vertices
// (k_adj_tile, k_adj_singular): no dG/dX is stored. The transposed solve
// reuses the LU factors (mixed form) or the block-Jacobi blocks (FP64 form).
// Constraint inhomogeneities are taken as functions of b only (exact for the
// Dirichlet-Neumann and Neumann-Neumann double nodes of the tank meshes).
#include <cuda_runtime.h>
#include <algorithm>
#include <vector>
#include "context.h"
#include "host_util.h"
#include "kernels.h"

namespace wbem {
cudaError_t upload_quadrature_force(const QuadTables& t);
static __constant__ QuadTables c_qa;
cudaError_t upload_quadrature_adjoint(const QuadTables& t) {
  cudaError_t e = cudaMemcpyToSymbol(c_qa, &t, sizeof(QuadTables));
  if (e != cudaSuccess) return e;
  return upload_quadrature_force(t);
}
int ensure_vectors(wbem_context* h, int restart);
int solve_assembled(wbem_context* h, const double* rhs, double* x, int transpose);

constexpr double kI4P = 0.07957747154594766788;

static int hull_dofs_upload(wbem_context* h, const int* hull_cells, int n_hull, int4** out,
                            std::vector<int>* cell_ids = nullptr) {
  std::vector<int4> hd(n_hull > 0 ? n_hull : 1);
  for (int k = 0; k < n_hull; ++k) {
    const int c = hull_cells[k];
    if (c < 0 || c >= h->C) return fail(h, WBEM_ERR_ARG, "hull cell index out of range");
    const int* v = &h->cells[4 * (size_t)c];
    hd[k] = make_int4(h->iperm[v[0]], h->iperm[v[1]], h->iperm[v[2]], h->iperm[v[3]]);
    if (cell_ids) cell_ids->push_back(c);
  }
  WB_CU(cudaMalloc(out, sizeof(int4) * hd.size()));
  WB_CU(cudaMemcpyAsync(*out, hd.data(), sizeof(int4) * hd.size(), cudaMemcpyHostToDevice, h->stream));
  WB_CU(cudaStreamSynchronize(h->stream));
  return WBEM_OK;
}

int hull_force_dev(wbem_context* h, const int* hull_cells, int n_hull, const double* U, int dir,
                   const double* d_phi, const double* d_dphi, double* force) {
  int4* hd = nullptr;
  double* part = nullptr;
  DeviceFreeGuard scratch{{reinterpret_cast<void**>(&hd), reinterpret_cast<void**>(&part)}};
  WB_CHK(hull_dofs_upload(h, hull_cells, n_hull, &hd));
  cudaError_t e = cudaMalloc(&part, sizeof(double) * (n_hull + 1));
  if (e == cudaSuccess) e = launch_hull_force(n_hull, hd, h->d_X, U, dir, d_phi, d_dphi, part, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(force, part + n_hull, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return fail(h, WBEM_ERR_CUDA, cudaGetErrorString(e));
  return WBEM_OK;
}

// ------------------------------------------------------------ K7: panel terms
__device__ __forceinline__ bool near_test_a(float xi, float yi, float zi, float4 g) {
  const float dx = __fsub_rn(g.x, xi), dy = __fsub_rn(g.y, yi), dz = __fsub_rn(g.z, zi);
  const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  return d2 < g.w;
}

// Derivatives of f = w' lam [ -(R.c)/r^3 dphi - |c|/r dn ] (w' = w/(4 pi)):
//   df/dR = -s1 c / r^3 + (3 s1 (R.c) / r^5 + s2 |c| / r^3) R
//   df/dc = -s1 R / r^3 - (s2 / (|c| r)) c
// with s1 = w' lam dphi, s2 = w' lam dn.
template <typename T>
__device__ __forceinline__ void point_grad(const T R[3], const T c[3], T J, T s1, T s2, T aR[3],
                                           T ac[3]) {
  const T r2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
  T ri;
  if constexpr (sizeof(T) == 8) ri = rsqrt(r2);
  else ri = rsqrtf(r2);
  const T ri3 = ri * ri * ri;
  const T ri5 = ri3 * ri * ri;
  const T u = R[0] * c[0] + R[1] * c[1] + R[2] * c[2];
  const T kr = 3 * s1 * u * ri5 + s2 * J * ri3;
  const T kc = s2 * ri / J;
  for (int d = 0; d < 3; ++d) {
    aR[d] = -s1 * ri3 * c[d] + kr * R[d];
    ac[d] = -s1 * ri3 * R[d] - kc * c[d];
  }
}

// smem point data per panel and point: x (3), jx (3), je (3), |c|, w'phi(q), w'dn(q)
constexpr int kAdjChunk = 8;
constexpr int kPt = 12;

// FP64 point data of regular point q of the panel with dofs d (layout above).
__device__ __forceinline__ void adj_point(const double* __restrict__ X, int4 d, int q,
                                          const double* __restrict__ phi,
                                          const double* __restrict__ dn, double* p) {
  const int id[4] = {d.x, d.y, d.z, d.w};
  const double s = c_qa.gp[q][0], u = c_qa.gp[q][1], w = c_qa.gp[q][2] * kI4P;
  const double Ns[4] = {-(1 - u), (1 - u), -u, u};
  const double Nt[4] = {-(1 - s), -s, (1 - s), s};
  double x[3] = {0, 0, 0}, jx[3] = {0, 0, 0}, je[3] = {0, 0, 0}, fp = 0, fn = 0;
  for (int v = 0; v < 4; ++v) {
    const double nv = c_qa.phi[q][v];
    for (int e = 0; e < 3; ++e) {
      const double P = X[3 * (size_t)id[v] + e];
      x[e] += nv * P;
      jx[e] += Ns[v] * P;
      je[e] += Nt[v] * P;
    }
    fp += nv * phi[id[v]];
    fn += nv * dn[id[v]];
  }
  for (int e = 0; e < 3; ++e) {
    p[e] = x[e];
    p[3 + e] = jx[e];
    p[6 + e] = je[e];
  }
  const double cr0 = jx[1] * je[2] - jx[2] * je[1], cr1 = jx[2] * je[0] - jx[0] * je[2],
               cr2 = jx[0] * je[1] - jx[1] * je[0];
  p[9] = sqrt(cr0 * cr0 + cr1 * cr1 + cr2 * cr2);
  p[10] = w * fp;
  p[11] = w * fn;
}

// FP64 terms of one (row, regular point) pair: row part into grow, the 4
// panel-vertex parts into g (vertex v, component e at 3 v + e).
__device__ __forceinline__ void adj_point_terms(const double* p, int q, const double xi[3],
                                                double li, double phii, double g[12],
                                                double grow[3]) {
  const double R[3] = {p[0] - xi[0], p[1] - xi[1], p[2] - xi[2]};
  const double c[3] = {p[4] * p[8] - p[5] * p[7], p[5] * p[6] - p[3] * p[8],
                       p[3] * p[7] - p[4] * p[6]};
  const double w = c_qa.gp[q][2] * kI4P;
  const double s1 = li * (p[10] - w * phii), s2 = li * p[11];
  double aR[3], ac[3];
  point_grad<double>(R, c, p[9], s1, s2, aR, ac);
  const double s = c_qa.gp[q][0], u = c_qa.gp[q][1];
  const double Ns[4] = {-(1 - u), (1 - u), -u, u};
  const double Nt[4] = {-(1 - s), -s, (1 - s), s};
  const double gjx[3] = {p[7] * ac[2] - p[8] * ac[1], p[8] * ac[0] - p[6] * ac[2],
                         p[6] * ac[1] - p[7] * ac[0]};
  const double gje[3] = {ac[1] * p[5] - ac[2] * p[4], ac[2] * p[3] - ac[0] * p[5],
                         ac[0] * p[4] - ac[1] * p[3]};
  for (int e = 0; e < 3; ++e) grow[e] -= aR[e];
  for (int v = 0; v < 4; ++v)
    for (int e = 0; e < 3; ++e)
      g[3 * v + e] += c_qa.phi[q][v] * aR[e] + Ns[v] * gjx[e] + Nt[v] * gje[e];
}

// FP64 terms of one near (row, regular point) pair of the mixed form, in the
// moment form of the far field (B_v += N4_v aR, D_v += N4_v ac, row part into
// grow). p: x (3), c = jx x je (3), w'phi(q), w'dn(q) |c|, w'dn(q) / |c|;
// lpw = lambda_i phi_i / (4 pi).
__device__ __forceinline__ void adj_near_moments(const double* __restrict__ p, int q,
                                                 const double xi[3], double li, double lpw,
                                                 double B[12], double D[12], double grow[3]) {
  const double R[3] = {p[0] - xi[0], p[1] - xi[1], p[2] - xi[2]};
  const double c[3] = {p[3], p[4], p[5]};
  const double r2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
  const double ri = rsqrt(r2), ri2 = ri * ri, ri3 = ri2 * ri;
  const double u = R[0] * c[0] + R[1] * c[1] + R[2] * c[2];
  const double s1 = li * p[6] - lpw * c_qa.gp[q][2];
  const double a = s1 * ri3;
  const double kr = 3.0 * s1 * u * ri3 * ri2 + li * p[7] * ri3;
  const double kc = li * p[8] * ri;
  double aR[3], ac[3];
  for (int e = 0; e < 3; ++e) {
    aR[e] = kr * R[e] - a * c[e];
    ac[e] = -a * R[e] - kc * c[e];
    grow[e] -= aR[e];
  }
  for (int v = 0; v < 4; ++v) {
    const double nv = c_qa.phi[q][v];
    for (int e = 0; e < 3; ++e) {
      B[3 * v + e] += nv * aR[e];
      D[3 * v + e] += nv * ac[e];
    }
  }
}

// Plain form. One CTA: 128 rows x a range of panels, FP64 throughout.
template <int Q1>
__global__ void __launch_bounds__(128)
    k_adj_tile(int N, int C, const double* __restrict__ X, const int* __restrict__ dnset,
               const int4* __restrict__ cell_dofs, const double* __restrict__ lam,
               const double* __restrict__ phi, const double* __restrict__ dn,
               double* __restrict__ grow_part, double* __restrict__ gcell_part,
               int cells_per_block) {
  constexpr int NQ = Q1 * Q1;
  __shared__ double pt[kAdjChunk][NQ][kPt];
  __shared__ double wred[4][kAdjChunk][12];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row = blockIdx.y * 128 + tid;
  const bool active = row < N;
  double xi[3] = {0, 0, 0}, li = 0, phii = 0;
  int set[kMaxSet];
  for (int k = 0; k < kMaxSet; ++k) set[k] = -2;
  if (active) {
    for (int d = 0; d < 3; ++d) xi[d] = X[3 * (size_t)row + d];
    li = lam[row];
    phii = phi[row];
    for (int k = 0; k < kMaxSet; ++k) set[k] = dnset[(size_t)row * kMaxSet + k];
  }
  double grow[3] = {0, 0, 0};
  const int c_begin = blockIdx.x * cells_per_block;
  const int c_end = min(C, c_begin + cells_per_block);
  for (int cb = c_begin; cb < c_end; cb += kAdjChunk) {
    const int cnt = min(kAdjChunk, c_end - cb);
    __syncthreads();
    for (int t = tid; t < cnt * NQ; t += 128) {
      const int k = t / NQ, q = t % NQ;
      adj_point(X, cell_dofs[cb + k], q, phi, dn, pt[k][q]);
    }
    __syncthreads();
    for (int k = 0; k < cnt; ++k) {
      const int4 d = cell_dofs[cb + k];
      bool sing = false;
      for (int s = 0; s < kMaxSet; ++s)
        sing |= (set[s] == d.x) | (set[s] == d.y) | (set[s] == d.z) | (set[s] == d.w);
      double g[12];
      for (int t = 0; t < 12; ++t) g[t] = 0;
      if (active && !sing && li != 0.0)
        for (int q = 0; q < NQ; ++q) adj_point_terms(pt[k][q], q, xi, li, phii, g, grow);
      // sum the 12 panel-vertex terms over the 32 rows of the warp
      for (int t = 0; t < 12; ++t) {
        double v = g[t];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) wred[warp][k][t] = v;
      }
    }
    __syncthreads();
    for (int t = tid; t < cnt * 12; t += 128) {
      const int k = t / 12, e = t % 12;
      const double v = wred[0][k][e] + wred[1][k][e] + wred[2][k][e] + wred[3][k][e];
      gcell_part[((size_t)blockIdx.y * C + cb + k) * 12 + e] = v;
    }
  }
  if (active)
    for (int e = 0; e < 3; ++e) grow_part[((size_t)blockIdx.x * N + row) * 3 + e] = grow[e];
}

// ---------------------------------------------------- mixed form (K7 mixed)
// Far pairs (panels that fail the assembly's near test) run in FP32, near
// pairs in FP64, singular pairs in k_adj_singular.
//
// The far-field sum over the regular points q of one panel is kept in the
// bilinear basis N4_v(q) of the panel:
//     B_v = sum_q N4_v aR_q,   D_v = sum_q N4_v ac_q      (v = 0..3)
// with aR, ac the derivatives with respect to the point offset R and the
// cross product c (point_grad). Since jx = (1-u) F0 + u F1 and
// je = (1-s) E0 + s E1 (F0 = P1-P0, F1 = P3-P2, E0 = P2-P0, E1 = P3-P1),
// the vertex gradients sum_q [N4_v aR + Ns_v (je x ac) + Nt_v (ac x jx)] are
//     g0 = B0 - X01 - Y02,  g1 = B1 + X01 - Y13,
//     g2 = B2 - X23 + Y02,  g3 = B3 + X23 + Y13,
//     X01 = E0 x D0 + E1 x D1,  X23 = E0 x D2 + E1 x D3,
//     Y02 = D0 x F0 + D2 x F1,  Y13 = D1 x F0 + D3 x F1.
// B and D are linear in the rows, so each thread sums them over its rows,
// the warp reduces them once per panel and the cross products are taken
// once per (CTA, panel) in FP64.
constexpr int kAdjRpt = 4;                  // rows per thread: r0 + 128 j + tid, j < kAdjRpt
constexpr int kAdjRowsCta = 128 * kAdjRpt;  // rows per CTA
static_assert(kMaxSet % 4 == 0, "double-node sets are read as int4");
static_assert(kAdjRpt * kAdjChunk <= 32, "near mask of a chunk in one word");

// Per (panel, regular point), once per adjoint call:
//   recd (12 doubles): x, c = jx x je, w'phi, w'dn |c|, w'dn / |c| (near pairs);
//   recf (3 float4):   (x_hi, c.x), (x_lo, c.y), (c.z, w'phi, w'dn |c|, w'dn / |c|)
//                      with x = x_hi + x_lo and c = jx x je;
// per panel pgeo (12 doubles): E0, E1, F0, F1.
template <int Q1>
__global__ void k_adj_points(int C, const double* __restrict__ X,
                             const int4* __restrict__ cell_dofs, const double* __restrict__ phi,
                             const double* __restrict__ dn, double* __restrict__ recd,
                             float4* __restrict__ recf, double* __restrict__ pgeo) {
  constexpr int NQ = Q1 * Q1;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= C * NQ) return;
  const int cell = t / NQ, q = t - cell * NQ;
  const int4 d = cell_dofs[cell];
  double p[kPt];
  adj_point(X, d, q, phi, dn, p);
  const double c0 = p[4] * p[8] - p[5] * p[7], c1 = p[5] * p[6] - p[3] * p[8],
               c2 = p[3] * p[7] - p[4] * p[6];
  const double rd[kPt] = {p[0], p[1], p[2], c0, c1, c2, p[10], p[11] * p[9], p[11] / p[9], 0.0, 0.0, 0.0};
  double* pd = recd + (size_t)t * kPt;
  for (int e = 0; e < kPt; ++e) pd[e] = rd[e];
  float hi[3], lo[3];
  for (int e = 0; e < 3; ++e) {
    hi[e] = (float)p[e];
    lo[e] = (float)(p[e] - (double)hi[e]);
  }
  recf[3 * (size_t)t + 0] = make_float4(hi[0], hi[1], hi[2], (float)c0);
  recf[3 * (size_t)t + 1] = make_float4(lo[0], lo[1], lo[2], (float)c1);
  recf[3 * (size_t)t + 2] =
      make_float4((float)c2, (float)p[10], (float)(p[11] * p[9]), (float)(p[11] / p[9]));
  if (q == 0) {
    const int id[4] = {d.x, d.y, d.z, d.w};
    double P[4][3];
    for (int v = 0; v < 4; ++v)
      for (int e = 0; e < 3; ++e) P[v][e] = X[3 * (size_t)id[v] + e];
    double* g = pgeo + (size_t)cell * 12;
    for (int e = 0; e < 3; ++e) {
      g[e] = P[2][e] - P[0][e];
      g[3 + e] = P[3][e] - P[1][e];
      g[6 + e] = P[1][e] - P[0][e];
      g[9 + e] = P[3][e] - P[2][e];
    }
  }
}

// Sum of v[0..23] over the 32 lanes of the warp by reduce-scatter (27
// shuffles): lane l returns the sums of v[3 (l >> 2) + i], i = 0..2.
template <typename T>
__device__ __forceinline__ void warp_sum24(const T v[24], int lane, T out[3]) {
  const bool h1 = lane & 16, h2 = lane & 8, h3 = lane & 4;
  T w[12], x[6];
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    const T keep = h1 ? v[12 + i] : v[i], send = h1 ? v[i] : v[12 + i];
    w[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const T keep = h2 ? w[6 + i] : w[i], send = h2 ? w[i] : w[6 + i];
    x[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const T keep = h3 ? x[3 + i] : x[i], send = h3 ? x[i] : x[3 + i];
    T y = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    y += __shfl_xor_sync(0xffffffffu, y, 2);
    y += __shfl_xor_sync(0xffffffffu, y, 1);
    out[i] = y;
  }
}

// One CTA: kAdjRowsCta consecutive rows (kAdjRpt per thread, 128 apart, so
// that the near rows of a panel fall on different lanes) x a range of panels,
// in chunks of kAdjChunk panels whose FP32 point data (offsets from the CTA's
// first row, so that the FP32 differences stay accurate) sit in shared memory.
// Near pairs add their FP64 moments to the same per-panel sums.
template <int Q1>
__global__ void __launch_bounds__(128, 4)
    k_adj_tile_mixed(int N, int C, const double* __restrict__ X, const int* __restrict__ dnset,
                     const int4* __restrict__ cell_dofs, const float4* __restrict__ cellgeo,
                     const float4* __restrict__ recf, const double* __restrict__ recd,
                     const double* __restrict__ pgeo, const double* __restrict__ lam,
                     const double* __restrict__ phi, double* __restrict__ grow_part,
                     double* __restrict__ gcell_part, int cells_per_block) {
  constexpr int NQ = Q1 * Q1;
  __shared__ __align__(16) float sp[kAdjChunk][NQ][12];
  __shared__ float wmom[4][kAdjChunk][24];
  __shared__ double wnmom[4][kAdjChunk][24];  // near-pair moments per warp
  __shared__ double smom[kAdjChunk][24];
  __shared__ double sgrow[kAdjRpt][3][128];
  __shared__ float sxf[kAdjRpt][3][128];
  __shared__ int4 sdofs[kAdjChunk];
  __shared__ float4 sgeo[kAdjChunk];
  __shared__ double cTd[3];
  __shared__ float cTs[6];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = blockIdx.y * kAdjRowsCta;
  if (tid < 3) {
    const double c = X[3 * (size_t)r0 + tid];
    const float hi = (float)c;
    cTd[tid] = c;
    cTs[tid] = hi;
    cTs[3 + tid] = (float)(c - (double)hi);
  }
  __syncthreads();
  float xr[kAdjRpt][3], lf[kAdjRpt], lpf[kAdjRpt];
  unsigned live = 0;
#pragma unroll
  for (int j = 0; j < kAdjRpt; ++j) {
    const int row = r0 + 128 * j + tid;
    double x[3] = {cTd[0], cTd[1], cTd[2]}, li = 0, ph = 0;
    if (row < N) {
      for (int e = 0; e < 3; ++e) x[e] = X[3 * (size_t)row + e];
      li = lam[row];
      ph = phi[row];
      if (li != 0.0) live |= 1u << j;
    }
    for (int e = 0; e < 3; ++e) {
      xr[j][e] = (float)(x[e] - cTd[e]);
      sxf[j][e][tid] = (float)x[e];
      sgrow[j][e][tid] = 0.0;
    }
    lf[j] = (float)li;
    lpf[j] = (float)(li * ph * kI4P);
  }
  const int c_begin = blockIdx.x * cells_per_block;
  const int c_end = min(C, c_begin + cells_per_block);
  for (int cb = c_begin; cb < c_end; cb += kAdjChunk) {
    const int cnt = min(kAdjChunk, c_end - cb);
    __syncthreads();
    for (int t = tid; t < cnt * NQ; t += 128) {
      const float4* r = recf + 3 * ((size_t)cb * NQ + t);
      const float4 a = r[0], b = r[1], c = r[2];
      float* s = &sp[0][0][0] + 12 * t;
      s[0] = (a.x - cTs[0]) + (b.x - cTs[3]);
      s[1] = (a.y - cTs[1]) + (b.y - cTs[4]);
      s[2] = (a.z - cTs[2]) + (b.z - cTs[5]);
      s[3] = a.w;
      s[4] = b.w;
      s[5] = c.x;
      s[6] = c.y;
      s[7] = c.z;
      s[8] = c.w;
    }
    if (tid < cnt) {
      sdofs[tid] = cell_dofs[cb + tid];
      sgeo[tid] = cellgeo[cb + tid];
    }
    __syncthreads();
    float gr[kAdjRpt][3];
#pragma unroll
    for (int j = 0; j < kAdjRpt; ++j) gr[j][0] = gr[j][1] = gr[j][2] = 0.f;
    unsigned nmask = 0;  // near (row j, panel k) pairs of the chunk at bit kAdjRpt k + j
    for (int k = 0; k < cnt; ++k) {
      const float4 g = sgeo[k];
      bool far[kAdjRpt];
      float lk[kAdjRpt], lpk[kAdjRpt];
#pragma unroll
      for (int j = 0; j < kAdjRpt; ++j) {
        const bool nt = near_test_a(sxf[j][0][tid], sxf[j][1][tid], sxf[j][2][tid], g);
        const bool lv = (live >> j) & 1u;
        far[j] = lv && !nt;
        if (lv && nt) nmask |= 1u << (kAdjRpt * k + j);
        lk[j] = far[j] ? lf[j] : 0.f;
        lpk[j] = far[j] ? lpf[j] : 0.f;
      }
      float v[24];
#pragma unroll
      for (int i = 0; i < 24; ++i) v[i] = 0.f;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const float* p = sp[k][q];
        const float4 A = *reinterpret_cast<const float4*>(p);
        const float4 B = *reinterpret_cast<const float4*>(p + 4);
        const float wnoj = p[8];
        const float c[3] = {A.w, B.x, B.y};
        const float gw = c_qa.gpf[q][2];
        float aR[3] = {0.f, 0.f, 0.f}, ac[3] = {0.f, 0.f, 0.f}, Ks = 0.f, Kc = 0.f;
#pragma unroll
        for (int j = 0; j < kAdjRpt; ++j) {
          const float R[3] = {A.x - xr[j][0], A.y - xr[j][1], A.z - xr[j][2]};
          float r2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
          r2 = far[j] ? r2 : 1.f;
          const float ri = rsqrtf(r2), ri2 = ri * ri, ri3 = ri2 * ri;
          const float u = R[0] * c[0] + R[1] * c[1] + R[2] * c[2];
          const float s1 = fmaf(lk[j], B.z, -lpk[j] * gw);
          const float a = s1 * ri3;
          const float kr = fmaf(s1 * u, ri3 * (3.f * ri2), (lk[j] * B.w) * ri3);
          const float kc = (lk[j] * wnoj) * ri;
          Ks += a;
          Kc += kc;
#pragma unroll
          for (int e = 0; e < 3; ++e) {
            aR[e] = fmaf(kr, R[e], aR[e]);
            ac[e] = fmaf(-a, R[e], ac[e]);
            gr[j][e] = fmaf(kr, R[e], fmaf(-a, c[e], gr[j][e]));
          }
        }
#pragma unroll
        for (int e = 0; e < 3; ++e) {
          aR[e] = fmaf(-Ks, c[e], aR[e]);
          ac[e] = fmaf(-Kc, c[e], ac[e]);
        }
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          const float nv = c_qa.phif[q][w];
#pragma unroll
          for (int e = 0; e < 3; ++e) {
            v[3 * w + e] = fmaf(nv, aR[e], v[3 * w + e]);
            v[12 + 3 * w + e] = fmaf(nv, ac[e], v[12 + 3 * w + e]);
          }
        }
      }
      float o3[3];
      warp_sum24<float>(v, lane, o3);
      if ((lane & 3) == 0)
        for (int i = 0; i < 3; ++i) wmom[warp][k][3 * (lane >> 2) + i] = o3[i];
    }
#pragma unroll
    for (int j = 0; j < kAdjRpt; ++j)
      for (int e = 0; e < 3; ++e) sgrow[j][e][tid] -= (double)gr[j][e];
    // near pairs of the chunk: FP64 terms, unless the pair is singular
    for (int k = 0; k < cnt; ++k) {
      unsigned nm = (nmask >> (kAdjRpt * k)) & ((1u << kAdjRpt) - 1u);
      if (__any_sync(0xffffffffu, nm != 0u)) {
        double m64[24];
        for (int t = 0; t < 24; ++t) m64[t] = 0.0;
        const int4 d = sdofs[k];
        const double* pc = recd + (size_t)(cb + k) * NQ * kPt;
        while (nm) {
          const int j = __ffs(nm) - 1;
          nm &= nm - 1u;
          const int row = r0 + 128 * j + tid;
          const int4* s4 = reinterpret_cast<const int4*>(dnset + (size_t)row * kMaxSet);
          bool sing = false;
          for (int h = 0; h < kMaxSet / 4; ++h) {
            const int4 s = s4[h];
            const int m[4] = {s.x, s.y, s.z, s.w};
            for (int i = 0; i < 4; ++i)
              sing |= (m[i] == d.x) | (m[i] == d.y) | (m[i] == d.z) | (m[i] == d.w);
          }
          if (sing) continue;
          const double xi[3] = {X[3 * (size_t)row], X[3 * (size_t)row + 1], X[3 * (size_t)row + 2]};
          const double li = lam[row], lpw = li * phi[row] * kI4P;
          double grow[3] = {0.0, 0.0, 0.0};
          for (int q = 0; q < NQ; ++q)
            adj_near_moments(pc + q * kPt, q, xi, li, lpw, m64, m64 + 12, grow);
          for (int e = 0; e < 3; ++e) sgrow[j][e][tid] += grow[e];
        }
        double n3[3];
        warp_sum24<double>(m64, lane, n3);
        if ((lane & 3) == 0)
          for (int i = 0; i < 3; ++i) wnmom[warp][k][3 * (lane >> 2) + i] = n3[i];
      } else if (lane < 24) {
        wnmom[warp][k][lane] = 0.0;
      }
    }
    __syncthreads();
    for (int t = tid; t < cnt * 24; t += 128) {
      const int k = t / 24, m = t - 24 * k;
      smom[k][m] = ((double)wmom[0][k][m] + (double)wmom[1][k][m]) +
                   ((double)wmom[2][k][m] + (double)wmom[3][k][m]) +
                   ((wnmom[0][k][m] + wnmom[1][k][m]) + (wnmom[2][k][m] + wnmom[3][k][m]));
    }
    __syncthreads();
    for (int t = tid; t < cnt * 12; t += 128) {
      const int k = t / 12, o = t - 12 * k, w = o / 3, e = o - 3 * w;
      const int e1 = e == 2 ? 0 : e + 1, e2 = e == 0 ? 2 : e - 1;
      const double* G = pgeo + (size_t)(cb + k) * 12;  // E0, E1, F0, F1
      const double* D = &smom[k][12];                  // D_i at D[3 i]
      // X-part: E0 x D_i + E1 x D_{i+1}, i = 0 (vertices 0, 1) or 2 (vertices 2, 3)
      const int ix = w < 2 ? 0 : 2;
      const double xs = G[e1] * D[3 * ix + e2] - G[e2] * D[3 * ix + e1] +
                        G[3 + e1] * D[3 * ix + 3 + e2] - G[3 + e2] * D[3 * ix + 3 + e1];
      // Y-part: D_i x F0 + D_{i+2} x F1, i = 0 (vertices 0, 2) or 1 (vertices 1, 3)
      const int iy = w & 1;
      const double ys = D[3 * iy + e1] * G[6 + e2] - D[3 * iy + e2] * G[6 + e1] +
                        D[3 * iy + 6 + e1] * G[9 + e2] - D[3 * iy + 6 + e2] * G[9 + e1];
      const double val = smom[k][o] + ((w & 1) ? xs : -xs) + (w >= 2 ? ys : -ys);
      gcell_part[((size_t)blockIdx.y * C + cb + k) * 12 + o] = val;
    }
  }
  // each thread reads back only the entries of sgrow it wrote itself
#pragma unroll
  for (int j = 0; j < kAdjRpt; ++j) {
    const int row = r0 + 128 * j + tid;
    if (row < N)
      for (int e = 0; e < 3; ++e)
        grow_part[((size_t)blockIdx.x * N + row) * 3 + e] = sgrow[j][e][tid];
  }
}

// Singular panels of each row (FP64, vertex rule): row part into grow_sing,
// panel-vertex part per (row, panel) pair into gpair[e][12].
__global__ void k_adj_singular(int N, const double* __restrict__ X, const int* __restrict__ dnset,
                               const int* __restrict__ sptr, const int* __restrict__ scell,
                               const int4* __restrict__ cell_dofs, const double* __restrict__ lam,
                               const double* __restrict__ phi, const double* __restrict__ dn,
                               double* __restrict__ grow_sing, double* __restrict__ gpair) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= N) return;
  double xi[3];
  for (int d = 0; d < 3; ++d) xi[d] = X[3 * (size_t)row + d];
  const double li = lam[row], phii = phi[row];
  int set[kMaxSet];
  for (int k = 0; k < kMaxSet; ++k) set[k] = dnset[(size_t)row * kMaxSet + k];
  double grow[3] = {0, 0, 0};
  for (int e = sptr[row]; e < sptr[row + 1]; ++e) {
    const int cell = scell[e];
    const int4 d = cell_dofs[cell];
    const int id[4] = {d.x, d.y, d.z, d.w};
    int v = -1;
    for (int j = 0; j < 4 && v < 0; ++j)
      for (int s = 0; s < kMaxSet; ++s)
        if (set[s] == id[j]) v = j;
    double g[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (v >= 0 && li != 0.0) {
      double P[4][3], ph[4], pn[4];
      for (int k = 0; k < 4; ++k) {
        for (int c = 0; c < 3; ++c) P[k][c] = X[3 * (size_t)id[k] + c];
        ph[k] = phi[id[k]];
        pn[k] = dn[id[k]];
      }
      for (int q = 0; q < c_qa.nsp; ++q) {
        const double s = c_qa.sp[v][q][0], u = c_qa.sp[v][q][1], w = c_qa.sp[v][q][2] * kI4P;
        const double N4[4] = {(1 - s) * (1 - u), s * (1 - u), (1 - s) * u, s * u};
        const double Ns[4] = {-(1 - u), (1 - u), -u, u};
        const double Nt[4] = {-(1 - s), -s, (1 - s), s};
        double x[3] = {0, 0, 0}, jx[3] = {0, 0, 0}, je[3] = {0, 0, 0}, fp = 0, fn = 0;
        for (int k = 0; k < 4; ++k) {
          for (int c = 0; c < 3; ++c) {
            x[c] += N4[k] * P[k][c];
            jx[c] += Ns[k] * P[k][c];
            je[c] += Nt[k] * P[k][c];
          }
          fp += N4[k] * ph[k];
          fn += N4[k] * pn[k];
        }
        const double R[3] = {x[0] - xi[0], x[1] - xi[1], x[2] - xi[2]};
        const double c[3] = {jx[1] * je[2] - jx[2] * je[1], jx[2] * je[0] - jx[0] * je[2],
                             jx[0] * je[1] - jx[1] * je[0]};
        const double J = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        double aR[3], ac[3];
        point_grad<double>(R, c, J, w * li * (fp - phii), w * li * fn, aR, ac);
        const double gjx[3] = {je[1] * ac[2] - je[2] * ac[1], je[2] * ac[0] - je[0] * ac[2],
                               je[0] * ac[1] - je[1] * ac[0]};
        const double gje[3] = {ac[1] * jx[2] - ac[2] * jx[1], ac[2] * jx[0] - ac[0] * jx[2],
                               ac[0] * jx[1] - ac[1] * jx[0]};
        for (int c2 = 0; c2 < 3; ++c2) grow[c2] -= aR[c2];
        for (int k = 0; k < 4; ++k)
          for (int c2 = 0; c2 < 3; ++c2) g[3 * k + c2] += N4[k] * aR[c2] + Ns[k] * gjx[c2] + Nt[k] * gje[c2];
      }
    }
    for (int t = 0; t < 12; ++t) gpair[(size_t)e * 12 + t] = g[t];
  }
  for (int c = 0; c < 3; ++c) grow_sing[3 * (size_t)row + c] = grow[c];
}

// lambda^T dG/dX per node (deterministic sums), minus, plus the direct force
// term of the hull panels:  out[p] = gdirect[p] - (row terms + panel-vertex terms).
__global__ void k_adj_reduce(int N, int C, int n_cb, int n_rb, const double* __restrict__ grow_part,
                             const double* __restrict__ grow_sing, const double* __restrict__ gcell_part,
                             const double* __restrict__ gpair, const int* __restrict__ cpair_ptr,
                             const int* __restrict__ cpair_idx, const int* __restrict__ ncptr,
                             const int* __restrict__ ncent, const int* __restrict__ hull_of_cell,
                             const double* __restrict__ ghull, double* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  double s[3] = {0, 0, 0}, dir[3] = {0, 0, 0};
  for (int b = 0; b < n_cb; ++b)
    for (int e = 0; e < 3; ++e) s[e] += grow_part[((size_t)b * N + p) * 3 + e];
  for (int e = 0; e < 3; ++e) s[e] += grow_sing[3 * (size_t)p + e];
  for (int t = ncptr[p]; t < ncptr[p + 1]; ++t) {
    const int cell = ncent[t] >> 2, v = ncent[t] & 3;
    for (int b = 0; b < n_rb; ++b)
      for (int e = 0; e < 3; ++e) s[e] += gcell_part[((size_t)b * C + cell) * 12 + 3 * v + e];
    for (int k = cpair_ptr[cell]; k < cpair_ptr[cell + 1]; ++k)
      for (int e = 0; e < 3; ++e) s[e] += gpair[(size_t)cpair_idx[k] * 12 + 3 * v + e];
    const int hc = hull_of_cell[cell];
    if (hc >= 0)
      for (int e = 0; e < 3; ++e) dir[e] += ghull[(size_t)hc * 12 + 3 * v + e];
  }
  for (int e = 0; e < 3; ++e) out[3 * (size_t)p + e] = dir[e] - s[e];
}

// direct force derivatives with respect to nodal phi / dphi_dn (per node)
__global__ void k_hull_node_sum(int N, const int* __restrict__ ncptr, const int* __restrict__ ncent,
                                const int* __restrict__ hull_of_cell, const double* __restrict__ gph,
                                const double* __restrict__ gpn, double* __restrict__ out_ph,
                                double* __restrict__ out_pn) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  double a = 0, b = 0;
  for (int t = ncptr[p]; t < ncptr[p + 1]; ++t) {
    const int hc = hull_of_cell[ncent[t] >> 2];
    if (hc >= 0) {
      a += gph[(size_t)hc * 4 + (ncent[t] & 3)];
      b += gpn[(size_t)hc * 4 + (ncent[t] & 3)];
    }
  }
  out_ph[p] = a;
  out_pn[p] = b;
}

// g_x = o * dF/dphi + s * dF/ddn ; fields phi / dn from sol and b
__global__ void k_fields(int N, const uint8_t* __restrict__ mask, const double* __restrict__ sol,
                         const double* __restrict__ b, double* __restrict__ phi,
                         double* __restrict__ dn) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (mask[i]) {
    phi[i] = b[i];
    dn[i] = sol[i];
  } else {
    phi[i] = sol[i];
    dn[i] = b[i];
  }
}
__global__ void k_gx(int N, const uint8_t* __restrict__ mask, const double* __restrict__ gph,
                     const double* __restrict__ gpn, double* __restrict__ gx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  gx[i] = mask[i] ? gpn[i] : gph[i];
}
// dF/db = s*gph + o*gpn + B^T lam_u - alpha s lam_u  (B^T lam_u given in bt)
__global__ void k_gb(int N, const uint8_t* __restrict__ mask, const double* __restrict__ gph,
                     const double* __restrict__ gpn, const double* __restrict__ bt,
                     const double* __restrict__ alpha, const double* __restrict__ lamu,
                     double* __restrict__ gb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double v = (mask[i] ? gph[i] : gpn[i]) + bt[i];
  if (mask[i]) v -= alpha[i] * lamu[i];
  gb[i] = v;
}

template <int Q1>
static cudaError_t launch_adj_tile_t(int N, int C, const double* X, const int* dnset,
                                     const int4* cd, const double* lam, const double* phi,
                                     const double* dn, double* grow_part, double* gcell_part,
                                     int cpb, cudaStream_t s) {
  dim3 grid((C + cpb - 1) / cpb, (N + 127) / 128);
  k_adj_tile<Q1><<<grid, 128, 0, s>>>(N, C, X, dnset, cd, lam, phi, dn, grow_part, gcell_part,
                                      cpb);
  return cudaGetLastError();
}

template <int Q1>
static cudaError_t launch_adj_mixed_t(int N, int C, const double* X, const int* dnset,
                                      const int4* cd, const float4* geo, const double* lam,
                                      const double* phi, const double* dn, double* recd,
                                      float4* recf, double* pgeo, double* grow_part,
                                      double* gcell_part, int cpb, cudaStream_t s) {
  constexpr int NQ = Q1 * Q1;
  k_adj_points<Q1><<<(C * NQ + 255) / 256, 256, 0, s>>>(C, X, cd, phi, dn, recd, recf, pgeo);
  dim3 grid((C + cpb - 1) / cpb, (N + kAdjRowsCta - 1) / kAdjRowsCta);
  k_adj_tile_mixed<Q1><<<grid, 128, 0, s>>>(N, C, X, dnset, cd, geo, recf, recd, pgeo, lam, phi,
                                            grow_part, gcell_part, cpb);
  return cudaGetLastError();
}

// Adjoint of assemble + solve_system for an objective J(X, phi, dphi_dn). Its
// direct partial derivatives come either from the hull force (hull_cells
// given: dF/dphi, dF/ddn and dF/dX|direct of the hull panels) or from the
// caller (dJ_dphi, dJ_ddn per node in caller order, no direct X term).
void constraints_adjoint(wbem_context* h, const double* tmp_rhs, const double* lam, double* dJ_dX,
                         double* dJ_db);

static int adjoint_run(wbem_context* h, const int* hull_cells, int n_hull, const double* U, int dir,
                       const double* dJ_dphi, const double* dJ_ddn, double* dF_dX,
                       double* dF_drhs) {
  const int N = h->N, C = h->C;
  const int q1 = h->opt.quadrature_order;
  if (h->assembled_prec == kAssembledFma)
    return fail(h, WBEM_ERR_STATE, "the adjoint needs the direct method (no FMA adjoint)");
  if (q1 < 2 || q1 > 6) return fail(h, WBEM_ERR_ARG, "adjoint supports quadrature orders 2..6");
  const bool mixed = h->assembled_prec == WBEM_PREC_MIXED;
  WB_CHK(ensure_vectors(h, h->opt.gmres_restart));
  EvTimer tm(h->stream);
  int4* hd = nullptr;
  int *d_hoc = nullptr, *d_cpptr = nullptr, *d_cpidx = nullptr;
  double *d_ghull = nullptr, *d_gph = nullptr, *d_gpn = nullptr;
  double *grow_part = nullptr, *gcell_part = nullptr, *grow_sing = nullptr, *gpair = nullptr;
  double *recd = nullptr, *pgeo = nullptr;
  float4* recf = nullptr;
  double *d_out = nullptr, *d_nph = nullptr;
  DeviceFreeGuard scratch{{reinterpret_cast<void**>(&hd), reinterpret_cast<void**>(&d_hoc),
                           reinterpret_cast<void**>(&d_cpptr), reinterpret_cast<void**>(&d_cpidx),
                           reinterpret_cast<void**>(&d_ghull), reinterpret_cast<void**>(&d_gph),
                           reinterpret_cast<void**>(&d_gpn), reinterpret_cast<void**>(&grow_part),
                           reinterpret_cast<void**>(&gcell_part),
                           reinterpret_cast<void**>(&grow_sing), reinterpret_cast<void**>(&gpair),
                           reinterpret_cast<void**>(&recd), reinterpret_cast<void**>(&pgeo),
                           reinterpret_cast<void**>(&recf), reinterpret_cast<void**>(&d_out),
                           reinterpret_cast<void**>(&d_nph)}};
  // hull panel data
  std::vector<int> hull_ids;
  WB_CHK(hull_dofs_upload(h, hull_cells, n_hull, &hd, &hull_ids));
  std::vector<int> hoc(C, -1);
  for (int k = 0; k < n_hull; ++k) hoc[hull_ids[k]] = k;
  // panels per CTA column and rows per CTA of the tile kernel
  const int cpb = mixed ? 128 : 64;
  const int rows_cta = mixed ? kAdjRowsCta : 128;
  const int n_cb = (C + cpb - 1) / cpb, n_rb = (N + rows_cta - 1) / rows_cta;
  const size_t npts = (size_t)C * q1 * q1;
  int st = WBEM_OK;
  // cell -> singular pair index lists (inverse of the per-row singular lists)
  std::vector<int> sptr(N + 1), scell;
  WB_CU(cudaMemcpyAsync(sptr.data(), h->d_sptr, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, h->stream));
  WB_CU(cudaStreamSynchronize(h->stream));
  scell.resize(sptr[N]);
  if (sptr[N] > 0)
    WB_CU(cudaMemcpyAsync(scell.data(), h->d_scell, sizeof(int) * sptr[N], cudaMemcpyDeviceToHost, h->stream));
  WB_CU(cudaStreamSynchronize(h->stream));
  std::vector<int> cpptr(C + 1, 0), cpidx(scell.size());
  for (int c : scell) cpptr[c + 1]++;
  for (int c = 0; c < C; ++c) cpptr[c + 1] += cpptr[c];
  {
    std::vector<int> fill(cpptr.begin(), cpptr.end() - 1);
    for (int e = 0; e < (int)scell.size(); ++e) cpidx[fill[scell[e]]++] = e;
  }
  do {
    if ((st = upload(h, &d_hoc, hoc)) != WBEM_OK) break;
    if ((st = upload(h, &d_cpptr, cpptr)) != WBEM_OK) break;
    if ((st = upload(h, &d_cpidx, cpidx)) != WBEM_OK) break;
    if ((st = dev_alloc(h, &d_ghull, (size_t)std::max(1, n_hull) * 12)) != WBEM_OK) break;
    if ((st = dev_alloc(h, &d_gph, (size_t)std::max(1, n_hull) * 4)) != WBEM_OK) break;
    if ((st = dev_alloc(h, &d_gpn, (size_t)std::max(1, n_hull) * 4)) != WBEM_OK) break;
    if ((st = dev_alloc(h, &grow_part, (size_t)n_cb * N * 3)) != WBEM_OK) break;
    if ((st = dev_alloc(h, &gcell_part, (size_t)n_rb * C * 12)) != WBEM_OK) break;
    if ((st = dev_alloc(h, &grow_sing, (size_t)N * 3)) != WBEM_OK) break;
    if ((st = dev_alloc(h, &gpair, (size_t)std::max<size_t>(1, scell.size()) * 12)) != WBEM_OK) break;
    if ((st = dev_alloc(h, &d_out, (size_t)N * 3)) != WBEM_OK) break;
    if ((st = dev_alloc(h, &d_nph, (size_t)N * 2)) != WBEM_OK) break;
    if (mixed) {
      if ((st = dev_alloc(h, &recd, npts * kPt)) != WBEM_OK) break;
      if ((st = dev_alloc(h, &recf, npts * 3)) != WBEM_OK) break;
      if ((st = dev_alloc(h, &pgeo, (size_t)C * 12)) != WBEM_OK) break;
    }
    double* phi = h->d_vec[3];
    double* dn = h->d_vec[4];
    double* gx = h->d_vec[5];
    double* lam = h->d_vec[6];
    double* nph = d_nph;  // per-node dF/dphi, dF/ddn
    double* npn = d_nph + N;
    const int bs = 256, nb = (N + bs - 1) / bs;
    // fields and direct force derivatives
    k_fields<<<nb, bs, 0, h->stream>>>(N, h->d_mask, h->d_sol, h->d_b, phi, dn);
    if (hull_cells) {
      WB_CU(launch_hull_force_grad(n_hull, hd, h->d_X, U, dir, phi, dn, d_ghull, d_gph, d_gpn, h->stream));
      k_hull_node_sum<<<nb, bs, 0, h->stream>>>(N, h->d_ncptr, h->d_ncent, d_hoc, d_gph, d_gpn, nph, npn);
    } else {
      std::vector<double> dj(2 * (size_t)N);
      for (int i = 0; i < N; ++i) {
        dj[i] = dJ_dphi[h->perm[i]];
        dj[N + i] = dJ_ddn[h->perm[i]];
      }
      WB_CU(cudaMemcpyAsync(d_nph, dj.data(), sizeof(double) * 2 * N, cudaMemcpyHostToDevice, h->stream));
      WB_CU(cudaStreamSynchronize(h->stream));
    }
    k_gx<<<nb, bs, 0, h->stream>>>(N, h->d_mask, nph, npn, gx);
    WB_CU(cudaGetLastError());
    // transposed solve A^T lambda = g_x (constrained operator)
    st = solve_assembled(h, gx, lam, 1);
    if (st != WBEM_OK) break;
    // lam_u: constrained rows take no part in dG/dX; keep lam for the b-terms
    double* lamu = h->d_vec[2];
    WB_CU(cudaMemcpyAsync(lamu, lam, sizeof(double) * N, cudaMemcpyDeviceToDevice, h->stream));
    if (h->n_crows) {
      WB_CU(cudaMemsetAsync(d_out, 0, sizeof(double) * h->n_crows, h->stream));
      WB_CU(launch_set_rows(h->n_crows, h->d_crow, d_out, lamu, h->stream));
    }
    // K7: recompute the panel terms with their derivatives
    const float4* geo = reinterpret_cast<const float4*>(h->d_cellgeo);
    cudaError_t e;
    if (mixed) {
      const int4* cd = h->d_cell_dofs;
      switch (q1) {
        case 2: e = launch_adj_mixed_t<2>(N, C, h->d_X, h->d_dnset, cd, geo, lamu, phi, dn, recd, recf, pgeo, grow_part, gcell_part, cpb, h->stream); break;
        case 3: e = launch_adj_mixed_t<3>(N, C, h->d_X, h->d_dnset, cd, geo, lamu, phi, dn, recd, recf, pgeo, grow_part, gcell_part, cpb, h->stream); break;
        case 4: e = launch_adj_mixed_t<4>(N, C, h->d_X, h->d_dnset, cd, geo, lamu, phi, dn, recd, recf, pgeo, grow_part, gcell_part, cpb, h->stream); break;
        case 5: e = launch_adj_mixed_t<5>(N, C, h->d_X, h->d_dnset, cd, geo, lamu, phi, dn, recd, recf, pgeo, grow_part, gcell_part, cpb, h->stream); break;
        default: e = launch_adj_mixed_t<6>(N, C, h->d_X, h->d_dnset, cd, geo, lamu, phi, dn, recd, recf, pgeo, grow_part, gcell_part, cpb, h->stream); break;
      }
    } else {
      switch (q1) {
        case 2: e = launch_adj_tile_t<2>(N, C, h->d_X, h->d_dnset, h->d_cell_dofs, lamu, phi, dn, grow_part, gcell_part, cpb, h->stream); break;
        case 3: e = launch_adj_tile_t<3>(N, C, h->d_X, h->d_dnset, h->d_cell_dofs, lamu, phi, dn, grow_part, gcell_part, cpb, h->stream); break;
        case 4: e = launch_adj_tile_t<4>(N, C, h->d_X, h->d_dnset, h->d_cell_dofs, lamu, phi, dn, grow_part, gcell_part, cpb, h->stream); break;
        case 5: e = launch_adj_tile_t<5>(N, C, h->d_X, h->d_dnset, h->d_cell_dofs, lamu, phi, dn, grow_part, gcell_part, cpb, h->stream); break;
        default: e = launch_adj_tile_t<6>(N, C, h->d_X, h->d_dnset, h->d_cell_dofs, lamu, phi, dn, grow_part, gcell_part, cpb, h->stream); break;
      }
    }
    WB_CU(e);
    k_adj_singular<<<(N + 63) / 64, 64, 0, h->stream>>>(N, h->d_X, h->d_dnset, h->d_sptr, h->d_scell,
                                                        h->d_cell_dofs, lamu, phi, dn, grow_sing, gpair);
    k_adj_reduce<<<nb, bs, 0, h->stream>>>(N, C, n_cb, n_rb, grow_part, grow_sing, gcell_part, gpair,
                                           d_cpptr, d_cpidx, h->d_ncptr, h->d_ncent, d_hoc, d_ghull,
                                           d_out);
    WB_CU(cudaGetLastError());
    // dF/db: complementary transposed operator B^T lam_u (B = mask ? -N : D, no alpha)
    double* bt = h->d_vec[7];
    double* part = h->d_part + 256 * 128;
    if (mixed)
      WB_CU(launch_matvec_t_mixed(N, h->d_B2, h->d_mask, nullptr, lamu, bt, part, h->stream));
    else
      WB_CU(launch_matvec_t_fp64(N, h->d_D, h->d_N, h->d_mask, nullptr, lamu, bt, part, h->stream));
    double* gb = h->d_vec[0];
    k_gb<<<nb, bs, 0, h->stream>>>(N, h->d_mask, nph, npn, bt, h->d_alpha, lamu, gb);
    WB_CU(cudaGetLastError());
    h->launches += (mixed ? 13 : 12) - (hull_cells ? 0 : 2);
    WB_CHK(check_device_error(h, "adjoint"));
    // back to the caller's order; constraint inhomogeneities tied to b
    std::vector<double> gXi(3 * (size_t)N), gbi(N), li(N);
    WB_CU(cudaMemcpyAsync(gXi.data(), d_out, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, h->stream));
    WB_CU(cudaMemcpyAsync(gbi.data(), gb, sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream));
    WB_CU(cudaMemcpyAsync(li.data(), lam, sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream));
    WB_CU(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < N; ++i) {
      const int p = h->perm[i];
      for (int d = 0; d < 3; ++d) dF_dX[3 * (size_t)p + d] = gXi[3 * (size_t)i + d];
      dF_drhs[p] = gbi[i];
    }
    // constraint inhomogeneities: a Dirichlet-Neumann line carries the datum
    // of its Dirichlet copy; a sharp Dirichlet-Dirichlet line carries a value
    // of the projected normals and surface gradients, i.e. of X and b
    std::vector<double> lc(N);
    for (int i = 0; i < N; ++i) lc[h->perm[i]] = li[i];
    constraints_adjoint(h, h->sol_b.data(), lc.data(), dF_dX, dF_drhs);
    h->stats.t_adjoint_ms = tm.ms();
  } while (0);
  return st;
}

int adjoint_force(wbem_context* h, const int* hull_cells, int n_hull, const double* U, int dir,
                  double* dF_dX, double* dF_drhs) {
  return adjoint_run(h, hull_cells, n_hull, U, dir, nullptr, nullptr, dF_dX, dF_drhs);
}

int adjoint_objective(wbem_context* h, const double* dJ_dphi, const double* dJ_ddn, double* dJ_dX,
                      double* dJ_drhs) {
  return adjoint_run(h, nullptr, 0, nullptr, 0, dJ_dphi, dJ_ddn, dJ_dX, dJ_drhs);
}

}  // namespace wbem
