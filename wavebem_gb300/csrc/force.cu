// Hull pressure force and its direct derivatives.
//
// F = sum over hull panels of  int p n_dir dS  with
// p = -(U . grad phi + |grad phi|^2 / 2),
// grad phi = tangential gradient of the Q1 interpolant of phi + (interpolated
// dphi/dn) n, n the unit panel normal, the regular Gauss rule of the assembly.
// This is the steady (phi_t = 0), rho = 1, g = 0 form of the reference's
// pressure force (source/free_surface.cc:6936-6942).
#include <cuda_runtime.h>
#include <stdint.h>
#include "kernels.h"
#include "../../include/wbem.h"

namespace wbem {

static __constant__ QuadTables c_qf;

cudaError_t upload_quadrature_force(const QuadTables& t) {
  return cudaMemcpyToSymbol(c_qf, &t, sizeof(QuadTables));
}

// Per-point force integrand and its partial derivatives with respect to the
// 4 panel vertices (12), the 4 nodal phi and the 4 nodal dphi/dn.
// When grad == nullptr only the value is computed.
__device__ void force_point(const double P[4][3], const double ph4[4], const double pn4[4],
                            const double U[3], int dir, double s, double t, double w,
                            double* val, double gP[4][3], double gph[4], double gpn[4]) {
  const double N4[4] = {(1 - s) * (1 - t), s * (1 - t), (1 - s) * t, s * t};
  const double Ns[4] = {-(1 - t), (1 - t), -t, t};
  const double Nt[4] = {-(1 - s), -s, (1 - s), s};
  double jx[3] = {0, 0, 0}, je[3] = {0, 0, 0};
  for (int k = 0; k < 4; ++k)
    for (int d = 0; d < 3; ++d) {
      jx[d] += Ns[k] * P[k][d];
      je[d] += Nt[k] * P[k][d];
    }
  double gs = 0, gt = 0, pn = 0;
  for (int k = 0; k < 4; ++k) {
    gs += Ns[k] * ph4[k];
    gt += Nt[k] * ph4[k];
    pn += N4[k] * pn4[k];
  }
  const double g11 = jx[0] * jx[0] + jx[1] * jx[1] + jx[2] * jx[2];
  const double g12 = jx[0] * je[0] + jx[1] * je[1] + jx[2] * je[2];
  const double g22 = je[0] * je[0] + je[1] * je[1] + je[2] * je[2];
  const double det = g11 * g22 - g12 * g12;
  const double c1 = (g22 * gs - g12 * gt) / det;
  const double c2 = (-g12 * gs + g11 * gt) / det;
  double cr[3] = {jx[1] * je[2] - jx[2] * je[1], jx[2] * je[0] - jx[0] * je[2],
                  jx[0] * je[1] - jx[1] * je[0]};
  const double A = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
  double n[3] = {cr[0] / A, cr[1] / A, cr[2] / A};
  double G[3];
  for (int d = 0; d < 3; ++d) G[d] = c1 * jx[d] + c2 * je[d] + pn * n[d];
  const double UG = U[0] * G[0] + U[1] * G[1] + U[2] * G[2];
  const double GG = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
  const double p = -(UG + 0.5 * GG);
  // F_q = p * n_dir * A * w = p * cr_dir * w
  *val = p * cr[dir] * w;
  if (!gP) return;
  // reverse mode by hand
  const double dF_dp = cr[dir] * w;
  double dF_dcr[3] = {0, 0, 0};
  dF_dcr[dir] = p * w;
  // p = -(U.G + G.G/2): dp/dG = -(U + G)
  double dG[3];
  for (int d = 0; d < 3; ++d) dG[d] = -(U[d] + G[d]) * dF_dp;
  // G = c1 jx + c2 je + pn n
  double dc1 = 0, dc2 = 0, dpn = 0, djx[3], dje[3], dn[3];
  for (int d = 0; d < 3; ++d) {
    dc1 += dG[d] * jx[d];
    dc2 += dG[d] * je[d];
    dpn += dG[d] * n[d];
    djx[d] = dG[d] * c1;
    dje[d] = dG[d] * c2;
    dn[d] = dG[d] * pn;
  }
  // n = cr / A: dcr += (dn - n (n.dn)) / A
  const double ndn = n[0] * dn[0] + n[1] * dn[1] + n[2] * dn[2];
  for (int d = 0; d < 3; ++d) dF_dcr[d] += (dn[d] - n[d] * ndn) / A;
  // c1 = (g22 gs - g12 gt)/det, c2 = (-g12 gs + g11 gt)/det
  const double dgs = (dc1 * g22 - dc2 * g12) / det;
  const double dgt = (-dc1 * g12 + dc2 * g11) / det;
  // d/dg11, g12, g22 of c1, c2
  // c = Ginv g with Ginv = [[g22,-g12],[-g12,g11]]/det; dc = -Ginv dG c
  // -> dL/dG_ab = -(Ginv^T dc)_a c_b, symmetric metric: g11 <- (a=b=1), g22, g12 (both off-diag)
  const double u1 = dgs, u2 = dgt;  // Ginv^T dc (Ginv symmetric)
  const double dg11 = -u1 * c1;
  const double dg22 = -u2 * c2;
  const double dg12 = -(u1 * c2 + u2 * c1);
  for (int d = 0; d < 3; ++d) {
    djx[d] += 2 * dg11 * jx[d] + dg12 * je[d];
    dje[d] += 2 * dg22 * je[d] + dg12 * jx[d];
  }
  // cr = jx x je
  djx[0] += je[1] * dF_dcr[2] - je[2] * dF_dcr[1];
  djx[1] += je[2] * dF_dcr[0] - je[0] * dF_dcr[2];
  djx[2] += je[0] * dF_dcr[1] - je[1] * dF_dcr[0];
  dje[0] += dF_dcr[1] * jx[2] - dF_dcr[2] * jx[1];
  dje[1] += dF_dcr[2] * jx[0] - dF_dcr[0] * jx[2];
  dje[2] += dF_dcr[0] * jx[1] - dF_dcr[1] * jx[0];
  for (int k = 0; k < 4; ++k) {
    for (int d = 0; d < 3; ++d) gP[k][d] += Ns[k] * djx[d] + Nt[k] * dje[d];
    gph[k] += Ns[k] * dgs + Nt[k] * dgt;
    gpn[k] += N4[k] * dpn;
  }
}

__global__ void k_hull_force(int nh, const int4* __restrict__ hd, const double* __restrict__ X,
                             double U0, double U1, double U2, int dir,
                             const double* __restrict__ phi, const double* __restrict__ dphi,
                             double* __restrict__ part) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nh) return;
  const int4 d = hd[c];
  const int id[4] = {d.x, d.y, d.z, d.w};
  double P[4][3], ph[4], pn[4];
  for (int k = 0; k < 4; ++k) {
    for (int e = 0; e < 3; ++e) P[k][e] = X[3 * (size_t)id[k] + e];
    ph[k] = phi[id[k]];
    pn[k] = dphi[id[k]];
  }
  const double U[3] = {U0, U1, U2};
  double F = 0;
  const int nq = c_qf.q1 * c_qf.q1;
  for (int q = 0; q < nq; ++q) {
    double v;
    force_point(P, ph, pn, U, dir, c_qf.gp[q][0], c_qf.gp[q][1], c_qf.gp[q][2], &v, nullptr,
                nullptr, nullptr);
    F += v;
  }
  part[c] = F;
}

__global__ void k_sum_serial(int n, const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double red[256];
  double s = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

cudaError_t launch_hull_force(int nh, const int4* hull_dofs, const double* X, const double* U,
                              int dir, const double* phi, const double* dphi, double* part,
                              cudaStream_t s) {
  if (nh > 0)
    k_hull_force<<<(nh + 127) / 128, 128, 0, s>>>(nh, hull_dofs, X, U[0], U[1], U[2], dir, phi,
                                                  dphi, part);
  k_sum_serial<<<1, 256, 0, s>>>(nh, part, part + nh);
  return cudaGetLastError();
}

__global__ void k_hull_force_grad(int nh, const int4* __restrict__ hd, const double* __restrict__ X,
                                  double U0, double U1, double U2, int dir,
                                  const double* __restrict__ phi, const double* __restrict__ dphi,
                                  double* __restrict__ gX, double* __restrict__ gph,
                                  double* __restrict__ gpn) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nh) return;
  const int4 d = hd[c];
  const int id[4] = {d.x, d.y, d.z, d.w};
  double P[4][3], ph[4], pn[4];
  for (int k = 0; k < 4; ++k) {
    for (int e = 0; e < 3; ++e) P[k][e] = X[3 * (size_t)id[k] + e];
    ph[k] = phi[id[k]];
    pn[k] = dphi[id[k]];
  }
  const double U[3] = {U0, U1, U2};
  double gP[4][3] = {}, g1[4] = {}, g2[4] = {};
  const int nq = c_qf.q1 * c_qf.q1;
  for (int q = 0; q < nq; ++q) {
    double v;
    force_point(P, ph, pn, U, dir, c_qf.gp[q][0], c_qf.gp[q][1], c_qf.gp[q][2], &v, gP, g1, g2);
  }
  for (int k = 0; k < 4; ++k) {
    for (int e = 0; e < 3; ++e) gX[(size_t)c * 12 + 3 * k + e] = gP[k][e];
    gph[(size_t)c * 4 + k] = g1[k];
    gpn[(size_t)c * 4 + k] = g2[k];
  }
}

cudaError_t launch_hull_force_grad(int nh, const int4* hull_dofs, const double* X,
                                   const double* U, int dir, const double* phi, const double* dphi,
                                   double* gX_cell, double* gphi_cell, double* gdphi_cell,
                                   cudaStream_t s) {
  if (nh > 0)
    k_hull_force_grad<<<(nh + 127) / 128, 128, 0, s>>>(nh, hull_dofs, X, U[0], U[1], U[2], dir,
                                                       phi, dphi, gX_cell, gphi_cell, gdphi_cell);
  return cudaGetLastError();
}

}  // namespace wbem
