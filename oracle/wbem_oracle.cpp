// CPU FP64 restatement of WaveBEM's collocation BEM hot path (BEMProblem<3>).
//
// TEST INFRASTRUCTURE ONLY: this file is the oracle that the CUDA library is
// checked against, and the timed CPU baseline. Nothing in the product library
// links or calls it.
//
// Parity status: the reference needs deal.II 8.4/8.5, which is not available,
// so it cannot be compiled or run here; the reference's own tests hold no
// golden vectors for this path. Parity with the real deal.II build is therefore
// UNPINNED. This restatement is pinned instead against closed-form answers
// (Gauss-Legendre exactness, the flat-panel vertex-singular integral
// 2 ln(1+sqrt 2), solid angles of the box corners, Green's identity for
// harmonic functions and the exact sphere solution); see tests/.
//
// Every function names the reference lines it restates. deal.II behaviour is
// restated from its documented mathematics (Gauss-Legendre rules, the Q1
// iso-parametric map, codimension-one normals and JxW, and the polar
// (Lachat-Watson / Duffy type) vertex rule behind QGaussOneOverR<2>); no
// deal.II source is used.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <map>
#include <set>
#include <algorithm>
#include <utility>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double PI = 3.14159265358979323846;

struct V3 {
  double x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 scl(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

inline V3 node(const double* X, int i) { return {X[3 * i], X[3 * i + 1], X[3 * i + 2]}; }

// Gauss-Legendre rule with n points on [0,1], ascending (deal.II QGauss<1>).
void gauss01(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < n; ++i) {
    long double z = std::cos(PI * (i + 0.75) / (n + 0.5));
    long double pp = 0;
    for (int it = 0; it < 100; ++it) {
      long double p1 = 1, p2 = 0;
      for (int k = 1; k <= n; ++k) {
        long double p3 = p2;
        p2 = p1;
        p1 = ((2.0L * k - 1.0L) * z * p2 - (k - 1.0L) * p3) / k;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0L);
      long double dz = p1 / pp;
      z -= dz;
      if (std::fabs((double)dz) < 1e-19) break;
    }
    // z descends with i, so (1 - z)/2 ascends on [0,1]; weight 2/((1-z^2)P'^2) / 2
    x[i] = (double)((1.0L - z) * 0.5L);
    w[i] = (double)(1.0L / ((1.0L - z * z) * pp * pp));
  }
}

// Tensor Gauss rule on the unit square, x fastest (deal.II QGauss<2>).
void gauss2d(int n, std::vector<double>& px, std::vector<double>& py, std::vector<double>& w) {
  std::vector<double> x1, w1;
  gauss01(n, x1, w1);
  px.clear();
  py.clear();
  w.clear();
  for (int b = 0; b < n; ++b)
    for (int a = 0; a < n; ++a) {
      px.push_back(x1[a]);
      py.push_back(x1[b]);
      w.push_back(w1[a] * w1[b]);
    }
}

// Vertex-singular 1/R rule on the unit square (the rule of
// QGaussOneOverR<2>(n, unit_support_point[v], factor_out=true) used at
// source/bem_problem.cc:116-120): the square is split into the two triangles
// that meet at the singular vertex; the triangle below the diagonal is mapped
// from (u,t) in [0,1]^2 by x = u, y = u tan(pi t / 4), whose Jacobian is
// (pi/4) R / cos(pi t / 4) with R the distance to the vertex; the other
// triangle is its mirror image x <-> y. With the singularity factored out the
// weight carries the full Jacobian (including R), so sum w_q f(q) integrates f.
// The rule for vertex 0 is then rotated about the square's centre onto
// vertex v (1:(1,0) 2:(0,1) 3:(1,1)).
void vertex_singular_rule(int n, int v, std::vector<double>& px, std::vector<double>& py,
                          std::vector<double>& w) {
  std::vector<double> gx, gy, gw;
  gauss2d(n, gx, gy, gw);
  const int m = n * n;
  px.assign(2 * m, 0);
  py.assign(2 * m, 0);
  w.assign(2 * m, 0);
  const double pi4 = PI / 4;
  for (int q = 0; q < m; ++q) {
    double x = gx[q];
    double y = gx[q] * std::tan(pi4 * gy[q]);
    double wq = gw[q] * pi4 / std::cos(pi4 * gy[q]);
    wq *= std::sqrt(x * x + y * y);
    px[q] = x;
    py[q] = y;
    w[q] = wq;
    px[m + q] = y;
    py[m + q] = x;
    w[m + q] = wq;
  }
  for (int q = 0; q < 2 * m; ++q) {
    double x = px[q], y = py[q];
    switch (v) {
      case 1: px[q] = 1 - y; py[q] = x; break;      // rotation by +pi/2
      case 2: px[q] = y; py[q] = 1 - x; break;      // rotation by -pi/2
      case 3: px[q] = 1 - x; py[q] = 1 - y; break;  // rotation by pi
      default: break;
    }
  }
}

// Q1 iso-parametric geometry at reference point (xi, eta) of a cell
// (FE_Q<2,3>(1) + MappingQEulerian degree 1; source/bem_problem.cc:133-137).
struct QPoint {
  V3 x;       // real-space point
  V3 n;       // unit normal  d_xi x  cross  d_eta x  / |.|
  double det; // |d_xi x  cross  d_eta x|
  double phi[4];
  double dphi[4][2];
  V3 jx, je;  // Jacobian columns
};

QPoint eval_q1(const V3 P[4], double xi, double eta) {
  QPoint q;
  q.phi[0] = (1 - xi) * (1 - eta);
  q.phi[1] = xi * (1 - eta);
  q.phi[2] = (1 - xi) * eta;
  q.phi[3] = xi * eta;
  q.dphi[0][0] = -(1 - eta); q.dphi[0][1] = -(1 - xi);
  q.dphi[1][0] = (1 - eta);  q.dphi[1][1] = -xi;
  q.dphi[2][0] = -eta;       q.dphi[2][1] = (1 - xi);
  q.dphi[3][0] = eta;        q.dphi[3][1] = xi;
  V3 x = {0, 0, 0}, jx = {0, 0, 0}, je = {0, 0, 0};
  for (int k = 0; k < 4; ++k) {
    x = add(x, scl(q.phi[k], P[k]));
    jx = add(jx, scl(q.dphi[k][0], P[k]));
    je = add(je, scl(q.dphi[k][1], P[k]));
  }
  V3 c = cross(jx, je);
  q.det = norm(c);
  q.n = scl(1.0 / q.det, c);
  q.x = x;
  q.jx = jx;
  q.je = je;
  return q;
}

// LaplaceKernel::kernels<3> (include/laplace_kernel.h:44-62).
inline void kernels(V3 R, V3& D, double& s) {
  double r = norm(R);
  double r2 = r * r;
  s = 1. / (r * 4 * PI);
  D = scl(1.0 / (-4 * PI * r2 * r), R);
}

bool in_set(const int* dn_ptr, const int* dn_idx, int i, int j) {
  for (int k = dn_ptr[i]; k < dn_ptr[i + 1]; ++k)
    if (dn_idx[k] == j) return true;
  return false;
}

struct CellRule {
  std::vector<QPoint> qp;
  std::vector<double> w;
};

CellRule cell_rule(const double* X, const int* cell, const std::vector<double>& px,
                   const std::vector<double>& py, const std::vector<double>& w) {
  V3 P[4];
  for (int k = 0; k < 4; ++k) P[k] = node(X, cell[k]);
  CellRule r;
  r.qp.resize(px.size());
  r.w = w;
  for (size_t q = 0; q < px.size(); ++q) r.qp[q] = eval_q1(P, px[q], py[q]);
  return r;
}

// One (row i, cell) contribution: 4 entries each of N (dG/dn) and D (G)
// (source/bem_problem.cc:241-260 regular, :495-522 singular).
void local_row(const CellRule& r, V3 xi, double ln[4], double ld[4]) {
  for (int j = 0; j < 4; ++j) ln[j] = ld[j] = 0;
  for (size_t q = 0; q < r.qp.size(); ++q) {
    const QPoint& Q = r.qp[q];
    V3 R = sub(Q.x, xi);
    V3 D;
    double s;
    kernels(R, D, s);
    double jxw = Q.det * r.w[q];
    for (int j = 0; j < 4; ++j) {
      ln[j] += (dot(D, Q.n) * Q.phi[j] * jxw);
      ld[j] += (s * Q.phi[j] * jxw);
    }
  }
}

// ------------------------------------------------------------- sparse helpers
// Consistent Q1 mass matrix on the surface (scalar; the vector FE system of
// the reference decouples into three copies of it).
struct Csr {
  int n = 0;
  std::vector<int> ptr, idx;
  std::vector<double> val;
};

Csr mass_matrix(int N, const double* X, int C, const int* cells, int qorder) {
  std::vector<double> px, py, w;
  gauss2d(qorder, px, py, w);
  std::vector<std::map<int, double>> rows(N);
  for (int c = 0; c < C; ++c) {
    CellRule r = cell_rule(X, cells + 4 * c, px, py, w);
    for (size_t q = 0; q < px.size(); ++q) {
      double jxw = r.qp[q].det * r.w[q];
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
          rows[cells[4 * c + a]][cells[4 * c + b]] += r.qp[q].phi[a] * r.qp[q].phi[b] * jxw;
    }
  }
  Csr M;
  M.n = N;
  M.ptr.assign(N + 1, 0);
  for (int i = 0; i < N; ++i) {
    for (auto& kv : rows[i]) {
      M.idx.push_back(kv.first);
      M.val.push_back(kv.second);
    }
    M.ptr[i + 1] = (int)M.idx.size();
  }
  return M;
}

void csr_mv(const Csr& M, const double* x, double* y) {
  for (int i = 0; i < M.n; ++i) {
    double s = 0;
    for (int k = M.ptr[i]; k < M.ptr[i + 1]; ++k) s += M.val[k] * x[M.idx[k]];
    y[i] = s;
  }
}

// Jacobi-preconditioned CG to machine precision (stands in for the UMFPACK
// direct solve of the SPD mass matrix at source/computational_domain.cc:1602-1604).
void cg_solve(const Csr& M, const double* b, double* x) {
  int n = M.n;
  std::vector<double> r(n), z(n), p(n), Ap(n), dinv(n);
  for (int i = 0; i < n; ++i) {
    double d = 0;
    for (int k = M.ptr[i]; k < M.ptr[i + 1]; ++k)
      if (M.idx[k] == i) d = M.val[k];
    dinv[i] = 1.0 / d;
    x[i] = 0;
    r[i] = b[i];
  }
  double bn = 0;
  for (int i = 0; i < n; ++i) bn += b[i] * b[i];
  bn = std::sqrt(bn);
  if (bn == 0) return;
  for (int i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
  p = z;
  double rz = 0;
  for (int i = 0; i < n; ++i) rz += r[i] * z[i];
  for (int it = 0; it < 10 * n + 100; ++it) {
    csr_mv(M, p.data(), Ap.data());
    double pAp = 0;
    for (int i = 0; i < n; ++i) pAp += p[i] * Ap[i];
    double a = rz / pAp;
    double rn = 0;
    for (int i = 0; i < n; ++i) {
      x[i] += a * p[i];
      r[i] -= a * Ap[i];
      rn += r[i] * r[i];
    }
    if (std::sqrt(rn) < 1e-15 * bn) break;
    for (int i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
    double rz2 = 0;
    for (int i = 0; i < n; ++i) rz2 += r[i] * z[i];
    double beta = rz2 / rz;
    rz = rz2;
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
  }
}

// Dense LU with partial pivoting, in place, row-major n x n.
int lu_factor(int n, double* A, int* piv) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    double m = std::fabs(A[(size_t)k * n + k]);
    for (int i = k + 1; i < n; ++i) {
      double v = std::fabs(A[(size_t)i * n + k]);
      if (v > m) { m = v; p = i; }
    }
    piv[k] = p;
    if (m == 0.0 || !std::isfinite(m)) return 5;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(A[(size_t)k * n + j], A[(size_t)p * n + j]);
    double inv = 1.0 / A[(size_t)k * n + k];
    for (int i = k + 1; i < n; ++i) A[(size_t)i * n + k] *= inv;
#pragma omp parallel for schedule(static)
    for (int i = k + 1; i < n; ++i) {
      double l = A[(size_t)i * n + k];
      if (l == 0.0) continue;
      double* ri = A + (size_t)i * n;
      const double* rk = A + (size_t)k * n;
      for (int j = k + 1; j < n; ++j) ri[j] -= l * rk[j];
    }
  }
  return 0;
}

void lu_solve(int n, const double* A, const int* piv, double* b) {
  for (int k = 0; k < n; ++k)
    if (piv[k] != k) std::swap(b[k], b[piv[k]]);
  for (int i = 0; i < n; ++i) {
    double s = b[i];
    const double* r = A + (size_t)i * n;
    for (int j = 0; j < i; ++j) s -= r[j] * b[j];
    b[i] = s;
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    const double* r = A + (size_t)i * n;
    for (int j = i + 1; j < n; ++j) s -= r[j] * b[j];
    b[i] = s / r[i];
  }
}

void matvec(int n, const double* A, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    const double* r = A + (size_t)i * n;
    double s = 0;
    for (int j = 0; j < n; ++j) s += r[j] * x[j];
    y[i] = s;
  }
}

// Constraint lines (deal.II ConstraintMatrix semantics as used at
// source/bem_problem.cc:990-1105 and include/constrained_matrix.h:72-94).
struct Constraints {
  std::map<int, std::vector<std::pair<int, double>>> lines;
  std::map<int, double> inhom;
  void add_line(int l) {
    if (!lines.count(l)) { lines[l] = {}; inhom[l] = 0.0; }
  }
  void add_entry(int l, int c, double v) {
    for (auto& e : lines[l])
      if (e.first == c) return;
    lines[l].push_back({c, v});
  }
  // close(): resolve entries that point at constrained dofs.
  void close() {
    for (int pass = 0; pass < 64; ++pass) {
      bool changed = false;
      for (auto& kv : lines) {
        std::vector<std::pair<int, double>> out;
        double inh = inhom[kv.first];
        for (auto& e : kv.second) {
          auto it = lines.find(e.first);
          if (it != lines.end() && e.first != kv.first) {
            changed = true;
            inh += e.second * inhom[e.first];
            for (auto& e2 : it->second) out.push_back({e2.first, e.second * e2.second});
          } else {
            out.push_back(e);
          }
        }
        // merge duplicate columns
        std::map<int, double> m;
        for (auto& e : out) m[e.first] += e.second;
        kv.second.assign(m.begin(), m.end());
        inhom[kv.first] = inh;
      }
      if (!changed) break;
    }
  }
};

// Nodal normals by L2 projection (source/computational_domain.cc:1525-1620).
void node_normals(int N, const double* X, int C, const int* cells, int qorder, double* nn) {
  Csr M = mass_matrix(N, X, C, cells, qorder);
  std::vector<double> px, py, w;
  gauss2d(qorder, px, py, w);
  std::vector<double> rhs(3 * (size_t)N, 0.0);
  for (int c = 0; c < C; ++c) {
    CellRule r = cell_rule(X, cells + 4 * c, px, py, w);
    for (size_t q = 0; q < px.size(); ++q) {
      double jxw = r.qp[q].det * r.w[q];
      for (int a = 0; a < 4; ++a) {
        int i = cells[4 * c + a];
        rhs[0 * (size_t)N + i] += r.qp[q].phi[a] * r.qp[q].n.x * jxw;
        rhs[1 * (size_t)N + i] += r.qp[q].phi[a] * r.qp[q].n.y * jxw;
        rhs[2 * (size_t)N + i] += r.qp[q].phi[a] * r.qp[q].n.z * jxw;
      }
    }
  }
  std::vector<double> sol(3 * (size_t)N);
  for (int d = 0; d < 3; ++d) cg_solve(M, rhs.data() + d * (size_t)N, sol.data() + d * (size_t)N);
  for (int i = 0; i < N; ++i) {
    V3 v = {sol[i], sol[N + i], sol[2 * (size_t)N + i]};
    double l = norm(v);
    nn[3 * i] = v.x / l;
    nn[3 * i + 1] = v.y / l;
    nn[3 * i + 2] = v.z / l;
  }
}

// Nodal surface gradients of (tmp_rhs * surface_nodes) by L2 projection
// (source/bem_problem.cc:1153-1293).
void surface_gradients(int N, const double* X, int C, const int* cells, int qorder,
                       const unsigned char* mask, const double* tmp_rhs, double* g) {
  Csr M = mass_matrix(N, X, C, cells, qorder);
  std::vector<double> px, py, w;
  gauss2d(qorder, px, py, w);
  std::vector<double> rhs(3 * (size_t)N, 0.0);
  for (int c = 0; c < C; ++c) {
    CellRule r = cell_rule(X, cells + 4 * c, px, py, w);
    double f[4];
    for (int a = 0; a < 4; ++a) {
      int i = cells[4 * c + a];
      f[a] = tmp_rhs[i] * (mask[i] ? 1.0 : 0.0);
    }
    for (size_t q = 0; q < px.size(); ++q) {
      const QPoint& Q = r.qp[q];
      // tangential gradient: J (J^T J)^{-1} grad_ref
      double gx = 0, ge = 0;
      for (int a = 0; a < 4; ++a) {
        gx += Q.dphi[a][0] * f[a];
        ge += Q.dphi[a][1] * f[a];
      }
      double g11 = dot(Q.jx, Q.jx), g12 = dot(Q.jx, Q.je), g22 = dot(Q.je, Q.je);
      double det = g11 * g22 - g12 * g12;
      double c1 = (g22 * gx - g12 * ge) / det, c2 = (-g12 * gx + g11 * ge) / det;
      V3 grad = add(scl(c1, Q.jx), scl(c2, Q.je));
      double jxw = Q.det * r.w[q];
      for (int a = 0; a < 4; ++a) {
        int i = cells[4 * c + a];
        rhs[0 * (size_t)N + i] += Q.phi[a] * grad.x * jxw;
        rhs[1 * (size_t)N + i] += Q.phi[a] * grad.y * jxw;
        rhs[2 * (size_t)N + i] += Q.phi[a] * grad.z * jxw;
      }
    }
  }
  std::vector<double> sol(3 * (size_t)N);
  for (int d = 0; d < 3; ++d) cg_solve(M, rhs.data() + d * (size_t)N, sol.data() + d * (size_t)N);
  for (int i = 0; i < N; ++i) {
    g[3 * i] = sol[i];
    g[3 * i + 1] = sol[N + i];
    g[3 * i + 2] = sol[2 * (size_t)N + i];
  }
}

Constraints build_constraints(int N, const double* X, int C, const int* cells, int qorder,
                              const int* dn_ptr, const int* dn_idx, const unsigned char* mask,
                              const double* tmp_rhs) {
  // normals / gradients are only consulted for Dirichlet-Dirichlet pairs
  bool need_geo = false;
  for (int i = 0; i < N && !need_geo; ++i)
    if (mask[i])
      for (int k = dn_ptr[i]; k < dn_ptr[i + 1]; ++k)
        if (dn_idx[k] != i && mask[dn_idx[k]]) { need_geo = true; break; }
  std::vector<double> nn, gg;
  if (need_geo) {
    nn.resize(3 * (size_t)N);
    gg.resize(3 * (size_t)N);
    node_normals(N, X, C, cells, qorder, nn.data());
    surface_gradients(N, X, C, cells, qorder, mask, tmp_rhs, gg.data());
  }
  auto NN = [&](int i) { return V3{nn[3 * i], nn[3 * i + 1], nn[3 * i + 2]}; };
  auto GG = [&](int i) { return V3{gg[3 * i], gg[3 * i + 1], gg[3 * i + 2]}; };
  Constraints c;
  for (int i = 0; i < N; ++i) {
    int first = dn_idx[dn_ptr[i]];
    for (int k = dn_ptr[i]; k < dn_ptr[i + 1]; ++k)
      if (mask[dn_idx[k]] == 1) { first = dn_idx[k]; break; }
    if (i != first) continue;
    for (int k = dn_ptr[i]; k < dn_ptr[i + 1]; ++k) {
      int m = dn_idx[k];
      if (m == i) continue;
      if (mask[i] == 1) {
        if (mask[m] == 1) {
          if (norm(sub(NN(m), NN(i))) < 1e-4) {
            c.add_line(m);
            c.add_entry(m, i, 1.0);
          } else {
            c.add_line(m);
            V3 ni = NN(i), nm = NN(m), gi = GG(i), gm = GG(m);
            double cij = dot(ni, nm);
            double this_g = (1.0 / (1.0 - cij * cij)) * (dot(gm, ni) + dot(gi, nm) * cij);
            double other_g = (1.0 / (1.0 - cij * cij)) * (dot(gi, nm) + dot(gm, ni) * cij);
            c.add_line(i);
            c.inhom[i] = this_g;
            c.add_line(m);
            c.inhom[m] = other_g;
          }
        } else {
          c.add_line(m);
          c.inhom[m] = tmp_rhs[i];
        }
      } else {
        c.add_line(m);
        c.add_entry(m, i, 1.0);
      }
    }
  }
  c.close();
  return c;
}

}  // namespace

extern "C" {

int orc_gauss01(int n, double* x, double* w) {
  std::vector<double> a, b;
  gauss01(n, a, b);
  std::copy(a.begin(), a.end(), x);
  std::copy(b.begin(), b.end(), w);
  return 0;
}

int orc_singular_rule(int n, int v, double* px, double* py, double* w) {
  std::vector<double> a, b, c;
  vertex_singular_rule(n, v, a, b, c);
  std::copy(a.begin(), a.end(), px);
  std::copy(b.begin(), b.end(), py);
  std::copy(c.begin(), c.end(), w);
  return (int)a.size();
}

// BEMProblem<3>::assemble_system, source/bem_problem.cc:106-590: loop over
// cells (:190), then over every collocation row i (:214); singular test
// (:223-230); regular 4x4 Gauss (:241-260) or vertex rule (:478-522);
// scatter into row i (:531-537). Serial, in the reference's loop order.
int orc_assemble(int N, const double* X, int C, const int* cells, const int* dn_ptr,
                 const int* dn_idx, int qorder, int sorder, double* Nm, double* Dm) {
  std::vector<double> px, py, w;
  gauss2d(qorder, px, py, w);
  std::vector<double> spx[4], spy[4], sw[4];
  for (int v = 0; v < 4; ++v) vertex_singular_rule(sorder, v, spx[v], spy[v], sw[v]);
  std::memset(Nm, 0, sizeof(double) * (size_t)N * N);
  std::memset(Dm, 0, sizeof(double) * (size_t)N * N);
  for (int c = 0; c < C; ++c) {
    const int* cell = cells + 4 * c;
    CellRule reg = cell_rule(X, cell, px, py, w);
    for (int i = 0; i < N; ++i) {
      int sing = -1;
      for (int j = 0; j < 4; ++j)
        if (in_set(dn_ptr, dn_idx, i, cell[j])) { sing = j; break; }
      double ln[4], ld[4];
      V3 xi = node(X, i);
      if (sing < 0) {
        local_row(reg, xi, ln, ld);
      } else {
        CellRule sr = cell_rule(X, cell, spx[sing], spy[sing], sw[sing]);
        local_row(sr, xi, ln, ld);
      }
      for (int j = 0; j < 4; ++j) {
        Nm[(size_t)i * N + cell[j]] += ln[j];
        Dm[(size_t)i * N + cell[j]] += ld[j];
      }
    }
  }
  return 0;
}

// Row-parallel variant (OpenMP over rows, cells in the reference order inside
// each row, so each entry is accumulated in the same order as orc_assemble).
// Assembles rows [r0, r1) only, into Nm/Dm of shape (r1-r0) x N.
int orc_assemble_rows(int N, const double* X, int C, const int* cells, const int* dn_ptr,
                      const int* dn_idx, int qorder, int sorder, int r0, int r1, double* Nm,
                      double* Dm) {
  std::vector<double> px, py, w;
  gauss2d(qorder, px, py, w);
  std::vector<double> spx[4], spy[4], sw[4];
  for (int v = 0; v < 4; ++v) vertex_singular_rule(sorder, v, spx[v], spy[v], sw[v]);
  std::vector<CellRule> reg(C);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < C; ++c) reg[c] = cell_rule(X, cells + 4 * c, px, py, w);
  const int R = r1 - r0;
  std::memset(Nm, 0, sizeof(double) * (size_t)R * N);
  std::memset(Dm, 0, sizeof(double) * (size_t)R * N);
#pragma omp parallel for schedule(dynamic, 4)
  for (int i = r0; i < r1; ++i) {
    double* nrow = Nm + (size_t)(i - r0) * N;
    double* drow = Dm + (size_t)(i - r0) * N;
    V3 xi = node(X, i);
    for (int c = 0; c < C; ++c) {
      const int* cell = cells + 4 * c;
      int sing = -1;
      for (int j = 0; j < 4; ++j)
        if (in_set(dn_ptr, dn_idx, i, cell[j])) { sing = j; break; }
      double ln[4], ld[4];
      if (sing < 0) {
        local_row(reg[c], xi, ln, ld);
      } else {
        CellRule sr = cell_rule(X, cell, spx[sing], spy[sing], sw[sing]);
        local_row(sr, xi, ln, ld);
      }
      for (int j = 0; j < 4; ++j) {
        nrow[cell[j]] += ln[j];
        drow[cell[j]] += ld[j];
      }
    }
  }
  return 0;
}

// BEMProblem<3>::compute_alpha, source/bem_problem.cc:594-618: alpha = N (-1).
int orc_alpha(int N, const double* Nm, double* alpha) {
  std::vector<double> ones(N, -1.0);
  matvec(N, Nm, ones.data(), alpha);
  return 0;
}

// BEMProblem<3>::compute_rhs, source/bem_problem.cc:673-706.
int orc_compute_rhs(int N, const double* Nm, const double* Dm, const double* alpha,
                    const unsigned char* mask, const double* src, double* dst) {
  std::vector<double> phi(N), dphi(N), t(N);
  for (int i = 0; i < N; ++i) {
    phi[i] = mask[i] ? src[i] : 0.0;
    dphi[i] = mask[i] ? 0.0 : src[i];
  }
  matvec(N, Nm, phi.data(), dst);
  for (int i = 0; i < N; ++i) dst[i] = -(dst[i] + phi[i] * alpha[i]);
  matvec(N, Dm, dphi.data(), t.data());
  for (int i = 0; i < N; ++i) dst[i] += t[i];
  return 0;
}

// BEMProblem<3>::vmult, source/bem_problem.cc:620-670.
int orc_vmult(int N, const double* Nm, const double* Dm, const double* alpha,
              const unsigned char* mask, const double* src, double* dst) {
  std::vector<double> phi(N), dphi(N), t(N);
  double linf = 0;
  for (int i = 0; i < N; ++i) {
    phi[i] = mask[i] ? 0.0 : src[i];
    dphi[i] = mask[i] ? src[i] : 0.0;
    linf = std::max(linf, (double)mask[i]);
  }
  matvec(N, Dm, dphi.data(), dst);
  matvec(N, Nm, phi.data(), t.data());
  for (int i = 0; i < N; ++i) dst[i] = -dst[i] + t[i] + phi[i] * alpha[i];
  if (linf < 1e-10) {
    double l2 = 0;
    for (int i = 0; i < N; ++i) l2 += dst[i] * dst[i];
    l2 = std::sqrt(l2);
    for (int i = 0; i < N; ++i) dst[i] -= l2;
  }
  return 0;
}

// BEMProblem<3>::compute_constraints, source/bem_problem.cc:990-1105 (after
// close()). Output: flags[N] (1 = constrained), inhom[N], and up to
// max_entries (row, col, coef) triples. Returns the number of entries or -1.
int orc_constraints(int N, const double* X, int C, const int* cells, int qorder,
                    const int* dn_ptr, const int* dn_idx, const unsigned char* mask,
                    const double* tmp_rhs, unsigned char* flags, double* inhom, int max_entries,
                    int* e_row, int* e_col, double* e_val) {
  Constraints c = build_constraints(N, X, C, cells, qorder, dn_ptr, dn_idx, mask, tmp_rhs);
  std::memset(flags, 0, N);
  for (int i = 0; i < N; ++i) inhom[i] = 0;
  int ne = 0;
  for (auto& kv : c.lines) {
    flags[kv.first] = 1;
    inhom[kv.first] = c.inhom[kv.first];
    for (auto& e : kv.second) {
      if (ne >= max_entries) return -1;
      e_row[ne] = kv.first;
      e_col[ne] = e.first;
      e_val[ne] = e.second;
      ++ne;
    }
  }
  return ne;
}

int orc_node_normals(int N, const double* X, int C, const int* cells, int qorder, double* nn) {
  node_normals(N, X, C, cells, qorder, nn);
  return 0;
}

int orc_surface_gradients(int N, const double* X, int C, const int* cells, int qorder,
                          const unsigned char* mask, const double* tmp_rhs, double* g) {
  surface_gradients(N, X, C, cells, qorder, mask, tmp_rhs, g);
  return 0;
}

// The constrained system matrix of solve_system (source/bem_problem.cc:821-895):
// rows of vmult's operator (no all-Neumann shift), constrained rows replaced by
// x_i - sum c_ij x_j (include/constrained_matrix.h:72-86); rhs from compute_rhs
// with distribute_rhs (:88-94).
int orc_system(int N, const double* X, int C, const int* cells, int qorder, const int* dn_ptr,
               const int* dn_idx, const double* Nm, const double* Dm, const double* alpha,
               const unsigned char* mask, const double* tmp_rhs, double* A, double* rhs) {
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      double v = mask[j] ? -Dm[(size_t)i * N + j] : Nm[(size_t)i * N + j];
      if (i == j && !mask[j]) v += alpha[i];
      A[(size_t)i * N + j] = v;
    }
  orc_compute_rhs(N, Nm, Dm, alpha, mask, tmp_rhs, rhs);
  Constraints c = build_constraints(N, X, C, cells, qorder, dn_ptr, dn_idx, mask, tmp_rhs);
  for (auto& kv : c.lines) {
    int i = kv.first;
    double* r = A + (size_t)i * N;
    for (int j = 0; j < N; ++j) r[j] = 0;
    r[i] = 1.0;
    for (auto& e : kv.second) r[e.first] -= e.second;
    rhs[i] = c.inhom[i];
  }
  return 0;
}

// solve_system with a dense direct solve of the constrained system (the
// converged answer of the reference's GMRES), then the unpack of
// source/bem_problem.cc:869-879. phi / dphi_dn are updated in place.
int orc_solve_system(int N, const double* X, int C, const int* cells, int qorder,
                     const int* dn_ptr, const int* dn_idx, const double* Nm, const double* Dm,
                     const double* alpha, const unsigned char* mask, const double* tmp_rhs,
                     double* phi, double* dphi_dn, double* sol_out) {
  std::vector<double> A((size_t)N * N), rhs(N);
  std::vector<int> piv(N);
  orc_system(N, X, C, cells, qorder, dn_ptr, dn_idx, Nm, Dm, alpha, mask, tmp_rhs, A.data(),
             rhs.data());
  int st = lu_factor(N, A.data(), piv.data());
  if (st) return st;
  lu_solve(N, A.data(), piv.data(), rhs.data());
  for (int i = 0; i < N; ++i) {
    if (mask[i] == 0) phi[i] = rhs[i];
    else dphi_dn[i] = rhs[i];
    if (sol_out) sol_out[i] = rhs[i];
  }
  return 0;
}

// Band preconditioner of source/bem_problem.cc:1107-1149: entries (j,i) with
// j in [i-band/2, i+band/2) of the system (Neumann column: N + alpha on the
// diagonal; Dirichlet column: -D), identity rows for constrained dofs; LU with
// partial pivoting in band storage (stands in for UMFPACK).
struct BandLU {
  int n = 0, kl = 0, ku = 0, ld = 0;
  std::vector<double> ab;  // column-major band, LAPACK gbtrf layout
  std::vector<int> piv;
  double& at(int i, int j) { return ab[(size_t)j * ld + (kl + ku + i - j)]; }
};

int band_factor(BandLU& B) {
  int n = B.n, kl = B.kl, ku = B.ku;
  int kv = ku + kl;
  B.piv.assign(n, 0);
  for (int j = 0; j < n; ++j) {
    int km = std::min(kl, n - 1 - j);
    int p = j;
    double m = std::fabs(B.at(j, j));
    for (int i = j + 1; i <= j + km; ++i)
      if (std::fabs(B.at(i, j)) > m) { m = std::fabs(B.at(i, j)); p = i; }
    B.piv[j] = p;
    if (m == 0.0) return 5;
    int jmax = std::min(n - 1, j + kv);
    if (p != j)
      for (int c = j; c <= jmax; ++c) std::swap(B.at(j, c), B.at(p, c));
    double inv = 1.0 / B.at(j, j);
    for (int i = j + 1; i <= j + km; ++i) B.at(i, j) *= inv;
    for (int c = j + 1; c <= jmax; ++c) {
      double u = B.at(j, c);
      if (u == 0.0) continue;
      for (int i = j + 1; i <= j + km; ++i) B.at(i, c) -= B.at(i, j) * u;
    }
  }
  return 0;
}

void band_solve(BandLU& B, double* x) {
  int n = B.n, kl = B.kl, kv = B.ku + B.kl;
  for (int j = 0; j < n; ++j) {
    if (B.piv[j] != j) std::swap(x[j], x[B.piv[j]]);
    int km = std::min(kl, n - 1 - j);
    for (int i = j + 1; i <= j + km; ++i) x[i] -= B.at(i, j) * x[j];
  }
  for (int j = n - 1; j >= 0; --j) {
    x[j] /= B.at(j, j);
    int i0 = std::max(0, j - kv);
    for (int i = i0; i < j; ++i) x[i] -= B.at(i, j) * x[j];
  }
}

// Reference-faithful solve_system: left-preconditioned GMRES(restart) with
// modified Gram-Schmidt and Givens rotations on the ConstrainedOperator, band
// preconditioner, absolute tolerance on the preconditioned residual, at most
// max_steps iterations (deal.II SolverGMRES / SolverControl semantics).
// Returns 0, or 6 if not converged. iters/res report the outcome.
int orc_solve_system_gmres(int N, const double* X, int C, const int* cells, int qorder,
                           const int* dn_ptr, const int* dn_idx, const double* Nm,
                           const double* Dm, const double* alpha, const unsigned char* mask,
                           const double* tmp_rhs, int restart, int max_steps, double tol,
                           int band, double* phi, double* dphi_dn, int* iters, double* res) {
  std::vector<double> rhs(N);
  orc_compute_rhs(N, Nm, Dm, alpha, mask, tmp_rhs, rhs.data());
  Constraints cons = build_constraints(N, X, C, cells, qorder, dn_ptr, dn_idx, mask, tmp_rhs);
  for (auto& kv : cons.lines) rhs[kv.first] = cons.inhom[kv.first];
  auto op = [&](const double* src, double* dst) {
    orc_vmult(N, Nm, Dm, alpha, mask, src, dst);
    for (auto& kv : cons.lines) {
      double v = src[kv.first];
      for (auto& e : kv.second) v -= e.second * src[e.first];
      dst[kv.first] = v;
    }
  };
  // band preconditioner
  BandLU B;
  B.n = N;
  B.kl = band / 2;
  B.ku = band / 2;
  B.ld = 2 * B.kl + B.ku + 1;
  B.ab.assign((size_t)B.ld * N, 0.0);
  for (int i = 0; i < N; ++i) {
    if (cons.lines.count(i)) B.at(i, i) = 1.0;
    for (int j = std::max(i - band / 2, 0); j < std::min(i + band / 2, N); ++j) {
      if (cons.lines.count(j)) continue;
      if (mask[i] == 0) {
        double v = Nm[(size_t)j * N + i];
        if (i == j) v += alpha[i];
        B.at(j, i) = v;
      } else {
        B.at(j, i) = -Dm[(size_t)j * N + i];
      }
    }
  }
  int st = band_factor(B);
  if (st) return st;
  std::vector<double> x(N, 0.0), r(N), w(N);
  std::vector<std::vector<double>> V(restart + 1, std::vector<double>(N));
  std::vector<double> H((size_t)(restart + 1) * restart), cs(restart), sn(restart), g(restart + 1);
  int it = 0;
  double rn = 0;
  bool conv = false;
  while (it < max_steps) {
    op(x.data(), r.data());
    for (int i = 0; i < N; ++i) r[i] = rhs[i] - r[i];
    band_solve(B, r.data());
    rn = 0;
    for (int i = 0; i < N; ++i) rn += r[i] * r[i];
    rn = std::sqrt(rn);
    if (rn < tol) { conv = true; break; }
    for (int i = 0; i < N; ++i) V[0][i] = r[i] / rn;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = rn;
    int k = 0;
    for (; k < restart && it < max_steps; ++k, ++it) {
      op(V[k].data(), w.data());
      band_solve(B, w.data());
      for (int j = 0; j <= k; ++j) {
        double h = 0;
        for (int i = 0; i < N; ++i) h += w[i] * V[j][i];
        H[(size_t)j * restart + k] = h;
        for (int i = 0; i < N; ++i) w[i] -= h * V[j][i];
      }
      double hn = 0;
      for (int i = 0; i < N; ++i) hn += w[i] * w[i];
      hn = std::sqrt(hn);
      H[(size_t)(k + 1) * restart + k] = hn;
      if (hn > 0)
        for (int i = 0; i < N; ++i) V[k + 1][i] = w[i] / hn;
      for (int j = 0; j < k; ++j) {
        double a = H[(size_t)j * restart + k], b = H[(size_t)(j + 1) * restart + k];
        H[(size_t)j * restart + k] = cs[j] * a + sn[j] * b;
        H[(size_t)(j + 1) * restart + k] = -sn[j] * a + cs[j] * b;
      }
      double a = H[(size_t)k * restart + k], b = H[(size_t)(k + 1) * restart + k];
      double d = std::sqrt(a * a + b * b);
      cs[k] = a / d;
      sn[k] = b / d;
      H[(size_t)k * restart + k] = d;
      H[(size_t)(k + 1) * restart + k] = 0;
      g[k + 1] = -sn[k] * g[k];
      g[k] = cs[k] * g[k];
      rn = std::fabs(g[k + 1]);
      if (rn < tol) { ++k; ++it; conv = true; break; }
    }
    // x += V y
    std::vector<double> y(k);
    for (int j = k - 1; j >= 0; --j) {
      double s = g[j];
      for (int l = j + 1; l < k; ++l) s -= H[(size_t)j * restart + l] * y[l];
      y[j] = s / H[(size_t)j * restart + j];
    }
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < N; ++i) x[i] += y[j] * V[j][i];
    if (conv) break;
  }
  if (iters) *iters = it;
  if (res) *res = rn;
  for (int i = 0; i < N; ++i) {
    if (mask[i] == 0) phi[i] = x[i];
    else dphi_dn[i] = x[i];
  }
  return conv ? 0 : 6;
}

// Hull force F_x = sum over the given cells of  integral p n_x dS  with
// p = -(U . grad phi + |grad phi|^2 / 2), grad phi = surface gradient of the
// Q1 interpolant of phi + (interpolated dphi/dn) n, n the cell normal
// (pointing out of the fluid), 4x4 Gauss (the steady, rho = 1, g = 0 form of
// source/free_surface.cc:6936-6942).
double orc_hull_force(int N, const double* X, int nh, const int* hull_cells_nodes, int qorder,
                      const double* U, const double* phi, const double* dphi_dn) {
  (void)N;
  std::vector<double> px, py, w;
  gauss2d(qorder, px, py, w);
  V3 u = {U[0], U[1], U[2]};
  double F = 0;
  for (int c = 0; c < nh; ++c) {
    const int* cell = hull_cells_nodes + 4 * c;
    CellRule r = cell_rule(X, cell, px, py, w);
    for (size_t q = 0; q < px.size(); ++q) {
      const QPoint& Q = r.qp[q];
      double gx = 0, ge = 0, pn = 0;
      for (int a = 0; a < 4; ++a) {
        gx += Q.dphi[a][0] * phi[cell[a]];
        ge += Q.dphi[a][1] * phi[cell[a]];
        pn += Q.phi[a] * dphi_dn[cell[a]];
      }
      double g11 = dot(Q.jx, Q.jx), g12 = dot(Q.jx, Q.je), g22 = dot(Q.je, Q.je);
      double det = g11 * g22 - g12 * g12;
      double c1 = (g22 * gx - g12 * ge) / det, c2 = (-g12 * gx + g11 * ge) / det;
      V3 grad = add(add(scl(c1, Q.jx), scl(c2, Q.je)), scl(pn, Q.n));
      double p = -(dot(u, grad) + 0.5 * dot(grad, grad));
      F += p * Q.n.x * Q.det * r.w[q];
    }
  }
  return F;
}

int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// Threads of the OpenMP row loops from here on (the CPU-baseline legs time
// 1 thread and all host threads in one process).
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

}  // extern "C"
