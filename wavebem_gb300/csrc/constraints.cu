// Double-node constraints of the collocation system and the L2 projections
// they need, on the host (all O(N) sparse work):
//   - BEMProblem<3>::compute_constraints (source/bem_problem.cc:990-1105) with
//     deal.II ConstraintMatrix semantics (add_line idempotent, close()
//     resolving entries that point at constrained dofs);
//   - ComputationalDomain::compute_normals (source/computational_domain.cc:
//     1525-1620) and BEMProblem::compute_surface_gradients
//     (source/bem_problem.cc:1153-1293): L2 projections onto Q1 with the
//     consistent mass matrix;
//   - the adjoint of the constraint inhomogeneities with respect to the node
//     positions and the known data (the sharp Dirichlet-Dirichlet lines depend
//     on both through the projected normals and surface gradients).
// Everything here works in the caller's dof numbering; the upload to the
// internal order happens in build_constraints.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <map>
#include <vector>
#include "context.h"
#include "host_util.h"

namespace wbem {

namespace {

// Gauss-Legendre rule of the handle (the regular panel rule's line rule).
void line_rule(const wbem_context* h, std::vector<double>& x, std::vector<double>& w) {
  x.assign(h->gauss_x, h->gauss_x + h->gauss_n);
  w.assign(h->gauss_w, h->gauss_w + h->gauss_n);
}

// ---------------------------------------------------------------- sparse
struct Csr {
  int n = 0;
  std::vector<int> ptr, idx;
  std::vector<double> val;
  void mv(const double* x, double* y) const {
    for (int i = 0; i < n; ++i) {
      double s = 0;
      for (int k = ptr[i]; k < ptr[i + 1]; ++k) s += val[k] * x[idx[k]];
      y[i] = s;
    }
  }
};

// Jacobi-preconditioned CG on the SPD mass matrix to a relative residual of
// 1e-15 (stands in for the reference's sparse direct solve).
void pcg(const Csr& M, const double* b, double* x) {
  const int n = M.n;
  std::vector<double> r(b, b + n), z(n), p(n), Ap(n), dinv(n);
  for (int i = 0; i < n; ++i) {
    double d = 0;
    for (int k = M.ptr[i]; k < M.ptr[i + 1]; ++k)
      if (M.idx[k] == i) d = M.val[k];
    dinv[i] = 1.0 / d;
    x[i] = 0;
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
    M.mv(p.data(), Ap.data());
    double pAp = 0;
    for (int i = 0; i < n; ++i) pAp += p[i] * Ap[i];
    const double al = rz / pAp;
    double rn = 0;
    for (int i = 0; i < n; ++i) {
      x[i] += al * p[i];
      r[i] -= al * Ap[i];
      rn += r[i] * r[i];
    }
    if (std::sqrt(rn) < 1e-15 * bn) break;
    double rz2 = 0;
    for (int i = 0; i < n; ++i) {
      z[i] = dinv[i] * r[i];
      rz2 += r[i] * z[i];
    }
    const double be = rz2 / rz;
    rz = rz2;
    for (int i = 0; i < n; ++i) p[i] = z[i] + be * p[i];
  }
}

// Three solves M x_d = b_d, b and x node-major (3 * i + d).
void pcg3(const Csr& M, const std::vector<double>& b, std::vector<double>& x) {
  const int n = M.n;
  std::vector<double> bd(n), xd(n);
  x.assign(3 * (size_t)n, 0.0);
  for (int d = 0; d < 3; ++d) {
    for (int i = 0; i < n; ++i) bd[i] = b[3 * (size_t)i + d];
    pcg(M, bd.data(), xd.data());
    for (int i = 0; i < n; ++i) x[3 * (size_t)i + d] = xd[i];
  }
}

// ----------------------------------------------------------- Q1 geometry
// Forward-mode dual number with K derivative slots (the adjoint of the L2
// projections differentiates per-panel expressions with respect to the 12
// vertex coordinates and the 4 vertex values of the data).
template <int K>
struct Dual {
  double v = 0;
  double d[K] = {};
  Dual() = default;
  Dual(double x) : v(x) {}  // NOLINT: constants promote implicitly
};
template <int K> Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v + b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int K> Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v - b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int K> Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v * b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <int K> Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v / b.v);
  for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
  return r;
}
inline double dsqrt(double a) { return std::sqrt(a); }
template <int K> Dual<K> dsqrt(const Dual<K>& a) {
  Dual<K> r(std::sqrt(a.v));
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] / (2.0 * r.v);
  return r;
}

// Per quadrature point of a Q1 panel: shape values, the cross product of the
// Jacobian columns (normal times area density) and the tangential gradient
// of the Q1 interpolant of f. P: vertex coordinates, f: vertex values.
template <typename T>
struct PanelPoint {
  double ph[4];
  T cr[3], area, grad[3];
};

template <typename T>
PanelPoint<T> panel_point(const T P[4][3], const T f[4], double s, double u) {
  PanelPoint<T> q;
  q.ph[0] = (1 - s) * (1 - u);
  q.ph[1] = s * (1 - u);
  q.ph[2] = (1 - s) * u;
  q.ph[3] = s * u;
  T jx[3], je[3];
  for (int d = 0; d < 3; ++d) {
    jx[d] = T(1 - u) * (P[1][d] - P[0][d]) + T(u) * (P[3][d] - P[2][d]);
    je[d] = T(1 - s) * (P[2][d] - P[0][d]) + T(s) * (P[3][d] - P[1][d]);
  }
  q.cr[0] = jx[1] * je[2] - jx[2] * je[1];
  q.cr[1] = jx[2] * je[0] - jx[0] * je[2];
  q.cr[2] = jx[0] * je[1] - jx[1] * je[0];
  q.area = dsqrt(q.cr[0] * q.cr[0] + q.cr[1] * q.cr[1] + q.cr[2] * q.cr[2]);
  const T gx = T(-(1 - u)) * f[0] + T(1 - u) * f[1] + T(-u) * f[2] + T(u) * f[3];
  const T ge = T(-(1 - s)) * f[0] + T(-s) * f[1] + T(1 - s) * f[2] + T(s) * f[3];
  T g11 = jx[0] * jx[0] + jx[1] * jx[1] + jx[2] * jx[2];
  T g12 = jx[0] * je[0] + jx[1] * je[1] + jx[2] * je[2];
  T g22 = je[0] * je[0] + je[1] * je[1] + je[2] * je[2];
  const T det = g11 * g22 - g12 * g12;
  const T c1 = (g22 * gx - g12 * ge) / det, c2 = (T(0.0) - g12 * gx + g11 * ge) / det;
  for (int d = 0; d < 3; ++d) q.grad[d] = c1 * jx[d] + c2 * je[d];
  return q;
}

Csr mass_matrix(const wbem_context* h, const double* X) {
  const int N = h->N, C = h->C;
  std::vector<double> x, w;
  line_rule(h, x, w);
  const int q1 = (int)x.size();
  std::vector<std::map<int, double>> rows(N);
  const double f0[4] = {0, 0, 0, 0};
  for (int c = 0; c < C; ++c) {
    const int* cc = &h->cells[4 * (size_t)c];
    double P[4][3];
    for (int a = 0; a < 4; ++a)
      for (int d = 0; d < 3; ++d) P[a][d] = X[3 * (size_t)cc[a] + d];
    for (int b = 0; b < q1; ++b)
      for (int a = 0; a < q1; ++a) {
        const PanelPoint<double> q = panel_point<double>(P, f0, x[a], x[b]);
        const double jxw = q.area * w[a] * w[b];
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 4; ++j) rows[cc[i]][cc[j]] += q.ph[i] * q.ph[j] * jxw;
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

// Right-hand sides of the two projections, node-major: rn = int phi_a n dS,
// rg = int phi_a grad_s f dS with f = tmp_rhs on Dirichlet nodes, 0 elsewhere.
void projection_rhs(const wbem_context* h, const double* X, const double* tmp_rhs,
                    std::vector<double>* rn, std::vector<double>* rg) {
  const int N = h->N, C = h->C;
  std::vector<double> x, w;
  line_rule(h, x, w);
  const int q1 = (int)x.size();
  if (rn) rn->assign(3 * (size_t)N, 0.0);
  if (rg) rg->assign(3 * (size_t)N, 0.0);
  for (int c = 0; c < C; ++c) {
    const int* cc = &h->cells[4 * (size_t)c];
    double P[4][3], f[4];
    for (int a = 0; a < 4; ++a) {
      for (int d = 0; d < 3; ++d) P[a][d] = X[3 * (size_t)cc[a] + d];
      f[a] = (tmp_rhs && h->mask[cc[a]]) ? tmp_rhs[cc[a]] : 0.0;
    }
    for (int b = 0; b < q1; ++b)
      for (int a = 0; a < q1; ++a) {
        const PanelPoint<double> q = panel_point<double>(P, f, x[a], x[b]);
        const double jxw = q.area * w[a] * w[b];
        for (int i = 0; i < 4; ++i)
          for (int d = 0; d < 3; ++d) {
            if (rn) (*rn)[3 * (size_t)cc[i] + d] += q.ph[i] * (q.cr[d] / q.area) * jxw;
            if (rg) (*rg)[3 * (size_t)cc[i] + d] += q.ph[i] * q.grad[d] * jxw;
          }
      }
  }
}

// --------------------------------------------------------- constraint lines
// Kinds of raw inhomogeneity a line can be given before close(): the known
// datum of a Dirichlet node (Dirichlet-Neumann pair) or one of the two
// sharp-edge formulas of a Dirichlet-Dirichlet pair (i = first node, o = the
// other).
enum SrcKind { kSrcData = 0, kSrcSharpThis = 1, kSrcSharpOther = 2 };
struct Src {
  int kind, i, o;
};

// deal.II ConstraintMatrix semantics. Every line's inhomogeneity is also kept
// as a linear combination of raw sources (the same operations applied to the
// source coefficients), so that the adjoint can route d(inhomogeneity) back to
// the quantities each raw value came from.
struct Lines {
  std::map<int, std::vector<std::pair<int, double>>> l;
  std::map<int, double> inh;
  std::map<int, std::map<int, double>> src;  // line -> (source id -> coefficient)
  std::vector<Src> sources;
  void add_line(int i) {
    if (!l.count(i)) {
      l[i] = {};
      inh[i] = 0;
      src[i] = {};
    }
  }
  void add_entry(int i, int j, double v) {
    for (auto& e : l[i])
      if (e.first == j) return;
    l[i].push_back({j, v});
  }
  void set_inhomogeneity(int i, double v, Src s) {
    inh[i] = v;
    sources.push_back(s);
    src[i] = {{(int)sources.size() - 1, 1.0}};
  }
  void close() {
    for (int pass = 0; pass < 64; ++pass) {
      bool changed = false;
      for (auto& kv : l) {
        std::vector<std::pair<int, double>> out;
        double v = inh[kv.first];
        std::map<int, double> sv = src[kv.first];
        for (auto& e : kv.second) {
          auto it = l.find(e.first);
          if (it != l.end() && e.first != kv.first) {
            changed = true;
            v += e.second * inh[e.first];
            for (auto& s : src[e.first]) sv[s.first] += e.second * s.second;
            for (auto& e2 : it->second) out.push_back({e2.first, e.second * e2.second});
          } else {
            out.push_back(e);
          }
        }
        std::map<int, double> m;
        for (auto& e : out) m[e.first] += e.second;
        kv.second.assign(m.begin(), m.end());
        inh[kv.first] = v;
        src[kv.first].swap(sv);
      }
      if (!changed) break;
    }
  }
};

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// The inhomogeneity of a sharp Dirichlet-Dirichlet line of node a paired with
// node b (source/bem_problem.cc:1058-1074): with c = n_a . n_b,
//   (g_b . n_a + (g_a . n_b) c) / (1 - c^2).
// "this" (the first node's line) is sharp(i, o), "other" is sharp(o, i).
double sharp_value(const double* na, const double* nb, const double* ga, const double* gb) {
  const double c = dot3(na, nb);
  return (1.0 / (1.0 - c * c)) * (dot3(gb, na) + dot3(ga, nb) * c);
}

// Its partial derivatives, scaled by mu, added to the node-major adjoints of
// the normals (mn) and gradients (mg).
void sharp_adjoint(int a, int b, const double* na, const double* nb, const double* ga,
                   const double* gb, double mu, double* mn, double* mg) {
  const double c = dot3(na, nb);
  const double s = 1.0 / (1.0 - c * c);
  const double A = dot3(gb, na) + dot3(ga, nb) * c;
  // d value / d c, with c's own dependence on the normals added below
  const double dc = 2.0 * c * s * s * A + s * dot3(ga, nb);
  for (int d = 0; d < 3; ++d) {
    mn[3 * (size_t)a + d] += mu * (s * gb[d] + dc * nb[d]);
    mn[3 * (size_t)b + d] += mu * (s * c * ga[d] + dc * na[d]);
    mg[3 * (size_t)b + d] += mu * s * na[d];
    mg[3 * (size_t)a + d] += mu * s * c * nb[d];
  }
}

// Projections the lines need, for the handle's current nodes.
struct Projections {
  bool have = false;
  std::vector<double> nt;  // unnormalised projected normals (node-major)
  std::vector<double> n;   // normalised
  std::vector<double> g;   // projected surface gradients of the Dirichlet data
};

bool needs_projections(const wbem_context* h) {
  const auto& m = h->mask;
  const auto& P = h->dn_ptr;
  const auto& I = h->dn_idx;
  for (int i = 0; i < h->N; ++i)
    if (m[i])
      for (int k = P[i]; k < P[i + 1]; ++k)
        if (I[k] != i && m[I[k]]) return true;
  return false;
}

void project_normals(wbem_context* h, const Csr& M, std::vector<double>& nt, std::vector<double>& n) {
  std::vector<double> rn;
  projection_rhs(h, h->X.data(), nullptr, &rn, nullptr);
  pcg3(M, rn, nt);
  n = nt;
  for (int i = 0; i < h->N; ++i) {
    double* v = &n[3 * (size_t)i];
    const double l = std::sqrt(dot3(v, v));
    for (int d = 0; d < 3; ++d) v[d] /= l;
  }
}

void project_gradients(wbem_context* h, const Csr& M, const double* tmp_rhs, std::vector<double>& g) {
  std::vector<double> rg;
  projection_rhs(h, h->X.data(), tmp_rhs, nullptr, &rg);
  pcg3(M, rg, g);
}

// The constraint lines of source/bem_problem.cc:1030-1105 for tmp_rhs, after
// close(); pr receives the projections when Dirichlet-Dirichlet pairs exist.
void make_lines(wbem_context* h, const double* tmp_rhs, Lines& c, Projections& pr) {
  const int N = h->N;
  const auto& m = h->mask;
  const auto& P = h->dn_ptr;
  const auto& I = h->dn_idx;
  pr.have = needs_projections(h);
  if (pr.have) {
    const Csr M = mass_matrix(h, h->X.data());
    project_normals(h, M, pr.nt, pr.n);
    project_gradients(h, M, tmp_rhs, pr.g);
  }
  for (int i = 0; i < N; ++i) {
    int first = I[P[i]];
    for (int k = P[i]; k < P[i + 1]; ++k)
      if (m[I[k]] == 1) {
        first = I[k];
        break;
      }
    if (i != first) continue;
    for (int k = P[i]; k < P[i + 1]; ++k) {
      const int o = I[k];
      if (o == i) continue;
      if (m[i] == 1) {
        if (m[o] == 1) {
          const double* ni = &pr.n[3 * (size_t)i];
          const double* no = &pr.n[3 * (size_t)o];
          const double dd = std::sqrt((ni[0] - no[0]) * (ni[0] - no[0]) + (ni[1] - no[1]) * (ni[1] - no[1]) +
                                      (ni[2] - no[2]) * (ni[2] - no[2]));
          if (dd < 1e-4) {  // flat edge: equal normal derivatives
            c.add_line(o);
            c.add_entry(o, i, 1.0);
          } else {  // sharp edge: both normal derivatives from the surface gradients
            const double* gi = &pr.g[3 * (size_t)i];
            const double* go = &pr.g[3 * (size_t)o];
            c.add_line(o);
            c.add_line(i);
            c.set_inhomogeneity(i, sharp_value(ni, no, gi, go), Src{kSrcSharpThis, i, o});
            c.add_line(o);
            c.set_inhomogeneity(o, sharp_value(no, ni, go, gi), Src{kSrcSharpOther, i, o});
          }
        } else {  // Dirichlet-Neumann: the Neumann copy's phi is the datum
          c.add_line(o);
          c.set_inhomogeneity(o, tmp_rhs[i], Src{kSrcData, i, o});
        }
      } else {  // Neumann-Neumann: equal potentials
        c.add_line(o);
        c.add_entry(o, i, 1.0);
      }
    }
  }
  c.close();
}

// d/dX and d/df of one panel's share of
//   L = psi_n . (rn - M nt) + psi_g . (rg - M g)
// (psi_*, nt, g node-major, constants); adds to dX (node-major, caller
// order) and df (per node, the derivative with respect to f = tmp_rhs on
// Dirichlet nodes).
void panel_projection_adjoint(const wbem_context* h, int c, const std::vector<double>& psin,
                              const std::vector<double>& psig, const std::vector<double>& nt,
                              const std::vector<double>& g, const double* tmp_rhs,
                              const std::vector<double>& x, const std::vector<double>& w,
                              std::vector<double>& dX, std::vector<double>& df) {
  using D = Dual<16>;
  const int* cc = &h->cells[4 * (size_t)c];
  D P[4][3], f[4];
  for (int a = 0; a < 4; ++a) {
    for (int d = 0; d < 3; ++d) {
      P[a][d] = D(h->X[3 * (size_t)cc[a] + d]);
      P[a][d].d[3 * a + d] = 1.0;
    }
    f[a] = D(h->mask[cc[a]] ? tmp_rhs[cc[a]] : 0.0);
    f[a].d[12 + a] = 1.0;
  }
  const int q1 = (int)x.size();
  D L(0.0);
  for (int b = 0; b < q1; ++b)
    for (int a = 0; a < q1; ++a) {
      const PanelPoint<D> q = panel_point<D>(P, f, x[a], x[b]);
      const D jxw = q.area * D(w[a] * w[b]);
      for (int i = 0; i < 4; ++i) {
        const double* pn = &psin[3 * (size_t)cc[i]];
        const double* pg = &psig[3 * (size_t)cc[i]];
        for (int d = 0; d < 3; ++d)
          L = L + D(q.ph[i]) * ((D(pn[d]) * (q.cr[d] / q.area) + D(pg[d]) * q.grad[d]) * jxw);
        // - sum_j M_ij (psi_n,i . nt_j + psi_g,i . g_j)
        double mm = 0.0;
        for (int j = 0; j < 4; ++j)
          mm += q.ph[j] * (dot3(pn, &nt[3 * (size_t)cc[j]]) + dot3(pg, &g[3 * (size_t)cc[j]]));
        L = L - D(q.ph[i] * mm) * jxw;
      }
    }
  for (int a = 0; a < 4; ++a) {
    for (int d = 0; d < 3; ++d) dX[3 * (size_t)cc[a] + d] += L.d[3 * a + d];
    if (h->mask[cc[a]]) df[cc[a]] += L.d[12 + a];
  }
}

}  // namespace

// BEMProblem<3>::compute_constraints for tmp_rhs (caller order); uploads the
// lines in the internal order. Lines and entries unchanged since the last
// upload (the usual case from one solve_system to the next) upload only the
// inhomogeneities.
int build_constraints(wbem_context* h, const double* tmp_rhs) {
  const int N = h->N;
  Lines c;
  Projections pr;
  make_lines(h, tmp_rhs, c, pr);
  const auto& ip = h->iperm;
  std::vector<std::pair<int, int>> rows;  // (internal row, caller row)
  for (auto& kv : c.l) rows.push_back({ip[kv.first], kv.first});
  std::sort(rows.begin(), rows.end());
  std::vector<int> crow, cptr{0}, ccol;
  std::vector<double> cval, cinh;
  for (auto& r : rows) {
    crow.push_back(r.first);
    cinh.push_back(c.inh[r.second]);
    for (auto& e : c.l[r.second]) {
      ccol.push_back(ip[e.first]);
      cval.push_back(e.second);
    }
    cptr.push_back((int)ccol.size());
  }
  h->n_crows = (int)crow.size();
  if (h->d_cinh && h->d_cflag && crow == h->c_crow && cptr == h->c_cptr && ccol == h->c_ccol &&
      cval == h->c_cval) {
    if (!cinh.empty()) {
      WB_CU(cudaMemcpyAsync(h->d_cinh, cinh.data(), sizeof(double) * cinh.size(), cudaMemcpyHostToDevice,
                            h->stream));
      WB_CU(cudaStreamSynchronize(h->stream));
    }
    return WBEM_OK;
  }
  std::vector<uint8_t> cflag(N, 0);
  std::vector<int> cptr_full(N + 1, 0), ccol_full;
  std::vector<double> cval_full;
  std::vector<std::vector<std::pair<int, double>>> byrow(N);
  for (size_t k = 0; k < crow.size(); ++k) {
    cflag[crow[k]] = 1;
    for (int e = cptr[k]; e < cptr[k + 1]; ++e) byrow[crow[k]].push_back({ccol[e], cval[e]});
  }
  for (int i = 0; i < N; ++i) {
    for (auto& e : byrow[i]) {
      ccol_full.push_back(e.first);
      cval_full.push_back(e.second);
    }
    cptr_full[i + 1] = (int)ccol_full.size();
  }
  // transposed entries: for column j, the constrained rows i with entry c_ij
  std::vector<int> tptr(N + 1, 0), tsrc;
  std::vector<double> tval;
  std::vector<std::vector<std::pair<int, double>>> bycol(N);
  for (int i = 0; i < N; ++i)
    for (auto& e : byrow[i]) bycol[e.first].push_back({i, e.second});
  for (int j = 0; j < N; ++j) {
    for (auto& e : bycol[j]) {
      tsrc.push_back(e.first);
      tval.push_back(e.second);
    }
    tptr[j + 1] = (int)tsrc.size();
  }
  WB_CHK(upload(h, &h->d_crow, crow));
  WB_CHK(upload(h, &h->d_cptr, cptr));
  WB_CHK(upload(h, &h->d_ccol, ccol));
  WB_CHK(upload(h, &h->d_cval, cval));
  WB_CHK(upload(h, &h->d_cinh, cinh));
  WB_CHK(upload(h, &h->d_cflag, cflag));
  WB_CHK(upload(h, &h->d_cptr_full, cptr_full));
  WB_CHK(upload(h, &h->d_ccol_full, ccol_full));
  WB_CHK(upload(h, &h->d_cval_full, cval_full));
  WB_CHK(upload(h, &h->d_tptr, tptr));
  WB_CHK(upload(h, &h->d_tsrc, tsrc));
  WB_CHK(upload(h, &h->d_tval, tval));
  h->c_crow.swap(crow);
  h->c_cptr.swap(cptr);
  h->c_ccol.swap(ccol);
  h->c_cval.swap(cval);
  return WBEM_OK;
}

// ComputationalDomain::compute_normals: normalised L2-projected normals,
// node-major N x 3, caller order.
void node_normals(wbem_context* h, std::vector<double>& n) {
  const Csr M = mass_matrix(h, h->X.data());
  std::vector<double> nt;
  project_normals(h, M, nt, n);
}

// BEMProblem::compute_surface_gradients: L2-projected surface gradients of
// tmp_rhs on the Dirichlet nodes (zero elsewhere), node-major N x 3.
void surface_gradients(wbem_context* h, const double* tmp_rhs, std::vector<double>& g) {
  const Csr M = mass_matrix(h, h->X.data());
  project_gradients(h, M, tmp_rhs, g);
}

// Adjoint of the constraint inhomogeneities: with lam (caller order) the
// transposed solve's solution, every constrained line l adds
// lam_l * d(inh_l) to the derivatives. Data lines route to the known data;
// sharp Dirichlet-Dirichlet lines route through the projected normals and
// surface gradients to the node positions (dJ_dX, node-major) and to the
// Dirichlet data (dJ_db).
void constraints_adjoint(wbem_context* h, const double* tmp_rhs, const double* lam, double* dJ_dX,
                         double* dJ_db) {
  const int N = h->N;
  Lines c;
  Projections pr;
  make_lines(h, tmp_rhs, c, pr);
  std::vector<double> mu(c.sources.size(), 0.0);
  for (auto& kv : c.src)
    for (auto& s : kv.second) mu[s.first] += lam[kv.first] * s.second;
  std::vector<double> mn, mg;
  bool sharp = false;
  for (size_t s = 0; s < c.sources.size(); ++s) {
    const Src& src = c.sources[s];
    if (mu[s] == 0.0) continue;
    if (src.kind == kSrcData) {
      dJ_db[src.i] += mu[s];
      continue;
    }
    if (!sharp) {
      mn.assign(3 * (size_t)N, 0.0);
      mg.assign(3 * (size_t)N, 0.0);
      sharp = true;
    }
    // sharp(a, b): this = sharp(i, o), other = sharp(o, i)
    const int a = src.kind == kSrcSharpThis ? src.i : src.o;
    const int b = src.kind == kSrcSharpThis ? src.o : src.i;
    sharp_adjoint(a, b, &pr.n[3 * (size_t)a], &pr.n[3 * (size_t)b], &pr.g[3 * (size_t)a],
                  &pr.g[3 * (size_t)b], mu[s], mn.data(), mg.data());
  }
  if (!sharp) return;
  // through the normalisation n = nt / |nt|
  std::vector<double> mnt(3 * (size_t)N);
  for (int i = 0; i < N; ++i) {
    const double* v = &pr.nt[3 * (size_t)i];
    const double* n = &pr.n[3 * (size_t)i];
    const double* m = &mn[3 * (size_t)i];
    const double l = std::sqrt(dot3(v, v)), nm = dot3(n, m);
    for (int d = 0; d < 3; ++d) mnt[3 * (size_t)i + d] = (m[d] - n[d] * nm) / l;
  }
  // through the projections nt = M^-1 rn(X), g = M^-1 rg(X, b)
  const Csr M = mass_matrix(h, h->X.data());
  std::vector<double> psin, psig;
  pcg3(M, mnt, psin);
  pcg3(M, mg, psig);
  std::vector<double> x, w;
  line_rule(h, x, w);
  std::vector<double> dX(3 * (size_t)N, 0.0), df(N, 0.0);
  for (int cell = 0; cell < h->C; ++cell)
    panel_projection_adjoint(h, cell, psin, psig, pr.nt, pr.g, tmp_rhs, x, w, dX, df);
  for (size_t k = 0; k < dX.size(); ++k) dJ_dX[k] += dX[k];
  for (int i = 0; i < N; ++i) dJ_db[i] += df[i];
}

}  // namespace wbem
