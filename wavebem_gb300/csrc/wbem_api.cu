// C ABI of the library (include/wbem.h): host orchestration of the device
// kernels. Host work here is limited to mesh topology bookkeeping (dof
// renumbering, panel lists, double-node sets, constraint lines), argument
// validation and the small least-squares updates of GMRES; every O(N^2) or
// O(N C) operation runs on the GPU.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <set>
#include <unordered_map>
#include <vector>
#include "context.h"
#include "host_util.h"
#include "fma_tree.h"
#include "quadrature_rules.h"
#include "../../include/wbem_kernels.h"

using namespace wbem;

namespace wbem {
cudaError_t upload_quadrature_fp64(const QuadTables& t);
cudaError_t upload_quadrature_mixed(const QuadTables& t);
cudaError_t upload_quadrature_adjoint(const QuadTables& t);
int solve_mixed(wbem_context* h, const double* d_rhs, double* d_x, int transpose);
void free_lu(wbem_context* h);
int assemble_mixed(wbem_context* h);
int factor_mixed(wbem_context* h);
void free_mixed(wbem_context* h);
int adjoint_force(wbem_context* h, const int* hull_cells, int n_hull, const double* U, int dir,
                  double* dF_dX, double* dF_drhs);
int adjoint_objective(wbem_context* h, const double* dJ_dphi, const double* dJ_ddn, double* dJ_dX,
                      double* dJ_drhs);
int assemble_fma(wbem_context* h, const QuadTables& qt);
int fma_apply(wbem_context* h, int mode, const double* x, double* y);
int fma_near_blocks(wbem_context* h, double** blocks);
void free_fma(wbem_context* h);
int hull_force_dev(wbem_context* h, const int* hull_cells, int n_hull, const double* U, int dir,
                   const double* d_phi, const double* d_dphi, double* force);
}  // namespace wbem

// ------------------------------------------------------------------ errors
#define CU WB_CU
#define CHK WB_CHK

namespace wbem {
// Copies ordered on the handle's (non-blocking) stream, then waited for.
static cudaError_t copy_sync(wbem_context* h, void* dst, const void* src, size_t bytes,
                             cudaMemcpyKind kind) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  return e;
}

int check_device_error(wbem_context* h, const char* what) {
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess)
    return fail(h, WBEM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  DevErr de;
  e = copy_sync(h, &de, h->d_err, sizeof(DevErr), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess)
    return fail(h, WBEM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  if (de.code != 0) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s: device error %d at site %d (%d, %d)", what, de.code, de.where,
             de.a, de.b);
    DevErr z{};
    copy_sync(h, h->d_err, &z, sizeof z, cudaMemcpyHostToDevice);
    return fail(h, de.code, buf);
  }
  return WBEM_OK;
}
}  // namespace wbem

// ------------------------------------------------------------ quadrature
static int build_quadrature(wbem_context* h, int q1, int sorder) {
  if (q1 < 1 || q1 > kMaxQ1) return fail(h, WBEM_ERR_ARG, "quadrature_order must be in [1,8]");
  if (sorder < 1 || 2 * sorder * sorder > kMaxSingular)
    return fail(h, WBEM_ERR_ARG, "singular_quadrature_order must be in [1,8]");
  QuadTables t{};
  t.q1 = q1;
  std::vector<double> x, w;
  quad::gauss_legendre01(q1, x, w);
  h->gauss_n = q1;
  for (int a = 0; a < q1; ++a) {
    h->gauss_x[a] = x[a];
    h->gauss_w[a] = w[a];
  }
  for (int b = 0; b < q1; ++b)
    for (int a = 0; a < q1; ++a) {
      const int q = a + q1 * b;
      const double s = x[a], u = x[b];
      t.gp[q][0] = s;
      t.gp[q][1] = u;
      t.gp[q][2] = w[a] * w[b];
      t.phi[q][0] = (1 - s) * (1 - u);
      t.phi[q][1] = s * (1 - u);
      t.phi[q][2] = (1 - s) * u;
      t.phi[q][3] = s * u;
      for (int k = 0; k < 3; ++k) t.gpf[q][k] = (float)t.gp[q][k];
      for (int k = 0; k < 4; ++k) t.phif[q][k] = (float)t.phi[q][k];
    }
  // vertex-singular rules (polar map of the two triangles at the vertex, with
  // the 1/R weight folded into the weights), see the oracle for the derivation
  const int m = sorder * sorder;
  t.nsp = 2 * m;
  for (int v = 0; v < 4; ++v) {
    std::vector<double> px, py, pw;
    quad::vertex_singular_points(sorder, v, px, py, pw);
    for (int k = 0; k < 2 * m; ++k) {
      t.sp[v][k][0] = px[k];
      t.sp[v][k][1] = py[k];
      t.sp[v][k][2] = pw[k];
    }
  }
  CU(upload_quadrature_fp64(t));
  CU(upload_quadrature_mixed(t));
  CU(upload_quadrature_adjoint(t));
  h->quad = t;
  return WBEM_OK;
}

// ------------------------------------------------------------- topology
static void find_double_nodes(int N, const double* X, int C, const int* cells,
                              std::vector<int>& ptr, std::vector<int>& idx) {
  // boundary dofs: nodes on an edge used by exactly one cell
  std::map<std::pair<int, int>, int> ecount;
  const int E[4][2] = {{0, 1}, {1, 3}, {3, 2}, {2, 0}};
  for (int c = 0; c < C; ++c)
    for (int e = 0; e < 4; ++e) {
      int a = cells[4 * c + E[e][0]], b = cells[4 * c + E[e][1]];
      if (a > b) std::swap(a, b);
      ecount[{a, b}]++;
    }
  std::vector<char> bnd(N, 0);
  for (auto& kv : ecount)
    if (kv.second == 1) bnd[kv.first.first] = bnd[kv.first.second] = 1;
  const double tol = 1e-8, cell = 1e-6;
  struct Key {
    long long x, y, z;
    bool operator==(const Key& o) const { return x == o.x && y == o.y && z == o.z; }
  };
  struct KH {
    size_t operator()(const Key& k) const {
      return (size_t)(k.x * 73856093LL) ^ (size_t)(k.y * 19349663LL) ^ (size_t)(k.z * 83492791LL);
    }
  };
  std::unordered_map<Key, std::vector<int>, KH> grid;
  auto key = [&](int i) {
    return Key{(long long)std::floor(X[3 * i] / cell), (long long)std::floor(X[3 * i + 1] / cell),
               (long long)std::floor(X[3 * i + 2] / cell)};
  };
  for (int i = 0; i < N; ++i) grid[key(i)].push_back(i);
  ptr.assign(N + 1, 0);
  idx.clear();
  for (int i = 0; i < N; ++i) {
    std::vector<int> s{i};
    if (bnd[i]) {
      Key k = key(i);
      for (long long dx = -1; dx <= 1; ++dx)
        for (long long dy = -1; dy <= 1; ++dy)
          for (long long dz = -1; dz <= 1; ++dz) {
            auto it = grid.find(Key{k.x + dx, k.y + dy, k.z + dz});
            if (it == grid.end()) continue;
            for (int j : it->second) {
              if (j == i) continue;
              double d0 = X[3 * i] - X[3 * j], d1 = X[3 * i + 1] - X[3 * j + 1],
                     d2 = X[3 * i + 2] - X[3 * j + 2];
              if (std::sqrt(d0 * d0 + d1 * d1 + d2 * d2) < tol) s.push_back(j);
            }
          }
    }
    std::sort(s.begin(), s.end());
    idx.insert(idx.end(), s.begin(), s.end());
    ptr[i + 1] = (int)idx.size();
  }
}

// Morton (Z-order) of the support points: the seed order of the patches
// below.
static void morton_order(int N, const double* X, std::vector<int>& perm, std::vector<int>& iperm) {
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < N; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], X[3 * i + d]);
      hi[d] = std::max(hi[d], X[3 * i + d]);
    }
  double ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
  if (!(ext > 0)) ext = 1;
  std::vector<std::pair<uint64_t, int>> k(N);
  for (int i = 0; i < N; ++i) {
    uint64_t q[3];
    for (int d = 0; d < 3; ++d) {
      double t = (X[3 * i + d] - lo[d]) / ext;
      t = std::min(std::max(t, 0.0), 1.0);
      q[d] = (uint64_t)(t * 2097151.0);
    }
    k[i] = {fma_tree::spread3((uint32_t)q[0]) | (fma_tree::spread3((uint32_t)q[1]) << 1) |
                (fma_tree::spread3((uint32_t)q[2]) << 2), i};
  }
  std::sort(k.begin(), k.end());
  perm.resize(N);
  iperm.resize(N);
  for (int i = 0; i < N; ++i) {
    perm[i] = k[i].second;
    iperm[k[i].second] = i;
  }
}

// Internal dof order in surface patches of at most ct nodes: each patch
// grows breadth-first over the mesh graph (nodes sharing a cell) from the
// first node not yet taken in the Morton order, so consecutive patches stay
// close in space. A patch is a column tile of the mixed far-field assembly,
// and groups of consecutive patches are the tiles of the FP64 one: BFS
// patches are rounder than runs of the Morton order, so fewer panels straddle
// two tiles (32,768-dof tank, 48-node tiles: 1.33 tiles per panel against
// 1.47; 20-node patches: 1.50; groups of four of them: 1.34).
// tstart[t] is the first internal dof of patch t, tstart[T] = N.
static void patch_order(int N, const double* X, int C, const int* cells, int ct, std::vector<int>& perm,
                        std::vector<int>& iperm, std::vector<int>& tstart) {
  std::vector<int> seed, seedinv;
  morton_order(N, X, seed, seedinv);
  std::vector<int> aptr(N + 1, 0), adj;
  {
    std::vector<std::pair<int, int>> e;
    e.reserve((size_t)C * 12);
    for (int c = 0; c < C; ++c)
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
          if (a != b) e.push_back({cells[4 * c + a], cells[4 * c + b]});
    std::sort(e.begin(), e.end());
    e.erase(std::unique(e.begin(), e.end()), e.end());
    for (auto& p : e) aptr[p.first + 1]++;
    for (int i = 0; i < N; ++i) aptr[i + 1] += aptr[i];
    adj.resize(e.size());
    for (size_t k = 0; k < e.size(); ++k) adj[k] = e[k].second;  // sorted by first, then second
  }
  std::vector<char> taken(N, 0);
  perm.clear();
  perm.reserve(N);
  tstart.assign(1, 0);
  size_t next = 0;
  while ((int)perm.size() < N) {
    while (taken[seed[next]]) ++next;
    const int s = seed[next];
    taken[s] = 1;
    perm.push_back(s);
    size_t head = perm.size() - 1;
    int got = 1;
    while (head < perm.size() && got < ct) {
      const int u = perm[head++];
      for (int k = aptr[u]; k < aptr[u + 1] && got < ct; ++k) {
        const int v = adj[k];
        if (!taken[v]) {
          taken[v] = 1;
          perm.push_back(v);
          ++got;
        }
      }
    }
    tstart.push_back((int)perm.size());
  }
  iperm.resize(N);
  for (int i = 0; i < N; ++i) iperm[perm[i]] = i;
}

static int build_topology(wbem_context* h) {
  const int N = h->N, C = h->C;
  const int CT = kColsPerTile;
  std::vector<int> tstart;
  patch_order(N, h->X.data(), C, h->cells.data(), CT, h->perm, h->iperm, tstart);
  const auto& ip = h->iperm;
  // cell dofs (internal)
  std::vector<int4> cd(C);
  for (int c = 0; c < C; ++c)
    cd[c] = make_int4(ip[h->cells[4 * c]], ip[h->cells[4 * c + 1]], ip[h->cells[4 * c + 2]],
                      ip[h->cells[4 * c + 3]]);
  // column tiles: the patches (mixed far field) and groups of kTileGroupF64
  // consecutive patches (FP64 far field). Per tile, the panels touching it as
  // (panel | owner bit, 4 slot bytes: the column of each vertex in the tile,
  // 255 outside); tile_ptr: [0, T] entry offsets, then [T + 1, 2T + 1] the
  // tiles' first columns (the tile kernels find them at gridDim.x + 1).
  auto tile_lists = [&](const std::vector<int>& ts, std::vector<int>& tptr, std::vector<int2>& tent) {
    const int T = (int)ts.size() - 1;
    std::vector<int> tile_of(N);
    for (int t = 0; t < T; ++t)
      for (int i = ts[t]; i < ts[t + 1]; ++i) tile_of[i] = t;
    std::vector<std::vector<int2>> tl(T);
    for (int c = 0; c < C; ++c) {
      const int d[4] = {cd[c].x, cd[c].y, cd[c].z, cd[c].w};
      int tiles[4];
      int nt = 0;
      for (int k = 0; k < 4; ++k) {
        int t = tile_of[d[k]];
        bool seen = false;
        for (int u = 0; u < nt; ++u) seen |= tiles[u] == t;
        if (!seen) tiles[nt++] = t;
      }
      const int owner = tile_of[d[0]];
      for (int u = 0; u < nt; ++u) {
        uint32_t slots = 0;
        for (int k = 0; k < 4; ++k) {
          uint32_t sl = (tile_of[d[k]] == tiles[u]) ? (uint32_t)(d[k] - ts[tiles[u]]) : 255u;
          slots |= sl << (8 * k);
        }
        int2 e;
        e.x = c | (tiles[u] == owner ? (int)0x80000000u : 0);
        e.y = (int)slots;
        tl[tiles[u]].push_back(e);
      }
    }
    tptr.assign(T + 1, 0);
    tent.clear();
    for (int t = 0; t < T; ++t) {
      tent.insert(tent.end(), tl[t].begin(), tl[t].end());
      tptr[t + 1] = (int)tent.size();
    }
    tptr.insert(tptr.end(), ts.begin(), ts.end());
  };
  h->n_tiles = (int)tstart.size() - 1;
  std::vector<int> tptr, tptr64;
  std::vector<int2> tent, tent64;
  tile_lists(tstart, tptr, tent);
  std::vector<int> tstart64;
  for (size_t t = 0; t < tstart.size(); t += kTileGroupF64) tstart64.push_back(tstart[t]);
  if (tstart64.back() != N) tstart64.push_back(N);
  h->n_tiles64 = (int)tstart64.size() - 1;
  tile_lists(tstart64, tptr64, tent64);
  // double-node sets (internal)
  std::vector<int> dnset((size_t)N * kMaxSet, -1);
  for (int p = 0; p < N; ++p) {
    const int i = ip[p];
    int k = 0;
    for (int e = h->dn_ptr[p]; e < h->dn_ptr[p + 1]; ++e) dnset[(size_t)i * kMaxSet + k++] = ip[h->dn_idx[e]];
  }
  // node -> (cell, vertex) adjacency (internal nodes)
  std::vector<int> ncptr(N + 1, 0), ncent;
  for (int c = 0; c < C; ++c) {
    const int d[4] = {cd[c].x, cd[c].y, cd[c].z, cd[c].w};
    for (int k = 0; k < 4; ++k) ncptr[d[k] + 1]++;
  }
  for (int i = 0; i < N; ++i) ncptr[i + 1] += ncptr[i];
  ncent.resize(ncptr[N]);
  {
    std::vector<int> fill(ncptr.begin(), ncptr.end() - 1);
    for (int c = 0; c < C; ++c) {
      const int d[4] = {cd[c].x, cd[c].y, cd[c].z, cd[c].w};
      for (int k = 0; k < 4; ++k) ncent[fill[d[k]]++] = c * 4 + k;
    }
  }
  // singular panels per row: cells adjacent to a node of the row's set
  std::vector<int> sptr(N + 1, 0), scell;
  for (int i = 0; i < N; ++i) {
    std::vector<int> s;
    for (int k = 0; k < kMaxSet; ++k) {
      const int j = dnset[(size_t)i * kMaxSet + k];
      if (j < 0) continue;
      for (int e = ncptr[j]; e < ncptr[j + 1]; ++e) s.push_back(ncent[e] / 4);
    }
    std::sort(s.begin(), s.end());
    s.erase(std::unique(s.begin(), s.end()), s.end());
    scell.insert(scell.end(), s.begin(), s.end());
    sptr[i + 1] = (int)scell.size();
  }
  std::vector<double> Xi((size_t)N * 3);
  for (int i = 0; i < N; ++i)
    for (int d = 0; d < 3; ++d) Xi[3 * (size_t)i + d] = h->X[3 * (size_t)h->perm[i] + d];
  CHK(upload(h, &h->d_X, Xi));
  CHK(upload(h, &h->d_cell_dofs, cd));
  CHK(upload(h, &h->d_dnset, dnset));
  CHK(upload(h, &h->d_tile_ptr, tptr));
  CHK(upload(h, &h->d_tile_ent, tent));
  CHK(upload(h, &h->d_tile_ptr64, tptr64));
  CHK(upload(h, &h->d_tile_ent64, tent64));
  CHK(upload(h, &h->d_sptr, sptr));
  CHK(upload(h, &h->d_scell, scell));
  CHK(upload(h, &h->d_perm, h->perm));
  CHK(upload(h, &h->d_iperm, h->iperm));
  CHK(upload(h, &h->d_ncptr, ncptr));
  CHK(upload(h, &h->d_ncent, ncent));
  return WBEM_OK;
}

// ------------------------------------------------------------ constraints
// (constraints.cu: compute_constraints, the L2 projections, their adjoint)
namespace wbem {
int build_constraints(wbem_context* h, const double* tmp_rhs);
void node_normals(wbem_context* h, std::vector<double>& n);
void surface_gradients(wbem_context* h, const double* tmp_rhs, std::vector<double>& g);
}  // namespace wbem

// ------------------------------------------------------------- workspaces
namespace wbem {
int ensure_vectors(wbem_context* h, int restart) {
  const int N = h->N;
  for (int k = 0; k < kNumVec; ++k)
    if (!h->d_vec[k]) CHK(dev_alloc(h, &h->d_vec[k], (size_t)N));
  if (!h->d_part) CHK(dev_alloc(h, &h->d_part, (size_t)256 * 128 + (size_t)40 * N));
  if (!h->d_small) CHK(dev_alloc(h, &h->d_small, (size_t)512));
  if (!h->d_sol) CHK(dev_alloc(h, &h->d_sol, (size_t)N));
  if (!h->d_rhs) CHK(dev_alloc(h, &h->d_rhs, (size_t)N));
  if (!h->d_b) CHK(dev_alloc(h, &h->d_b, (size_t)N));
  if (h->V_cap < restart + 1) {
    // Arnoldi basis V (restart + 1 vectors), then the preconditioned basis Z
    CHK(dev_alloc(h, &h->d_V, (size_t)(2 * restart + 1) * N));
    h->V_cap = restart + 1;
  }
  return WBEM_OK;
}

// y = A x (constrained system operator), FP64 or mixed storage.
int apply_system(wbem_context* h, const double* x, double* y) {
  if (h->assembled_prec == kAssembledFma)
    CHK(fma_apply(h, 0, x, y));
  else if (h->assembled_prec == WBEM_PREC_FP64)
    CU(launch_matvec_fp64(h->N, 0, h->d_N, h->d_D, h->d_mask, h->d_alpha, x, y, h->stream));
  else {
    if (h->profiling) h->prof_matvec.begin(h->stream);
    CU(launch_matvec_mixed(h->N, 0, h->d_A2, h->d_mask, h->d_alpha, x, y, h->stream));
    if (h->profiling) h->prof_matvec.end(h->stream, 8.0 * (double)h->N * h->N);
  }
  CU(launch_constraint_rows(h->n_crows, h->d_crow, h->d_cptr, h->d_ccol, h->d_cval, x, y, h->stream));
  h->launches += 2;
  return WBEM_OK;
}

// y = A^T x for the constrained operator.
int apply_system_t(wbem_context* h, const double* x, double* y) {
  if (h->assembled_prec == kAssembledFma)
    return fail(h, WBEM_ERR_STATE, "the FMA method has no transposed operator");
  // x with its constrained entries zeroed feeds the unconstrained rows
  double* xz = h->d_vec[7];
  CU(cudaMemcpyAsync(xz, x, sizeof(double) * h->N, cudaMemcpyDeviceToDevice, h->stream));
  if (h->n_crows) {
    double* zeros = h->d_part;
    CU(cudaMemsetAsync(zeros, 0, sizeof(double) * h->n_crows, h->stream));
    CU(launch_set_rows(h->n_crows, h->d_crow, zeros, xz, h->stream));
  }
  double* part = h->d_part + 256 * 128;
  if (h->assembled_prec == WBEM_PREC_FP64)
    CU(launch_matvec_t_fp64(h->N, h->d_N, h->d_D, h->d_mask, h->d_alpha, xz, y, part, h->stream));
  else
    CU(launch_matvec_t_mixed(h->N, h->d_A2, h->d_mask, h->d_alpha, xz, y, part, h->stream));
  if (h->n_crows)
    CU(launch_constraint_rows_t(h->N, h->n_crows, h->d_crow, h->d_cptr, h->d_ccol, h->d_cval,
                                h->d_tptr, h->d_tsrc, h->d_tval, h->d_cflag, x, y, h->stream));
  h->launches += 5;
  return WBEM_OK;
}

static int read_scalar(wbem_context* h, const double* d, double* v) {
  CU(cudaMemcpyAsync(v, d, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CU(cudaStreamSynchronize(h->stream));
  return WBEM_OK;
}

// Right-preconditioned GMRES(m) with classical Gram-Schmidt and one
// re-orthogonalisation, Givens rotations on the host. prec(z <- M^{-1} v).
// Stops when the residual norm is <= max(tol, 1e-14 ||rhs||) (absolute
// tolerance as deal.II's SolverControl, floored at round-off level).
// Flexible form (right preconditioning with the preconditioned vectors
// z_k = M^-1 v_k kept): the update x += Z y uses exactly the vectors the
// Arnoldi relation was built from. The FP32 LU applied in FP32 is not an
// exactly linear map, so re-applying it to V y (the plain right-preconditioned
// update) leaves a true residual near the FP32 round-off of x above the
// estimate and costs a restart cycle; the flexible update does not.
template <typename Op, typename Prec>
int gmres(wbem_context* h, const double* rhs, double* x, int restart, int max_steps, double tol,
          Op op, Prec prec, int* iters, double* resid) {
  const int N = h->N;
  double* r = h->d_vec[0];
  double* w = h->d_vec[1];
  double* Z = h->d_V + (size_t)h->V_cap * N;  // restart vectors
  double* hbuf = h->d_small;  // [0..restart+1] h, [256..] h2
  double* part = h->d_part;
  double bnorm;
  CU(launch_nrm2(N, rhs, part, hbuf, h->stream));
  CHK(read_scalar(h, hbuf, &bnorm));
  const double target = std::max(tol, 1e-14 * bnorm);
  CU(cudaMemsetAsync(x, 0, sizeof(double) * N, h->stream));
  int it = 0;
  double res = bnorm;
  std::vector<double> H((size_t)(restart + 1) * restart), cs(restart), sn(restart), g(restart + 1),
      hv(restart + 2), hv2(restart + 2), y(restart);
  bool first = true;
  while (true) {
    // r = rhs - A x
    if (first) {
      CU(cudaMemcpyAsync(r, rhs, sizeof(double) * N, cudaMemcpyDeviceToDevice, h->stream));
      first = false;
    } else {
      CHK(op(x, r));
      CU(launch_axpby(N, 1.0, rhs, -1.0, r, h->stream));
    }
    CU(launch_nrm2(N, r, part, hbuf, h->stream));
    double beta;
    CHK(read_scalar(h, hbuf, &beta));
    res = beta;
    if (!std::isfinite(beta)) return fail(h, WBEM_ERR_NONFINITE, "GMRES: non-finite residual");
    if (beta <= target) break;
    if (it >= max_steps) {
      if (iters) *iters = it;
      if (resid) *resid = res;
      return fail(h, WBEM_ERR_NOCONV, "GMRES: no convergence within max_steps");
    }
    CU(launch_scale(N, r, 1.0 / beta, h->d_V, h->stream));
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;
    for (; k < restart && it < max_steps; ++k) {
      double* vk = h->d_V + (size_t)k * N;
      double* vk1 = h->d_V + (size_t)(k + 1) * N;
      double* z = Z + (size_t)k * N;
      CHK(prec(vk, z));
      CHK(op(z, w));
      CU(launch_multidot(N, k + 1, h->d_V, w, part, hbuf, h->stream));
      CU(launch_axpy_basis(N, k + 1, h->d_V, hbuf, w, -1.0, h->stream));
      CU(launch_multidot(N, k + 1, h->d_V, w, part, hbuf + 256, h->stream));
      CU(launch_axpy_basis(N, k + 1, h->d_V, hbuf + 256, w, -1.0, h->stream));
      CU(launch_nrm2(N, w, part, hbuf + 255, h->stream));
      CU(cudaMemcpyAsync(hv.data(), hbuf, sizeof(double) * (k + 1), cudaMemcpyDeviceToHost, h->stream));
      CU(cudaMemcpyAsync(hv2.data(), hbuf + 256, sizeof(double) * (k + 1), cudaMemcpyDeviceToHost, h->stream));
      double hn;
      CU(cudaMemcpyAsync(&hn, hbuf + 255, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      CU(cudaStreamSynchronize(h->stream));
      h->launches += 9;
      ++it;
      for (int j = 0; j <= k; ++j) H[(size_t)j * restart + k] = hv[j] + hv2[j];
      H[(size_t)(k + 1) * restart + k] = hn;
      if (hn > 0) CU(launch_scale(N, w, 1.0 / hn, vk1, h->stream));
      for (int j = 0; j < k; ++j) {
        double a = H[(size_t)j * restart + k], b = H[(size_t)(j + 1) * restart + k];
        H[(size_t)j * restart + k] = cs[j] * a + sn[j] * b;
        H[(size_t)(j + 1) * restart + k] = -sn[j] * a + cs[j] * b;
      }
      double a = H[(size_t)k * restart + k], b = H[(size_t)(k + 1) * restart + k];
      double d = std::hypot(a, b);
      if (d == 0) return fail(h, WBEM_ERR_SINGULAR, "GMRES: breakdown");
      cs[k] = a / d;
      sn[k] = b / d;
      H[(size_t)k * restart + k] = d;
      H[(size_t)(k + 1) * restart + k] = 0;
      g[k + 1] = -sn[k] * g[k];
      g[k] = cs[k] * g[k];
      res = std::fabs(g[k + 1]);
      if (res <= target || hn == 0) {
        ++k;
        break;
      }
    }
    for (int j = k - 1; j >= 0; --j) {
      double s = g[j];
      for (int l = j + 1; l < k; ++l) s -= H[(size_t)j * restart + l] * y[l];
      y[j] = s / H[(size_t)j * restart + j];
    }
    CU(cudaMemcpyAsync(hbuf, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, h->stream));
    CU(launch_axpy_basis(N, k, Z, hbuf, x, 1.0, h->stream));
    // the host vector y must stay alive until the copy above completes
    CU(cudaStreamSynchronize(h->stream));
    // converged on the Arnoldi estimate: with the flexible update it is the
    // true residual up to FP64 round-off, so no residual mat-vec follows
    // (deal.II's SolverGMRES also stops on the estimate)
    if (res <= target) break;
  }
  if (iters) *iters = it;
  if (resid) *resid = res;
  return WBEM_OK;
}

int gmres_fp64(wbem_context* h, const double* rhs, double* x, int transpose) {
  auto op = [&](const double* a, double* b) {
    return transpose ? apply_system_t(h, a, b) : apply_system(h, a, b);
  };
  auto prec = [&](const double* a, double* b) -> int {
    CU(launch_bj_apply(h->N, h->d_binv, a, b, transpose, h->stream));
    return WBEM_OK;
  };
  int it = 0;
  double res = 0;
  int st = gmres(h, rhs, x, h->opt.gmres_restart, h->opt.max_steps, h->opt.tolerance, op, prec,
                 &it, &res);
  h->stats.iterations = it;
  h->stats.residual = res;
  return st;
}

int lu_apply(wbem_context* h, const double* v, double* z, int transpose);

// GMRES iterative refinement in FP64 on the mixed-storage operator,
// preconditioned by the FP32 LU factors (right preconditioning).
int gmres_mixed_driver(wbem_context* h, const double* rhs, double* x, int transpose) {
  auto op = [&](const double* a, double* b) {
    return transpose ? apply_system_t(h, a, b) : apply_system(h, a, b);
  };
  auto prec = [&](const double* a, double* b) { return lu_apply(h, a, b, transpose); };
  int it = 0;
  double res = 0;
  int st = gmres(h, rhs, x, h->opt.gmres_restart, h->opt.max_steps, h->opt.tolerance, op, prec,
                 &it, &res);
  h->stats.iterations = it;
  h->stats.residual = res;
  return st;
}

int build_block_jacobi(wbem_context* h) {
  const int nb = (h->N + kBJ - 1) / kBJ;
  CHK(dev_alloc(h, &h->d_binv, (size_t)nb * kBJ * kBJ));
  const bool fp64 = h->assembled_prec == WBEM_PREC_FP64;
  double* blocks = nullptr;  // FMA: the near field's diagonal blocks
  if (h->assembled_prec == kAssembledFma) CHK(fma_near_blocks(h, &blocks));
  CU(launch_bj_build(h->N, fp64 ? h->d_N : nullptr, fp64 ? h->d_D : nullptr,
                     blocks ? nullptr : h->d_A2, blocks, h->d_mask, h->d_alpha, h->d_cflag,
                     h->d_cptr_full, h->d_ccol_full, h->d_cval_full, h->d_binv, h->d_err,
                     h->stream));
  h->launches++;
  return check_device_error(h, "block-Jacobi");
}

int form_system_f32(wbem_context* h);
int system_ld(int N);

// Mixed-precision iterative refinement: x_{k+1} = x_k + d_k with d_k an
// inner block-Jacobi GMRES solve of S d = r_k on the FP32 system matrix S
// (4 bytes per entry streamed per inner step) to a relative residual of
// 10^-inner_digits, and r_k = rhs - A x_k with the (hi, lo) operator in
// double-float (8 bytes per entry, once per refinement step). Each step
// contracts the error by about max(10^-inner_digits, cond(A) |S - A| / |A|).
// The iteration count reported is the total of inner GMRES steps.
int gmres_ir(wbem_context* h, const double* rhs, double* x, int transpose) {
  const int N = h->N;
  const int ld = system_ld(N);
  double* r = h->d_vec[8];
  double* d = h->d_vec[9];
  double* part = h->d_part;
  double* hbuf = h->d_small;
  const int digits = h->opt.inner_digits > 0 ? h->opt.inner_digits : 4;
  const double eta = std::pow(10.0, -(double)digits);
  auto op32 = [&](const double* a, double* b) -> int {
    if (transpose)
      CU(launch_matvec_s32_t(N, ld, h->d_lu, a, b, h->d_part + 256 * 128, h->stream));
    else
      CU(launch_matvec_s32(N, ld, h->d_lu, a, b, h->stream));
    h->launches += transpose ? 2 : 1;
    return WBEM_OK;
  };
  auto prec = [&](const double* a, double* b) -> int {
    CU(launch_bj_apply(N, h->d_binv, a, b, transpose, h->stream));
    h->launches++;
    return WBEM_OK;
  };
  double bnorm;
  CU(launch_nrm2(N, rhs, part, hbuf, h->stream));
  CHK(read_scalar(h, hbuf, &bnorm));
  const double target = std::max(h->opt.tolerance, 1e-14 * bnorm);
  CU(cudaMemsetAsync(x, 0, sizeof(double) * N, h->stream));
  CU(cudaMemcpyAsync(r, rhs, sizeof(double) * N, cudaMemcpyDeviceToDevice, h->stream));
  double rnorm = bnorm;
  int total = 0, outer = 0;
  constexpr int kMaxOuter = 40;
  while (rnorm > target) {
    if (total >= h->opt.max_steps || outer >= kMaxOuter) {
      h->stats.iterations = total;
      h->stats.residual = rnorm;
      h->stats.outer_iterations = outer;
      return fail(h, WBEM_ERR_NOCONV, "GMRES-IR: no convergence within max_steps");
    }
    const int budget = std::min(h->opt.gmres_restart, h->opt.max_steps - total);
    int it = 0;
    double res = 0;
    const int st = gmres(h, r, d, h->opt.gmres_restart, budget, std::max(eta * rnorm, 0.5 * target),
                         op32, prec, &it, &res);
    // an inner solve that stops at its step budget still gives a correction
    if (st != WBEM_OK && st != WBEM_ERR_NOCONV) return st;
    total += it;
    ++outer;
    CU(launch_axpby(N, 1.0, d, 1.0, x, h->stream));
    CHK(transpose ? apply_system_t(h, x, r) : apply_system(h, x, r));
    CU(launch_axpby(N, 1.0, rhs, -1.0, r, h->stream));
    CU(launch_nrm2(N, r, part, hbuf, h->stream));
    CHK(read_scalar(h, hbuf, &rnorm));
    h->launches += 3;
    if (!std::isfinite(rnorm)) return fail(h, WBEM_ERR_NONFINITE, "GMRES-IR: non-finite residual");
  }
  h->stats.iterations = total;
  h->stats.residual = rnorm;
  h->stats.outer_iterations = outer;
  return WBEM_OK;
}

// Constraint rows and entries for the current mask and geometry (the
// inhomogeneities, which depend on tmp_rhs, are left at zero): what the FP32
// system matrix needs when no solve has run yet.
int build_constraint_structure(wbem_context* h) {
  std::vector<double> zero(h->N, 0.0);
  return build_constraints(h, zero.data());
}

// The solver an assembly uses (the AUTO choice resolved), or -1 if the
// option does not apply to the assembled precision.
int resolved_solver(const wbem_context* h) {
  if (h->assembled_prec == kAssembledFma)
    return (h->opt.solver == WBEM_SOLVER_AUTO || h->opt.solver == WBEM_SOLVER_GMRES) ? WBEM_SOLVER_GMRES : -1;
  const bool fp64 = h->assembled_prec == WBEM_PREC_FP64;
  switch (h->opt.solver) {
    case WBEM_SOLVER_AUTO:
      return fp64 ? WBEM_SOLVER_GMRES : WBEM_SOLVER_LU;
    case WBEM_SOLVER_GMRES:
      return WBEM_SOLVER_GMRES;
    case WBEM_SOLVER_LU:
    case WBEM_SOLVER_GMRES_IR:
      return fp64 ? -1 : h->opt.solver;
    default:
      return -1;
  }
}

// Solve A x = rhs (transpose: A^T x = rhs) with the solver of the current
// assembly, preparing its preconditioner once per assembly.
int solve_assembled(wbem_context* h, const double* rhs, double* x, int transpose) {
  const int solver = resolved_solver(h);
  if (solver < 0) return fail(h, WBEM_ERR_ARG, "solver option does not apply to this precision");
  if (!h->factors_valid || h->factors_kind != solver) {
    if (solver == WBEM_SOLVER_LU) {
      CHK(factor_mixed(h));  // times the system formation and the factorisation itself
    } else {
      h->stats.t_system_ms = 0.0;
      if (solver == WBEM_SOLVER_GMRES_IR) CHK(form_system_f32(h));
      EvTimer tm(h->stream);
      CHK(build_block_jacobi(h));
      h->stats.t_factor_ms = tm.ms();
    }
    h->factors_valid = true;
    h->factors_kind = solver;
  } else {
    h->stats.t_system_ms = 0.0;
    h->stats.t_factor_ms = 0.0;
  }
  h->stats.outer_iterations = 0;
  if (h->rhs_pending) {  // the right-hand side computed beside the preparation
    CU(cudaStreamWaitEvent(h->stream, h->ev_rhs, 0));
    h->rhs_pending = false;
  }
  if (solver == WBEM_SOLVER_GMRES) return gmres_fp64(h, rhs, x, transpose);
  if (solver == WBEM_SOLVER_LU) return solve_mixed(h, rhs, x, transpose);
  return gmres_ir(h, rhs, x, transpose);
}

}  // namespace wbem

// ---------------------------------------------------------------- timing
namespace {
struct Timer {
  cudaEvent_t a, b;
  cudaStream_t s;
  explicit Timer(cudaStream_t st) : s(st) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
  }
  double ms() {
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float t = 0;
    cudaEventElapsedTime(&t, a, b);
    cudaEventRecord(a, s);
    return t;
  }
  ~Timer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};
}  // namespace

// ================================================================ C ABI
extern "C" {

int wbem_default_options(wbem_options* o) {
  if (!o) return WBEM_ERR_ARG;
  std::memset(o, 0, sizeof *o);
  o->precision = WBEM_PREC_FP64;
  o->solver = WBEM_SOLVER_AUTO;
  o->quadrature_order = 4;
  o->singular_quadrature_order = 5;
  o->gmres_restart = 100;
  o->max_steps = 1000;
  o->tolerance = 1e-12;
  o->near_field_ratio = 2.0;
  o->keep_matrices = 1;
  o->method = WBEM_METHOD_DIRECT;
  o->fma_order = 6;
  return WBEM_OK;
}

int wbem_create(wbem_handle* out, int device) {
  if (!out) return WBEM_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return WBEM_ERR_CUDA;
  if (device < 0 || device >= n) return WBEM_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return WBEM_ERR_CUDA;
  wbem_context* h = new wbem_context();
  h->device = device;
  wbem_default_options(&h->opt);
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return WBEM_ERR_CUDA;
  }
  h->own_stream = true;
  if (cudaMalloc(&h->d_err, sizeof(DevErr)) != cudaSuccess) {
    cudaStreamDestroy(h->stream);
    delete h;
    return WBEM_ERR_NOMEM;
  }
  cudaMemset(h->d_err, 0, sizeof(DevErr));
  *out = h;
  return WBEM_OK;
}

// Frees every device buffer whose size depends on the mesh (all but the
// error word) and forgets the sizes, so that the next calls allocate for the
// current mesh.
static void release_mesh_buffers(wbem_context* h) {
  cudaStreamSynchronize(h->stream);
  free_lu(h);
  free_fma(h);
  void** ptrs[] = {(void**)&h->d_X, (void**)&h->d_cell_dofs, (void**)&h->d_dnset, (void**)&h->d_tile_ptr,
                   (void**)&h->d_tile_ent, (void**)&h->d_tile_ptr64, (void**)&h->d_tile_ent64, (void**)&h->d_sptr, (void**)&h->d_scell, (void**)&h->d_perm,
                   (void**)&h->d_iperm, (void**)&h->d_ncptr, (void**)&h->d_ncent, (void**)&h->d_mask,
                   (void**)&h->d_rec, (void**)&h->d_rec32, (void**)&h->d_cellc, (void**)&h->d_cellgeo,
                   (void**)&h->d_N, (void**)&h->d_D, (void**)&h->d_A2, (void**)&h->d_B2,
                   (void**)&h->d_selmask, (void**)&h->d_flips, (void**)&h->d_alpha,
                   (void**)&h->d_alpha_part, (void**)&h->d_alpha_near, (void**)&h->d_alpha_sing,
                   (void**)&h->d_near_cnt, (void**)&h->d_near_cells, (void**)&h->d_item_val,
                   (void**)&h->d_item_dof, (void**)&h->d_item_cnt, (void**)&h->d_crow, (void**)&h->d_cptr,
                   (void**)&h->d_ccol, (void**)&h->d_cval, (void**)&h->d_cinh, (void**)&h->d_cflag,
                   (void**)&h->d_cptr_full, (void**)&h->d_ccol_full, (void**)&h->d_cval_full,
                   (void**)&h->d_tptr, (void**)&h->d_tsrc, (void**)&h->d_tval, (void**)&h->d_binv,
                   (void**)&h->d_V, (void**)&h->d_part, (void**)&h->d_small, (void**)&h->d_lu,
                   (void**)&h->d_split, (void**)&h->d_lutmp, (void**)&h->d_info, (void**)&h->d_sol,
                   (void**)&h->d_rhs, (void**)&h->d_b};
  for (void** p : ptrs)
    if (*p) {
      cudaFree(*p);
      *p = nullptr;
    }
  for (int k = 0; k < kNumVec; ++k)
    if (h->d_vec[k]) {
      cudaFree(h->d_vec[k]);
      h->d_vec[k] = nullptr;
    }
  h->rec_cells = 0;
  h->mat_elems = 0;
  h->item_rows = 0;
  h->near_cap = 0;
  h->V_cap = 0;
  h->lu_elems = 0;
  h->flips_cap = 0;
  h->s32_state = 0;
  h->assembled_prec = -1;
  h->factors_valid = false;
  h->have_solution = false;
  h->sel_mask.clear();
  h->c_crow.clear();
  h->c_cptr.clear();
  h->c_ccol.clear();
  h->c_cval.clear();
  h->n_crows = 0;
}

int wbem_destroy(wbem_handle h) {
  if (!h) return WBEM_ERR_ARG;
  cudaSetDevice(h->device);
  release_mesh_buffers(h);
  if (h->d_err) cudaFree(h->d_err);
  if (h->aux_stream) cudaStreamDestroy(h->aux_stream);
  if (h->ev_aux_fork) cudaEventDestroy(h->ev_aux_fork);
  if (h->ev_aux_join) cudaEventDestroy(h->ev_aux_join);
  if (h->ev_rhs) cudaEventDestroy(h->ev_rhs);
  if (h->rhs_stream) cudaStreamDestroy(h->rhs_stream);
  if (h->own_stream) cudaStreamDestroy(h->stream);
  delete h;
  return WBEM_OK;
}

const char* wbem_last_error(wbem_handle h) {
  if (!h) return "invalid handle";
  return h->err.c_str();
}

int wbem_set_geometry(wbem_handle h, const double* X, int n_dofs, const int* cells, int n_cells,
                      const int* dn_ptr, const int* dn_idx) {
  if (!h) return WBEM_ERR_ARG;
  if (!X || !cells || n_dofs < 1 || n_cells < 1)
    return fail(h, WBEM_ERR_ARG, "wbem_set_geometry: empty mesh or NULL pointer");
  if ((dn_ptr == nullptr) != (dn_idx == nullptr))
    return fail(h, WBEM_ERR_ARG, "wbem_set_geometry: dn_ptr and dn_idx must both be given or both NULL");
  for (long long k = 0; k < 3LL * n_dofs; ++k)
    if (!std::isfinite(X[k])) return fail(h, WBEM_ERR_NONFINITE, "wbem_set_geometry: non-finite support point");
  for (long long k = 0; k < 4LL * n_cells; ++k)
    if (cells[k] < 0 || cells[k] >= n_dofs)
      return fail(h, WBEM_ERR_ARG, "wbem_set_geometry: cell vertex index out of range");
  for (int c = 0; c < n_cells; ++c)
    for (int a = 0; a < 4; ++a)
      for (int b = a + 1; b < 4; ++b)
        if (cells[4 * c + a] == cells[4 * c + b])
          return fail(h, WBEM_ERR_ARG, "wbem_set_geometry: repeated vertex in a cell");
  cudaSetDevice(h->device);
  // a mesh of another size: every size-dependent buffer is allocated anew
  if (h->N != 0 && (h->N != n_dofs || h->C != n_cells)) release_mesh_buffers(h);
  h->N = n_dofs;
  h->C = n_cells;
  h->X.assign(X, X + 3 * (size_t)n_dofs);
  h->cells.assign(cells, cells + 4 * (size_t)n_cells);
  if (dn_ptr) {
    if (dn_ptr[0] != 0) return fail(h, WBEM_ERR_ARG, "wbem_set_geometry: dn_ptr[0] must be 0");
    h->dn_ptr.assign(dn_ptr, dn_ptr + n_dofs + 1);
    h->dn_idx.assign(dn_idx, dn_idx + dn_ptr[n_dofs]);
    for (int i = 0; i < n_dofs; ++i) {
      const int a = dn_ptr[i], b = dn_ptr[i + 1];
      if (b <= a || b - a > kMaxSet)
        return fail(h, WBEM_ERR_ARG, "wbem_set_geometry: double-node set empty or larger than 8");
      bool self = false;
      for (int k = a; k < b; ++k) {
        if (dn_idx[k] < 0 || dn_idx[k] >= n_dofs)
          return fail(h, WBEM_ERR_ARG, "wbem_set_geometry: double-node index out of range");
        if (k > a && dn_idx[k] <= dn_idx[k - 1])
          return fail(h, WBEM_ERR_ARG, "wbem_set_geometry: double-node set not strictly ascending");
        self |= dn_idx[k] == i;
      }
      if (!self) return fail(h, WBEM_ERR_ARG, "wbem_set_geometry: double-node set must contain its own dof");
    }
  } else {
    find_double_nodes(n_dofs, X, n_cells, cells, h->dn_ptr, h->dn_idx);
    for (int i = 0; i < n_dofs; ++i)
      if (h->dn_ptr[i + 1] - h->dn_ptr[i] > kMaxSet)
        return fail(h, WBEM_ERR_ARG, "wbem_set_geometry: more than 8 coincident nodes");
  }
  h->assembled_prec = -1;
  h->factors_valid = false;
  h->have_solution = false;
  h->fma_geometry_stale = true;
  CHK(build_quadrature(h, h->opt.quadrature_order, h->opt.singular_quadrature_order));
  CHK(build_topology(h));
  if (h->have_mask && (int)h->mask.size() == n_dofs) {
    std::vector<uint8_t> mi(n_dofs);
    for (int i = 0; i < n_dofs; ++i) mi[i] = h->mask[h->perm[i]];
    CHK(upload(h, &h->d_mask, mi));
  } else {
    h->have_mask = false;
  }
  return WBEM_OK;
}

int wbem_update_nodes(wbem_handle h, const double* X) {
  if (!h) return WBEM_ERR_ARG;
  if (!X || h->N == 0) return fail(h, WBEM_ERR_STATE, "wbem_update_nodes: no geometry");
  for (long long k = 0; k < 3LL * h->N; ++k)
    if (!std::isfinite(X[k])) return fail(h, WBEM_ERR_NONFINITE, "wbem_update_nodes: non-finite support point");
  cudaSetDevice(h->device);
  h->X.assign(X, X + 3 * (size_t)h->N);
  std::vector<double> Xi((size_t)h->N * 3);
  for (int i = 0; i < h->N; ++i)
    for (int d = 0; d < 3; ++d) Xi[3 * (size_t)i + d] = X[3 * (size_t)h->perm[i] + d];
  CU(copy_sync(h, h->d_X, Xi.data(), Xi.size() * sizeof(double), cudaMemcpyHostToDevice));
  h->fma_geometry_stale = true;  // the octree follows the nodes
  h->assembled_prec = -1;
  h->factors_valid = false;
  h->have_solution = false;
  return WBEM_OK;
}

int wbem_set_bc(wbem_handle h, const unsigned char* m) {
  if (!h) return WBEM_ERR_ARG;
  if (!m || h->N == 0) return fail(h, WBEM_ERR_STATE, "wbem_set_bc: set the geometry first");
  cudaSetDevice(h->device);
  std::vector<unsigned char> nm(m, m + h->N);
  for (auto& v : nm) v = v ? 1 : 0;
  // an unchanged mask keeps the factors and the FP32 system matrix
  if (h->have_mask && nm == h->mask) return WBEM_OK;
  h->mask.swap(nm);
  std::vector<uint8_t> mi(h->N);
  for (int i = 0; i < h->N; ++i) mi[i] = h->mask[h->perm[i]];
  CHK(upload(h, &h->d_mask, mi));
  if (h->assembled_prec == WBEM_PREC_MIXED && h->d_A2 && (int)h->sel_mask.size() == h->N) {
    // the mixed pairs carry the old selection: swap the changed columns
    std::vector<int> flips;
    for (int i = 0; i < h->N; ++i)
      if (h->sel_mask[i] != mi[i]) flips.push_back(i);
    if (!flips.empty()) {
      if (h->flips_cap < flips.size()) {
        CHK(dev_alloc(h, &h->d_flips, flips.size()));
        h->flips_cap = flips.size();
      }
      CU(cudaMemcpyAsync(h->d_flips, flips.data(), sizeof(int) * flips.size(), cudaMemcpyHostToDevice,
                         h->stream));
      CU(launch_reselect_pairs(h->N, (int)flips.size(), h->d_flips, h->d_A2, h->d_B2, h->stream));
      h->sel_mask = mi;
      CU(cudaMemcpyAsync(h->d_selmask, h->sel_mask.data(), (size_t)h->N, cudaMemcpyHostToDevice,
                         h->stream));
      CU(cudaStreamSynchronize(h->stream));
    }
  }
  h->have_mask = true;
  h->factors_valid = false;
  h->have_solution = false;
  h->s32_state = 0;
  return WBEM_OK;
}

int wbem_assemble(wbem_handle h, const wbem_options* opt) {
  if (!h) return WBEM_ERR_ARG;
  if (h->N == 0) return fail(h, WBEM_ERR_STATE, "wbem_assemble: set the geometry first");
  wbem_options o;
  if (opt) o = *opt;
  else wbem_default_options(&o);
  if (o.precision != WBEM_PREC_FP64 && o.precision != WBEM_PREC_MIXED)
    return fail(h, WBEM_ERR_ARG, "wbem_assemble: unknown precision");
  if (o.gmres_restart < 1 || o.gmres_restart > 250)
    return fail(h, WBEM_ERR_ARG, "wbem_assemble: gmres_restart must be in [1,250]");
  if (o.max_steps < 1) return fail(h, WBEM_ERR_ARG, "wbem_assemble: max_steps must be >= 1");
  if (!(o.tolerance >= 0)) return fail(h, WBEM_ERR_ARG, "wbem_assemble: tolerance must be >= 0");
  if (o.method != WBEM_METHOD_DIRECT && o.method != WBEM_METHOD_FMA)
    return fail(h, WBEM_ERR_ARG, "wbem_assemble: unknown method");
  if (o.method == WBEM_METHOD_DIRECT && (long long)h->N * h->N > (1LL << 34))
    return fail(h, WBEM_ERR_ARG, "wbem_assemble: n_dofs too large for dense N x N matrices (use the FMA method)");
  h->opt = o;
  cudaSetDevice(h->device);
  CHK(build_quadrature(h, o.quadrature_order, o.singular_quadrature_order));
  h->launches = 0;
  h->stats = wbem_stats{};
  h->stats.n_dofs = h->N;
  h->stats.n_cells = h->C;
  h->factors_valid = false;
  h->have_solution = false;
  const int N = h->N;
  Timer tm(h->stream);
  if (o.method == WBEM_METHOD_FMA) {
    // no dense matrices in this method
    free_mixed(h);
    free_lu(h);
    if (h->d_N) { cudaFree(h->d_N); h->d_N = nullptr; }
    if (h->d_D) { cudaFree(h->d_D); h->d_D = nullptr; }
    h->mat_elems = 0;
    CHK(assemble_fma(h, h->quad));
    h->assembled_prec = kAssembledFma;
  } else if (o.precision == WBEM_PREC_FP64) {
    free_mixed(h);
    const size_t nn = (size_t)N * N;
    if (!h->d_N || h->mat_elems != nn || h->d_A2) {
      if (h->d_A2) { cudaFree(h->d_A2); h->d_A2 = nullptr; }
      if (h->d_B2) { cudaFree(h->d_B2); h->d_B2 = nullptr; }
      CHK(dev_alloc(h, &h->d_N, nn));
      CHK(dev_alloc(h, &h->d_D, nn));
      h->mat_elems = nn;
    }
    if (!h->d_alpha) CHK(dev_alloc(h, &h->d_alpha, (size_t)N));
    const int nq = o.quadrature_order * o.quadrature_order;
    if (h->rec_cells != (size_t)h->C * nq || !h->d_rec) {
      CHK(dev_alloc(h, &h->d_rec, (size_t)h->C * nq * 8));
      h->rec_cells = (size_t)h->C * nq;
    }
    CU(launch_cell_records_fp64(h->C, h->d_X, h->d_cell_dofs, h->d_rec, o.quadrature_order, h->stream));
    h->stats.t_geometry_ms = tm.ms();
    CU(launch_tile_fp64(N, o.quadrature_order, h->d_X, h->d_dnset, h->n_tiles64, h->d_tile_ptr64,
                        h->d_tile_ent64, h->d_cell_dofs, h->d_rec, h->d_N, h->d_D, h->d_err, h->stream));
    h->stats.t_assemble_ms = tm.ms();
    CU(launch_singular_fp64(N, h->d_X, h->d_dnset, h->d_sptr, h->d_scell, h->d_cell_dofs, h->d_N,
                            h->d_D, h->d_err, h->stream));
    h->stats.t_singular_ms = tm.ms();
    CU(launch_alpha_rowsum(N, h->d_N, h->d_alpha, h->stream));
    h->stats.t_alpha_ms = tm.ms();
    h->launches += 4;
    CHK(check_device_error(h, "wbem_assemble"));
    h->assembled_prec = WBEM_PREC_FP64;
  } else {
    CHK(assemble_mixed(h));
    h->assembled_prec = WBEM_PREC_MIXED;
  }
  return WBEM_OK;
}

// Known data in internal order, rhs = compute_rhs(tmp_rhs), constraints.
// beside = true: the mat-vec runs on a low-priority stream, beside whatever
// the caller queues next on the handle's stream (the factorisation); the
// Krylov solve waits for it (rhs_pending / ev_rhs).
static int prepare_rhs(wbem_handle h, const double* tmp_rhs, bool beside = false) {
  const int N = h->N;
  CHK(build_constraints(h, tmp_rhs));
  std::vector<double> bi(N);
  for (int i = 0; i < N; ++i) bi[i] = tmp_rhs[h->perm[i]];
  CU(cudaMemcpyAsync(h->d_b, bi.data(), sizeof(double) * N, cudaMemcpyHostToDevice, h->stream));
  cudaStream_t rs = h->stream;
  if (beside) {
    if (!h->rhs_stream) {
      int lo = 0, hi = 0;
      CU(cudaDeviceGetStreamPriorityRange(&lo, &hi));
      CU(cudaStreamCreateWithPriority(&h->rhs_stream, cudaStreamNonBlocking, lo));
      CU(cudaEventCreateWithFlags(&h->ev_rhs, cudaEventDisableTiming));
    }
    CU(cudaEventRecord(h->ev_rhs, h->stream));
    CU(cudaStreamWaitEvent(h->rhs_stream, h->ev_rhs, 0));
    rs = h->rhs_stream;
  }
  if (h->assembled_prec == kAssembledFma) {
    if (rs != h->stream) {  // the FMA product runs on the handle's stream
      CU(cudaStreamWaitEvent(h->stream, h->ev_rhs, 0));
      rs = h->stream;
    }
    CHK(fma_apply(h, 1, h->d_b, h->d_rhs));
  } else if (h->assembled_prec == WBEM_PREC_FP64)
    CU(launch_matvec_fp64(N, 1, h->d_N, h->d_D, h->d_mask, h->d_alpha, h->d_b, h->d_rhs, rs));
  else
    CU(launch_matvec_mixed(N, 1, h->d_B2, h->d_mask, h->d_alpha, h->d_b, h->d_rhs, rs));
  CU(launch_set_rows(h->n_crows, h->d_crow, h->d_cinh, h->d_rhs, rs));
  h->launches += 2;
  if (rs != h->stream) {
    CU(cudaEventRecord(h->ev_rhs, rs));
    h->rhs_pending = true;
  }
  CU(cudaStreamSynchronize(h->stream));  // bi is read by the copy above
  return WBEM_OK;
}

int wbem_solve_system(wbem_handle h, const double* tmp_rhs, double* phi, double* dphi_dn) {
  if (!h) return WBEM_ERR_ARG;
  if (!tmp_rhs || !phi || !dphi_dn) return fail(h, WBEM_ERR_ARG, "wbem_solve_system: NULL pointer");
  if (h->assembled_prec < 0) return fail(h, WBEM_ERR_STATE, "wbem_solve_system: assemble first");
  if (!h->have_mask) return fail(h, WBEM_ERR_STATE, "wbem_solve_system: set the boundary conditions first");
  const int N = h->N;
  for (int i = 0; i < N; ++i)
    if (!std::isfinite(tmp_rhs[i])) return fail(h, WBEM_ERR_NONFINITE, "wbem_solve_system: non-finite tmp_rhs");
  bool any_dir = false;
  for (int i = 0; i < N; ++i) any_dir |= h->mask[i] != 0;
  if (!any_dir)
    return fail(h, WBEM_ERR_ARG,
                "wbem_solve_system: all-Neumann problems are singular (the reference's norm shift is not a linear operator)");
  cudaSetDevice(h->device);
  CHK(ensure_vectors(h, h->opt.gmres_restart));
  Timer tm(h->stream);
  CHK(prepare_rhs(h, tmp_rhs, /*beside=*/true));
  const double t_rhs = tm.ms();
  CHK(solve_assembled(h, h->d_rhs, h->d_sol, 0));
  // right-hand side + Krylov iterations, without the preconditioner set-up
  // (system formation and factorisation have their own timers)
  h->stats.t_solve_ms = t_rhs + tm.ms() - h->stats.t_system_ms - h->stats.t_factor_ms;
  CHK(check_device_error(h, "wbem_solve_system"));
  // unpack (source/bem_problem.cc:869-879)
  std::vector<double> si(N);
  CU(copy_sync(h, si.data(), h->d_sol, sizeof(double) * N, cudaMemcpyDeviceToHost));
  for (int i = 0; i < N; ++i) {
    if (!std::isfinite(si[i])) return fail(h, WBEM_ERR_NONFINITE, "wbem_solve_system: non-finite solution");
    const int p = h->perm[i];
    if (h->mask[p] == 0) phi[p] = si[i];
    else dphi_dn[p] = si[i];
  }
  h->sol_b.assign(tmp_rhs, tmp_rhs + N);
  h->have_solution = true;
  h->stats.kernel_launches = h->launches;
  return WBEM_OK;
}

int wbem_solve(wbem_handle h, const wbem_options* opt, const double* tmp_rhs, double* phi,
               double* dphi_dn) {
  CHK(wbem_assemble(h, opt));
  return wbem_solve_system(h, tmp_rhs, phi, dphi_dn);
}

int wbem_get_alpha(wbem_handle h, double* alpha) {
  if (!h) return WBEM_ERR_ARG;
  if (!alpha) return fail(h, WBEM_ERR_ARG, "wbem_get_alpha: NULL pointer");
  if (h->assembled_prec < 0) return fail(h, WBEM_ERR_STATE, "wbem_get_alpha: assemble first");
  cudaSetDevice(h->device);
  std::vector<double> a(h->N);
  CU(copy_sync(h, a.data(), h->d_alpha, sizeof(double) * h->N, cudaMemcpyDeviceToHost));
  for (int i = 0; i < h->N; ++i) alpha[h->perm[i]] = a[i];
  return WBEM_OK;
}

int wbem_get_matrices(wbem_handle h, double* neumann, double* dirichlet) {
  if (!h) return WBEM_ERR_ARG;
  if (h->assembled_prec < 0) return fail(h, WBEM_ERR_STATE, "wbem_get_matrices: assemble first");
  if (h->assembled_prec == kAssembledFma)
    return fail(h, WBEM_ERR_STATE, "wbem_get_matrices: the FMA method keeps no dense matrices");
  cudaSetDevice(h->device);
  const int N = h->N;
  const int rows_per = std::max(1, (int)std::min<size_t>((size_t)N, (size_t)(64u << 20) / (8 * (size_t)N)));
  double* buf = nullptr;
  CU(cudaMalloc(&buf, sizeof(double) * (size_t)rows_per * N));
  int st = WBEM_OK;
  for (int which = 0; which < 2 && st == WBEM_OK; ++which) {
    double* out = which == 0 ? neumann : dirichlet;
    if (!out) continue;
    const double* A = which == 0 ? h->d_N : h->d_D;
    // mixed: N = sel ? -B2 : A2, D = sel ? -A2 : B2
    const float2* P0 = which == 0 ? h->d_A2 : h->d_B2;
    const float2* P1 = which == 0 ? h->d_B2 : h->d_A2;
    for (int r0 = 0; r0 < N && st == WBEM_OK; r0 += rows_per) {
      const int nr = std::min(rows_per, N - r0);
      cudaError_t e = launch_gather_rows(N, r0, nr, h->d_iperm, A, P0, P1, h->d_selmask, buf, h->stream);
      if (e != cudaSuccess) st = fail(h, WBEM_ERR_CUDA, cudaGetErrorString(e));
      if (st == WBEM_OK) {
        e = cudaMemcpyAsync(out + (size_t)r0 * N, buf, sizeof(double) * (size_t)nr * N,
                            cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) st = fail(h, WBEM_ERR_CUDA, cudaGetErrorString(e));
      }
    }
  }
  cudaFree(buf);
  return st;
}

static int op_caller(wbem_handle h, int mode, const double* src, double* dst) {
  if (!h) return WBEM_ERR_ARG;
  if (!src || !dst) return fail(h, WBEM_ERR_ARG, "NULL pointer");
  if (h->assembled_prec < 0) return fail(h, WBEM_ERR_STATE, "assemble first");
  if (!h->have_mask) return fail(h, WBEM_ERR_STATE, "set the boundary conditions first");
  cudaSetDevice(h->device);
  CHK(ensure_vectors(h, h->opt.gmres_restart));
  const int N = h->N;
  std::vector<double> xi(N), yi(N);
  for (int i = 0; i < N; ++i) xi[i] = src[h->perm[i]];
  CU(copy_sync(h, h->d_vec[3], xi.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
  if (h->assembled_prec == kAssembledFma)
    CHK(fma_apply(h, mode, h->d_vec[3], h->d_vec[4]));
  else if (h->assembled_prec == WBEM_PREC_FP64)
    CU(launch_matvec_fp64(N, mode, h->d_N, h->d_D, h->d_mask, h->d_alpha, h->d_vec[3], h->d_vec[4], h->stream));
  else
    CU(launch_matvec_mixed(N, mode, mode == 0 ? h->d_A2 : h->d_B2, h->d_mask, h->d_alpha, h->d_vec[3],
                           h->d_vec[4], h->stream));
  CU(copy_sync(h, yi.data(), h->d_vec[4], sizeof(double) * N, cudaMemcpyDeviceToHost));
  for (int i = 0; i < N; ++i) dst[h->perm[i]] = yi[i];
  if (mode == 0) {
    // all-Neumann case of the reference: dst -= ||dst||_2 (source/bem_problem.cc:667-668)
    bool any = false;
    for (int i = 0; i < N; ++i) any |= h->mask[i] != 0;
    if (!any) {
      double s = 0;
      for (int i = 0; i < N; ++i) s += dst[i] * dst[i];
      s = std::sqrt(s);
      for (int i = 0; i < N; ++i) dst[i] -= s;
    }
  }
  return WBEM_OK;
}

int wbem_vmult(wbem_handle h, const double* src, double* dst) { return op_caller(h, 0, src, dst); }
int wbem_compute_rhs(wbem_handle h, const double* src, double* dst) { return op_caller(h, 1, src, dst); }

// BEMProblem::residual (source/bem_problem.cc:903-961): the known data of
// (phi, dphi_dn) forms the right-hand side (compute_rhs + constraints, as a
// solve does), the unknown entries the solution vector, and
// res = A_c sol - rhs_c with the constrained operator.
int wbem_residual(wbem_handle h, const double* phi, const double* dphi_dn, double* res) {
  if (!h) return WBEM_ERR_ARG;
  if (!phi || !dphi_dn || !res) return fail(h, WBEM_ERR_ARG, "wbem_residual: NULL pointer");
  if (h->assembled_prec < 0) return fail(h, WBEM_ERR_STATE, "wbem_residual: assemble first");
  if (!h->have_mask) return fail(h, WBEM_ERR_STATE, "wbem_residual: set the boundary conditions first");
  const int N = h->N;
  for (int i = 0; i < N; ++i)
    if (!std::isfinite(phi[i]) || !std::isfinite(dphi_dn[i]))
      return fail(h, WBEM_ERR_NONFINITE, "wbem_residual: non-finite input");
  cudaSetDevice(h->device);
  CHK(ensure_vectors(h, h->opt.gmres_restart));
  std::vector<double> tmp(N), xi(N), yi(N), ri(N);
  for (int p = 0; p < N; ++p) tmp[p] = h->mask[p] ? phi[p] : dphi_dn[p];
  CHK(prepare_rhs(h, tmp.data()));
  for (int i = 0; i < N; ++i) {
    const int p = h->perm[i];
    xi[i] = h->mask[p] ? dphi_dn[p] : phi[p];
  }
  CU(copy_sync(h, h->d_vec[3], xi.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
  CHK(apply_system(h, h->d_vec[3], h->d_vec[4]));
  CU(copy_sync(h, yi.data(), h->d_vec[4], sizeof(double) * N, cudaMemcpyDeviceToHost));
  CU(copy_sync(h, ri.data(), h->d_rhs, sizeof(double) * N, cudaMemcpyDeviceToHost));
  for (int i = 0; i < N; ++i) res[h->perm[i]] = yi[i];
  bool any = false;
  for (int i = 0; i < N; ++i) any |= h->mask[i] != 0;
  if (!any) {
    // all-Neumann case of the reference's vmult: dst -= ||dst||_2
    double sn = 0;
    for (int i = 0; i < N; ++i) sn += res[i] * res[i];
    sn = std::sqrt(sn);
    for (int i = 0; i < N; ++i) res[i] -= sn;
  }
  for (int i = 0; i < N; ++i) res[h->perm[i]] -= ri[i];
  CHK(check_device_error(h, "wbem_residual"));
  if (h->have_solution) {
    // the adjoint reads the known data of the last solve from d_b
    std::vector<double> bi(N);
    for (int i = 0; i < N; ++i) bi[i] = h->sol_b[h->perm[i]];
    CU(copy_sync(h, h->d_b, bi.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
  }
  return WBEM_OK;
}

int wbem_node_normals(wbem_handle h, double* normals) {
  if (!h) return WBEM_ERR_ARG;
  if (!normals) return fail(h, WBEM_ERR_ARG, "wbem_node_normals: NULL pointer");
  if (h->N == 0) return fail(h, WBEM_ERR_STATE, "wbem_node_normals: set the geometry first");
  std::vector<double> n;
  node_normals(h, n);
  std::copy(n.begin(), n.end(), normals);
  return WBEM_OK;
}

int wbem_surface_gradients(wbem_handle h, const double* tmp_rhs, double* gradients) {
  if (!h) return WBEM_ERR_ARG;
  if (!tmp_rhs || !gradients) return fail(h, WBEM_ERR_ARG, "wbem_surface_gradients: NULL pointer");
  if (h->N == 0) return fail(h, WBEM_ERR_STATE, "wbem_surface_gradients: set the geometry first");
  if (!h->have_mask) return fail(h, WBEM_ERR_STATE, "wbem_surface_gradients: set the boundary conditions first");
  for (int i = 0; i < h->N; ++i)
    if (!std::isfinite(tmp_rhs[i])) return fail(h, WBEM_ERR_NONFINITE, "wbem_surface_gradients: non-finite tmp_rhs");
  std::vector<double> g;
  surface_gradients(h, tmp_rhs, g);
  std::copy(g.begin(), g.end(), gradients);
  return WBEM_OK;
}

int wbem_hull_force(wbem_handle h, const int* hull_cells, int n_hull, const double* U, int dir,
                    const double* phi, const double* dphi_dn, double* force) {
  if (!h) return WBEM_ERR_ARG;
  if (!hull_cells || !U || !phi || !dphi_dn || !force || n_hull < 0 || dir < 0 || dir > 2)
    return fail(h, WBEM_ERR_ARG, "wbem_hull_force: bad argument");
  if (h->N == 0) return fail(h, WBEM_ERR_STATE, "wbem_hull_force: set the geometry first");
  cudaSetDevice(h->device);
  CHK(ensure_vectors(h, h->opt.gmres_restart));
  const int N = h->N;
  std::vector<double> pi(N), qi(N);
  for (int i = 0; i < N; ++i) {
    pi[i] = phi[h->perm[i]];
    qi[i] = dphi_dn[h->perm[i]];
  }
  CU(copy_sync(h, h->d_vec[3], pi.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
  CU(copy_sync(h, h->d_vec[4], qi.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
  return hull_force_dev(h, hull_cells, n_hull, U, dir, h->d_vec[3], h->d_vec[4], force);
}

int wbem_force_adjoint(wbem_handle h, const int* hull_cells, int n_hull, const double* U, int dir,
                       const double* tmp_rhs, double* dF_dX, double* dF_drhs) {
  if (!h) return WBEM_ERR_ARG;
  if (!hull_cells || !U || !tmp_rhs || !dF_dX || !dF_drhs || n_hull < 0 || dir < 0 || dir > 2)
    return fail(h, WBEM_ERR_ARG, "wbem_force_adjoint: bad argument");
  if (!h->have_solution) return fail(h, WBEM_ERR_STATE, "wbem_force_adjoint: solve first");
  cudaSetDevice(h->device);
  return adjoint_force(h, hull_cells, n_hull, U, dir, dF_dX, dF_drhs);
}

int wbem_adjoint(wbem_handle h, const double* dJ_dphi, const double* dJ_ddn, double* dJ_dX,
                 double* dJ_drhs) {
  if (!h) return WBEM_ERR_ARG;
  if (!dJ_dphi || !dJ_ddn || !dJ_dX || !dJ_drhs) return fail(h, WBEM_ERR_ARG, "wbem_adjoint: NULL pointer");
  if (!h->have_solution) return fail(h, WBEM_ERR_STATE, "wbem_adjoint: solve first");
  cudaSetDevice(h->device);
  return adjoint_objective(h, dJ_dphi, dJ_ddn, dJ_dX, dJ_drhs);
}

int wbem_set_profiling(wbem_handle h, int on) {
  if (!h) return WBEM_ERR_ARG;
  h->profiling = on != 0;
  return WBEM_OK;
}

int wbem_get_kernel_profile(wbem_handle h, wbem_kernel_profile* p) {
  if (!h || !p) return WBEM_ERR_ARG;
  std::memset(p, 0, sizeof *p);
  p->gemm_ms = h->prof_gemm.total_ms();
  p->gemm_flop = h->prof_gemm.work;
  p->gemm_launches = (int)h->prof_gemm.used;
  p->diag_ms = h->prof_diag.total_ms();
  p->diag_launches = (int)h->prof_diag.used;
  p->panel_ms = h->prof_panel.total_ms();
  p->panel_launches = (int)h->prof_panel.used;
  p->matvec_ms = h->prof_matvec.total_ms();
  p->matvec_bytes = h->prof_matvec.work;
  p->matvec_launches = (int)h->prof_matvec.used;
  p->trsv_ms = h->prof_trsv.total_ms();
  p->trsv_bytes = h->prof_trsv.work;
  p->trsv_launches = (int)h->prof_trsv.used;
  return WBEM_OK;
}

int wbem_set_stream(wbem_handle h, void* cuda_stream) {
  if (!h) return WBEM_ERR_ARG;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  if (h->own_stream) {
    cudaStreamDestroy(h->stream);
    h->own_stream = false;
  }
  if (cuda_stream) {
    h->stream = static_cast<cudaStream_t>(cuda_stream);
  } else {
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
      return fail(h, WBEM_ERR_CUDA, "wbem_set_stream: stream creation failed");
    h->own_stream = true;
  }
  // graphs captured on the previous stream stay valid (they are launched on h->stream)
  return WBEM_OK;
}

int wbem_get_stats(wbem_handle h, wbem_stats* st) {
  if (!h || !st) return WBEM_ERR_ARG;
  *st = h->stats;
  return WBEM_OK;
}

}  // extern "C"
