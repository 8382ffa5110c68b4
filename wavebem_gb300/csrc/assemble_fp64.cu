// Plain (FP64) assembly of the single-layer matrix D (G) and the double-layer
// matrix N (dG/dn), the vertex-singular correction and alpha.
//
// Restates BEMProblem<3>::assemble_system (source/bem_problem.cc:106-590) and
// compute_alpha (:594-618) of the reference for the GPU:
//   - per-cell quadrature data (Q1 map, normal, JxW; :133-137, :192-196) is
//     computed once per assembly into a record per cell;
//   - k_tile_fp64 gives each CTA a tile of 128 collocation rows x 64 dofs; the
//     records of the panels that touch the tile's dofs are staged into shared
//     memory by the TMA bulk-copy engine (cp.async.bulk, double-buffered on
//     mbarriers); each thread owns one row and accumulates the 4 shape-function
//     entries of every regular panel (:241-260) into a shared-memory tile that
//     is written out with coalesced stores;
//   - panels that hold a node of the row's double-node set are skipped there
//     (:223-230) and integrated by k_singular_fp64 with the vertex-singular
//     rule (:478-522);
//   - alpha = N (-1) is a row reduction (:594-618).
#include <cuda_runtime.h>
#include <stdint.h>
#include "kernels.h"
#include "../../include/wbem.h"

namespace wbem {

static __constant__ QuadTables c_q;

cudaError_t upload_quadrature_fp64(const QuadTables& t) {
  return cudaMemcpyToSymbol(c_q, &t, sizeof(QuadTables));
}

constexpr double kInv4Pi = 0.07957747154594766788;  // 1 / (4 pi)

__device__ __forceinline__ void q1_geometry(const double P[4][3], double xi, double eta,
                                            double x[3], double cr[3]) {
  const double a0 = (1 - xi) * (1 - eta), a1 = xi * (1 - eta), a2 = (1 - xi) * eta, a3 = xi * eta;
  double jx[3], je[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    x[d] = a0 * P[0][d] + a1 * P[1][d] + a2 * P[2][d] + a3 * P[3][d];
    jx[d] = (1 - eta) * (P[1][d] - P[0][d]) + eta * (P[3][d] - P[2][d]);
    je[d] = (1 - xi) * (P[2][d] - P[0][d]) + xi * (P[3][d] - P[1][d]);
  }
  cr[0] = jx[1] * je[2] - jx[2] * je[1];
  cr[1] = jx[2] * je[0] - jx[0] * je[2];
  cr[2] = jx[0] * je[1] - jx[1] * je[0];
}

// Per-cell record: for each regular point q: {x, y, z, JxW/(4 pi), n_x JxW/(4 pi),
// n_y JxW/(4 pi), n_z JxW/(4 pi), 0}.
__global__ void k_cell_records_fp64(int C, const double* __restrict__ X,
                                    const int4* __restrict__ cell_dofs, double* __restrict__ rec) {
  const int nq = c_q.q1 * c_q.q1;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = gid / nq, q = gid % nq;
  if (c >= C) return;
  int4 d = cell_dofs[c];
  double P[4][3];
  const int id[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int e = 0; e < 3; ++e) P[k][e] = X[3 * (size_t)id[k] + e];
  double x[3], cr[3];
  q1_geometry(P, c_q.gp[q][0], c_q.gp[q][1], x, cr);
  const double w = c_q.gp[q][2] * kInv4Pi;
  const double det = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
  double* r = rec + ((size_t)c * nq + q) * 8;
  r[0] = x[0];
  r[1] = x[1];
  r[2] = x[2];
  r[3] = det * w;
  r[4] = cr[0] * w;
  r[5] = cr[1] * w;
  r[6] = cr[2] * w;
  r[7] = 0.0;
}

cudaError_t launch_cell_records_fp64(int C, const double* X, const int4* cell_dofs, double* rec,
                                     int q1, cudaStream_t s) {
  const long total = (long)C * q1 * q1;
  const int bs = 128;
  k_cell_records_fp64<<<(unsigned)((total + bs - 1) / bs), bs, 0, s>>>(C, X, cell_dofs, rec);
  return cudaGetLastError();
}

__device__ __forceinline__ bool in_set(const int set[kMaxSet], int v) {
  bool r = false;
#pragma unroll
  for (int k = 0; k < kMaxSet; ++k) r |= (set[k] == v);
  return r;
}

constexpr int kChunk = 6;  // panels per staged chunk

// Two threads per row (2 * kRowsF64 threads): each takes every other
// quadrature point of a panel; the partial sums are combined through a lane
// shuffle, then one thread adds the N entries and the other the D entries.
constexpr int kF64Threads = 2 * kRowsF64;

template <int Q1>
__global__ void __launch_bounds__(kF64Threads)
    k_tile_fp64(int N, const double* __restrict__ X, const int* __restrict__ dnset,
                const int* __restrict__ tile_ptr, const int2* __restrict__ tile_ent,
                const int4* __restrict__ cell_dofs, const double* __restrict__ rec,
                double* __restrict__ Nm, double* __restrict__ Dm, DevErr* err) {
  constexpr int NQ = Q1 * Q1;
  constexpr int RECD = NQ * 8;  // doubles per panel record
  constexpr int RT = kRowsF64, CT = kColsPerTileF64, LDA = RT + 1;
  extern __shared__ __align__(128) unsigned char smem[];
  double* stage = reinterpret_cast<double*>(smem);  // [2][kChunk][RECD], 128-byte aligned
  double* accN = stage + 2 * kChunk * RECD;         // [CT][LDA]
  double* accD = accN + CT * LDA;
  ChunkMeta* meta = reinterpret_cast<ChunkMeta*>(accD + CT * LDA);
  uint64_t* bar = reinterpret_cast<uint64_t*>(meta + 2 * kChunk);

  const int tid = threadIdx.x;
  const int rt = tid >> 1, half = tid & 1;  // row in the tile, point parity
  const int tile = blockIdx.x;
  const int row0 = blockIdx.y * RT;
  const int row = row0 + rt;
  const bool active = row < N;
  double xi = 0, yi = 0, zi = 0;
  int set[kMaxSet];
#pragma unroll
  for (int k = 0; k < kMaxSet; ++k) set[k] = -2;
  if (active) {
    xi = X[3 * (size_t)row];
    yi = X[3 * (size_t)row + 1];
    zi = X[3 * (size_t)row + 2];
#pragma unroll
    for (int k = 0; k < kMaxSet; ++k) set[k] = dnset[(size_t)row * kMaxSet + k];
  }
  for (int k = tid; k < CT * LDA; k += kF64Threads) {
    accN[k] = 0.0;
    accD[k] = 0.0;
  }
  const int e0 = tile_ptr[tile], e1 = tile_ptr[tile + 1];
  const int nch = (e1 - e0 + kChunk - 1) / kChunk;
  auto load_meta = [&](int c) {
    const int k = tid - 32;
    const int base = e0 + c * kChunk;
    if (k >= 0 && k < kChunk && base + k < e1) {
      const int2 ent = tile_ent[base + k];
      ChunkMeta m;
      m.cell = ent.x & 0x7fffffff;
      m.slots = (uint32_t)ent.y;
      m.owner = ent.x < 0;
      m.pad = 0;
      m.dofs = cell_dofs[m.cell];
      m.geo = make_float4(0.f, 0.f, 0.f, 0.f);
      meta[(c & 1) * kChunk + k] = m;
    }
  };
  if (nch > 0) load_meta(0);
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto issue = [&](int c) {
    const int sidx = c & 1;
    const int base = e0 + c * kChunk;
    const int cnt = min(kChunk, e1 - base);
    mbar_arrive_expect_tx(&bar[sidx], (uint32_t)(cnt * RECD * 8));
    for (int k = 0; k < cnt; ++k) {
      const int cell = tile_ent[base + k].x & 0x7fffffff;
      bulk_g2s(stage + (size_t)(sidx * kChunk + k) * RECD, rec + (size_t)cell * RECD,
               (uint32_t)(RECD * 8), &bar[sidx]);
    }
  };
  if (tid == 0 && nch > 0) issue(0);
  bool in_flight_next = false;

  for (int c = 0; c < nch; ++c) {
    if (tid == 0 && c + 1 < nch) {
      fence_proxy_async_smem();
      issue(c + 1);
    }
    if (c + 1 < nch) load_meta(c + 1);
    in_flight_next = (c + 1 < nch);
    const bool ok = mbar_wait_bounded(&bar[c & 1], (uint32_t)((c >> 1) & 1));
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        dev_fail(err, WBEM_ERR_TIMEOUT, 11, tile, c);
        if (in_flight_next) mbar_wait_bounded(&bar[(c + 1) & 1], (uint32_t)(((c + 1) >> 1) & 1));
      }
      return;
    }
    const int base = e0 + c * kChunk;
    const int cnt = min(kChunk, e1 - base);
    for (int k = 0; k < cnt; ++k) {
      const ChunkMeta& mt = meta[(c & 1) * kChunk + k];
      const uint32_t slots = mt.slots;
      const int4 d = mt.dofs;
      const bool sing = in_set(set, d.x) || in_set(set, d.y) || in_set(set, d.z) || in_set(set, d.w);
      // a skipped row (inactive, or the panel is singular for it) runs no
      // points but still takes part in the shuffle below: every lane of the
      // warp reaches it
      const bool skip = !active || sing;
      const double* r = stage + (size_t)((c & 1) * kChunk + k) * RECD;
      double ln0 = 0, ln1 = 0, ln2 = 0, ln3 = 0, ld0 = 0, ld1 = 0, ld2 = 0, ld3 = 0;
#pragma unroll 4
      for (int q = skip ? NQ : half; q < NQ; q += 2) {
        const double2 p01 = *reinterpret_cast<const double2*>(r + q * 8);
        const double2 p23 = *reinterpret_cast<const double2*>(r + q * 8 + 2);
        const double2 p45 = *reinterpret_cast<const double2*>(r + q * 8 + 4);
        const double p6 = r[q * 8 + 6];
        const double Rx = p01.x - xi, Ry = p01.y - yi, Rz = p23.x - zi;
        const double r2 = fma(Rx, Rx, fma(Ry, Ry, Rz * Rz));
        const double ri = rsqrt(r2);
        const double sq = ri * p23.y;
        const double rn = fma(Rx, p45.x, fma(Ry, p45.y, Rz * p6));
        const double dq = -rn * (ri * ri * ri);
        ln0 = fma(dq, c_q.phi[q][0], ln0);
        ln1 = fma(dq, c_q.phi[q][1], ln1);
        ln2 = fma(dq, c_q.phi[q][2], ln2);
        ln3 = fma(dq, c_q.phi[q][3], ln3);
        ld0 = fma(sq, c_q.phi[q][0], ld0);
        ld1 = fma(sq, c_q.phi[q][1], ld1);
        ld2 = fma(sq, c_q.phi[q][2], ld2);
        ld3 = fma(sq, c_q.phi[q][3], ld3);
      }
      // the row's sums: even points + odd points (the same on both threads)
      double lnv[4] = {ln0, ln1, ln2, ln3}, ldv[4] = {ld0, ld1, ld2, ld3};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const double on = __shfl_xor_sync(0xffffffffu, lnv[j], 1);
        const double od = __shfl_xor_sync(0xffffffffu, ldv[j], 1);
        lnv[j] = half ? on + lnv[j] : lnv[j] + on;
        ldv[j] = half ? od + ldv[j] : ldv[j] + od;
      }
      if (skip) continue;
      double* acc = half ? accD : accN;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t sl = (slots >> (8 * j)) & 255u;
        if (sl != 255u) acc[sl * LDA + rt] += half ? ldv[j] : lnv[j];
      }
    }
    __syncthreads();
  }

  // coalesced write-out of the tile (row-major N x N); the tile's columns:
  // tile_ptr[gridDim.x + 1 + tile] .. (+ 1)
  const int col0 = tile_ptr[gridDim.x + 1 + tile], ncol = tile_ptr[gridDim.x + 2 + tile] - col0;
  for (int idx = tid; idx < RT * CT; idx += kF64Threads) {
    const int rr = idx / CT, cc = idx % CT;
    const int gr = row0 + rr, gc = col0 + cc;
    if (gr < N && cc < ncol) {
      Nm[(size_t)gr * N + gc] = accN[cc * LDA + rr];
      Dm[(size_t)gr * N + gc] = accD[cc * LDA + rr];
    }
  }
}

template <int Q1>
static cudaError_t launch_tile_fp64_t(int N, const double* X, const int* dnset, int n_tiles,
                                      const int* tile_ptr, const int2* tile_ent,
                                      const int4* cell_dofs, const double* rec, double* Nm,
                                      double* Dm, DevErr* err, cudaStream_t s) {
  constexpr int RECD = Q1 * Q1 * 8;
  const size_t smem = (size_t)2 * kChunk * RECD * 8 +
                      (size_t)2 * kColsPerTileF64 * (kRowsF64 + 1) * 8 +
                      2 * kChunk * sizeof(ChunkMeta) + 2 * sizeof(uint64_t);
  cudaError_t e = cudaFuncSetAttribute(k_tile_fp64<Q1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(n_tiles, (N + kRowsF64 - 1) / kRowsF64);
  k_tile_fp64<Q1><<<grid, kF64Threads, smem, s>>>(N, X, dnset, tile_ptr, tile_ent, cell_dofs, rec,
                                                   Nm, Dm, err);
  return cudaGetLastError();
}

cudaError_t launch_tile_fp64(int N, int q1, const double* X, const int* dnset, int n_tiles,
                             const int* tile_ptr, const int2* tile_ent, const int4* cell_dofs,
                             const double* rec, double* Nm, double* Dm, DevErr* err,
                             cudaStream_t s) {
  switch (q1) {
    case 1: return launch_tile_fp64_t<1>(N, X, dnset, n_tiles, tile_ptr, tile_ent, cell_dofs, rec, Nm, Dm, err, s);
    case 2: return launch_tile_fp64_t<2>(N, X, dnset, n_tiles, tile_ptr, tile_ent, cell_dofs, rec, Nm, Dm, err, s);
    case 3: return launch_tile_fp64_t<3>(N, X, dnset, n_tiles, tile_ptr, tile_ent, cell_dofs, rec, Nm, Dm, err, s);
    case 4: return launch_tile_fp64_t<4>(N, X, dnset, n_tiles, tile_ptr, tile_ent, cell_dofs, rec, Nm, Dm, err, s);
    case 5: return launch_tile_fp64_t<5>(N, X, dnset, n_tiles, tile_ptr, tile_ent, cell_dofs, rec, Nm, Dm, err, s);
    case 6: return launch_tile_fp64_t<6>(N, X, dnset, n_tiles, tile_ptr, tile_ent, cell_dofs, rec, Nm, Dm, err, s);
    default: return cudaErrorInvalidValue;
  }
}

// Vertex-singular panels: for row i, every panel holding a node of its
// double-node set; the singular vertex is the first local vertex in the set
// (source/bem_problem.cc:223-230), the rule is the polar vertex rule for that
// vertex (:478-522). One thread per row, panels in ascending order.
__global__ void k_singular_fp64(int N, const double* __restrict__ X, const int* __restrict__ dnset,
                                const int* __restrict__ sptr, const int* __restrict__ scell,
                                const int4* __restrict__ cell_dofs, double* __restrict__ Nm,
                                double* __restrict__ Dm, DevErr* err) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= N) return;
  const double xi = X[3 * (size_t)row], yi = X[3 * (size_t)row + 1], zi = X[3 * (size_t)row + 2];
  int set[kMaxSet];
#pragma unroll
  for (int k = 0; k < kMaxSet; ++k) set[k] = dnset[(size_t)row * kMaxSet + k];
  const int nsp = c_q.nsp;
  for (int e = sptr[row]; e < sptr[row + 1]; ++e) {
    const int cell = scell[e];
    const int4 d = cell_dofs[cell];
    const int id[4] = {d.x, d.y, d.z, d.w};
    int v = -1;
    for (int j = 0; j < 4 && v < 0; ++j)
      if (in_set(set, id[j])) v = j;
    if (v < 0) {
      dev_fail(err, WBEM_ERR_ARG, 21, row, cell);
      continue;
    }
    double P[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) P[k][c] = X[3 * (size_t)id[k] + c];
    double ln[4] = {0, 0, 0, 0}, ld[4] = {0, 0, 0, 0};
    for (int q = 0; q < nsp; ++q) {
      const double s = c_q.sp[v][q][0], t = c_q.sp[v][q][1], w = c_q.sp[v][q][2] * kInv4Pi;
      double x[3], cr[3];
      q1_geometry(P, s, t, x, cr);
      const double det = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      const double Rx = x[0] - xi, Ry = x[1] - yi, Rz = x[2] - zi;
      const double ri = rsqrt(fma(Rx, Rx, fma(Ry, Ry, Rz * Rz)));
      const double sq = ri * det * w;
      const double dq = -(Rx * cr[0] + Ry * cr[1] + Rz * cr[2]) * (ri * ri * ri) * w;
      const double ph[4] = {(1 - s) * (1 - t), s * (1 - t), (1 - s) * t, s * t};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        ln[j] = fma(dq, ph[j], ln[j]);
        ld[j] = fma(sq, ph[j], ld[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      Nm[(size_t)row * N + id[j]] += ln[j];
      Dm[(size_t)row * N + id[j]] += ld[j];
    }
  }
}

cudaError_t launch_singular_fp64(int N, const double* X, const int* dnset, const int* sptr,
                                 const int* scell, const int4* cell_dofs, double* Nm, double* Dm,
                                 DevErr* err, cudaStream_t s) {
  const int bs = 64;
  k_singular_fp64<<<(N + bs - 1) / bs, bs, 0, s>>>(N, X, dnset, sptr, scell, cell_dofs, Nm, Dm, err);
  return cudaGetLastError();
}

// alpha_i = - sum_j N_ij (one warp per row, FP64).
__global__ void k_alpha_rowsum(int N, const double* __restrict__ Nm, double* __restrict__ alpha) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= N) return;
  const double* r = Nm + (size_t)warp * N;
  double s = 0;
  for (int j = lane; j < N; j += 32) s += r[j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) alpha[warp] = -s;
}

cudaError_t launch_alpha_rowsum(int N, const double* Nm, double* alpha, cudaStream_t s) {
  const int bs = 256;
  k_alpha_rowsum<<<(unsigned)(((size_t)N * 32 + bs - 1) / bs), bs, 0, s>>>(N, Nm, alpha);
  return cudaGetLastError();
}

}  // namespace wbem
