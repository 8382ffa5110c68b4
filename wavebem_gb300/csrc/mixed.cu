// Mixed-precision assembly of N (dG/dn) and D (G).
//
// Regular panels far from the collocation point are integrated with the same
// Gauss rule as the reference (source/bem_problem.cc:241-260), but evaluated as
//     k(x_q - x_i) = k(c - x_i) + [k(x_q - x_i) - k(c - x_i)]
// with c the panel centre: the panel term k(c - x_i) (and its contraction with
// the exact panel moments sum_q phi_j(q) JxW_q) is computed once per
// (row, panel) pair in double-float arithmetic on FP32 units, and the
// per-quadrature-point differences are computed in FP32 from cancellation-free
// forms (1/a - 1/b = (b^2 - a^2) / (a b (a + b)) etc.). The FP32 rounding
// then only touches the O(h/r) difference terms, which keeps entries accurate
// to about 1e-9 relative instead of the 1e-7 of plain FP32 evaluation.
// Panels within `ratio` diameters of the collocation point and the singular
// panels are integrated in FP64 (k_near_mixed, k_singular_mixed).
// Entries are stored as (hi, lo) float pairs; alpha = -sum_j N_ij is
// accumulated in FP64 from the three parts.
#include <cuda_runtime.h>
#include <stdint.h>
#include "context.h"
#include "host_util.h"
#include "kernels.h"

namespace wbem {

static __constant__ QuadTables c_qm;
cudaError_t upload_quadrature_mixed(const QuadTables& t) {
  return cudaMemcpyToSymbol(c_qm, &t, sizeof(QuadTables));
}

constexpr double kInv4PiM = 0.07957747154594766788;

__host__ __device__ constexpr int mixed_rec_floats(int nq) { return ((9 * nq + 24 + 3) / 4) * 4; }

// Same near test in every kernel (no contraction: explicit round-to-nearest ops).
__device__ __forceinline__ bool near_test(float xi, float yi, float zi, float4 g) {
  const float dx = __fsub_rn(g.x, xi), dy = __fsub_rn(g.y, yi), dz = __fsub_rn(g.z, zi);
  const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  return d2 < g.w;
}

__device__ __forceinline__ bool in_set_m(const int set[kMaxSet], int v) {
  bool r = false;
#pragma unroll
  for (int k = 0; k < kMaxSet; ++k) r |= (set[k] == v);
  return r;
}

__device__ __forceinline__ void q1_geo(const double P[4][3], double s, double t, double x[3],
                                       double cr[3]) {
  const double a0 = (1 - s) * (1 - t), a1 = s * (1 - t), a2 = (1 - s) * t, a3 = s * t;
  double jx[3], je[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    x[d] = a0 * P[0][d] + a1 * P[1][d] + a2 * P[2][d] + a3 * P[3][d];
    jx[d] = (1 - t) * (P[1][d] - P[0][d]) + t * (P[3][d] - P[2][d]);
    je[d] = (1 - s) * (P[2][d] - P[0][d]) + s * (P[3][d] - P[1][d]);
  }
  cr[0] = jx[1] * je[2] - jx[2] * je[1];
  cr[1] = jx[2] * je[0] - jx[0] * je[2];
  cr[2] = jx[0] * je[1] - jx[1] * je[0];
}

// Outputs of the mixed assembly. The entries are stored with the column's
// boundary condition already applied (sel_j = 1: Dirichlet column):
//   A2_ij = sel_j ? -D_ij : N_ij   (system operator, as vmult applies it)
//   B2_ij = sel_j ? -N_ij : D_ij   (right-hand-side operator, compute_rhs)
// as (hi, lo) float pairs, so that each mat-vec streams one matrix. Optional
// FP32 copy S_ij = hi(A2_ij) (row-major, leading dimension ld); the diagonal
// free term and the constraint rows are added at solve time.
struct SysOut {
  float* S;                  // nullptr: not written
  int ld;
  const uint8_t* sel;        // column selection of A2 / B2
};

// One thread per panel: FP64 geometry -> mixed record + near-test data.
__global__ void k_cell_records_mixed(int C, const double* __restrict__ X,
                                     const int4* __restrict__ cell_dofs, float* __restrict__ rec,
                                     float4* __restrict__ cellgeo, float ratio) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int nq = c_qm.q1 * c_qm.q1;
  const int RF = mixed_rec_floats(nq);
  const int4 d = cell_dofs[c];
  const int id[4] = {d.x, d.y, d.z, d.w};
  double P[4][3];
  for (int k = 0; k < 4; ++k)
    for (int e = 0; e < 3; ++e) P[k][e] = X[3 * (size_t)id[k] + e];
  double cen[3], nu[3] = {0, 0, 0};
  for (int e = 0; e < 3; ++e) cen[e] = 0.25 * (P[0][e] + P[1][e] + P[2][e] + P[3][e]);
  double M[4] = {0, 0, 0, 0};
  for (int q = 0; q < nq; ++q) {
    double x[3], cr[3];
    q1_geo(P, c_qm.gp[q][0], c_qm.gp[q][1], x, cr);
    const double w = c_qm.gp[q][2];
    for (int e = 0; e < 3; ++e) nu[e] += cr[e] * w;
    const double jw = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]) * w * kInv4PiM;
    for (int j = 0; j < 4; ++j) M[j] += c_qm.phi[q][j] * jw;
  }
  const double nl = sqrt(nu[0] * nu[0] + nu[1] * nu[1] + nu[2] * nu[2]);
  for (int e = 0; e < 3; ++e) nu[e] /= nl;
  float* r = rec + (size_t)c * RF;
  for (int q = 0; q < nq; ++q) {
    double x[3], cr[3];
    q1_geo(P, c_qm.gp[q][0], c_qm.gp[q][1], x, cr);
    const double det = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    double del[3], n[3];
    for (int e = 0; e < 3; ++e) {
      del[e] = x[e] - cen[e];
      n[e] = cr[e] / det;
    }
    r[4 * q + 0] = (float)del[0];
    r[4 * q + 1] = (float)del[1];
    r[4 * q + 2] = (float)del[2];
    r[4 * q + 3] = (float)(del[0] * del[0] + del[1] * del[1] + del[2] * del[2]);
    r[4 * nq + 4 * q + 0] = (float)(n[0] - nu[0]);
    r[4 * nq + 4 * q + 1] = (float)(n[1] - nu[1]);
    r[4 * nq + 4 * q + 2] = (float)(n[2] - nu[2]);
    r[4 * nq + 4 * q + 3] = (float)(del[0] * n[0] + del[1] * n[1] + del[2] * n[2]);
    r[8 * nq + q] = (float)(det * c_qm.gp[q][2] * kInv4PiM);
  }
  float* cd = r + 9 * nq;
  for (int e = 0; e < 3; ++e) {
    const df a = df_from_double(cen[e]);
    cd[e] = a.hi;
    cd[3 + e] = a.lo;
    const df b = df_from_double(nu[e]);
    cd[6 + e] = b.hi;
    cd[9 + e] = b.lo;
  }
  double Mt = 0;
  for (int j = 0; j < 4; ++j) {
    const df a = df_from_double(M[j]);
    cd[12 + j] = a.hi;
    cd[16 + j] = a.lo;
    Mt += M[j];
  }
  const df t = df_from_double(Mt);
  cd[20] = t.hi;
  cd[21] = t.lo;
  cd[22] = 0.f;
  cd[23] = 0.f;
  for (int k = 9 * nq + 24; k < RF; ++k) r[k] = 0.f;
  // near test: centre (float) and (ratio * largest diagonal)^2, at least
  // 1.01 x the farthest vertex, so that every panel with the collocation
  // point (or a double-node partner of it) as a vertex tests near: the
  // regular far-field kernel then needs no singular test of its own
  double d1 = 0, d2 = 0, dv = 0;
  for (int e = 0; e < 3; ++e) {
    d1 += (P[3][e] - P[0][e]) * (P[3][e] - P[0][e]);
    d2 += (P[2][e] - P[1][e]) * (P[2][e] - P[1][e]);
  }
  for (int k = 0; k < 4; ++k) {
    double v = 0;
    for (int e = 0; e < 3; ++e) v += (P[k][e] - cen[e]) * (P[k][e] - cen[e]);
    dv = v > dv ? v : dv;
  }
  const double diam = sqrt(d1 > d2 ? d1 : d2);
  const double rad = fmax((double)ratio * diam, 1.01 * sqrt(dv));
  cellgeo[c] = make_float4((float)cen[0], (float)cen[1], (float)cen[2], (float)(rad * rad));
}

constexpr int kChunkM = 8;

template <int Q1>
__global__ void __launch_bounds__(kRowsPerTile)
    k_tile_mixed(int N, const double* __restrict__ X, const int* __restrict__ dnset,
                 const int* __restrict__ tile_ptr, const int2* __restrict__ tile_ent,
                 const int4* __restrict__ cell_dofs, const float* __restrict__ rec,
                 const float4* __restrict__ cellgeo, float2* __restrict__ A2,
                 float2* __restrict__ B2, double* __restrict__ alpha_part, SysOut so,
                 DevErr* err) {
  constexpr int NQ = Q1 * Q1;
  constexpr int RF = mixed_rec_floats(NQ);
  constexpr int RT = kRowsPerTile, CT = kColsPerTile, LDA = RT + 1;
  extern __shared__ __align__(128) unsigned char smem[];
  float* stage = reinterpret_cast<float*>(smem);  // [2][kChunkM][RF]
  float* aNh = stage + 2 * kChunkM * RF;          // [CT][LDA] x 4
  float* aNl = aNh + CT * LDA;
  float* aDh = aNl + CT * LDA;
  float* aDl = aDh + CT * LDA;
  ChunkMeta* meta = reinterpret_cast<ChunkMeta*>(aDl + CT * LDA + ((4 - ((CT * LDA) & 3)) & 3));
  uint64_t* bar = reinterpret_cast<uint64_t*>(meta + 2 * kChunkM);

  const int tid = threadIdx.x;
  const int tile = blockIdx.x;
  const int row0 = blockIdx.y * RT;
  const int row = row0 + tid;
  const bool active = row < N;
  df xr[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  if (active) {
#pragma unroll
    for (int d = 0; d < 3; ++d) xr[d] = df_from_double(X[3 * (size_t)row + d]);
  }
  const float xf = active ? __double2float_rn(X[3 * (size_t)row]) : 0.f;
  const float yf = active ? __double2float_rn(X[3 * (size_t)row + 1]) : 0.f;
  const float zf = active ? __double2float_rn(X[3 * (size_t)row + 2]) : 0.f;
  for (int k = tid; k < CT * LDA; k += RT) {
    aNh[k] = 0.f;
    aNl[k] = 0.f;
    aDh[k] = 0.f;
    aDl[k] = 0.f;
  }
  const int e0 = tile_ptr[tile], e1 = tile_ptr[tile + 1];
  const int nch = (e1 - e0 + kChunkM - 1) / kChunkM;
  // metadata of chunk c into meta[c & 1] (threads 32 .. 32 + kChunkM - 1)
  auto load_meta = [&](int c) {
    const int k = tid - 32;
    const int base = e0 + c * kChunkM;
    if (k >= 0 && k < kChunkM && base + k < e1) {
      const int2 ent = tile_ent[base + k];
      ChunkMeta m;
      m.cell = ent.x & 0x7fffffff;
      m.slots = (uint32_t)ent.y;
      m.owner = ent.x < 0;
      m.pad = 0;
      m.dofs = cell_dofs[m.cell];
      m.geo = cellgeo[m.cell];
      meta[(c & 1) * kChunkM + k] = m;
    }
  };
  if (nch > 0) load_meta(0);
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  df alpha_acc = {0.f, 0.f};

  auto issue = [&](int c) {
    const int sidx = c & 1;
    const int base = e0 + c * kChunkM;
    const int cnt = min(kChunkM, e1 - base);
    mbar_arrive_expect_tx(&bar[sidx], (uint32_t)(cnt * RF * 4));
    for (int k = 0; k < cnt; ++k) {
      const int cell = tile_ent[base + k].x & 0x7fffffff;
      bulk_g2s(stage + (size_t)(sidx * kChunkM + k) * RF, rec + (size_t)cell * RF,
               (uint32_t)(RF * 4), &bar[sidx]);
    }
  };
  if (tid == 0 && nch > 0) issue(0);

  for (int c = 0; c < nch; ++c) {
    if (tid == 0 && c + 1 < nch) {
      fence_proxy_async_smem();
      issue(c + 1);
    }
    if (c + 1 < nch) load_meta(c + 1);
    const bool ok = mbar_wait_bounded(&bar[c & 1], (uint32_t)((c >> 1) & 1));
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        dev_fail(err, WBEM_ERR_TIMEOUT, 41, tile, c);
        if (c + 1 < nch) mbar_wait_bounded(&bar[(c + 1) & 1], (uint32_t)(((c + 1) >> 1) & 1));
      }
      return;
    }
    const int base = e0 + c * kChunkM;
    const int cnt = min(kChunkM, e1 - base);
    for (int k = 0; k < cnt; ++k) {
      const ChunkMeta& mt = meta[(c & 1) * kChunkM + k];
      const bool owner = mt.owner != 0;
      const uint32_t slots = mt.slots;
      // near (FP64 kernel) or singular (always near, see the cell records)
      if (!active || near_test(xf, yf, zf, mt.geo)) continue;
      const float* r = stage + (size_t)((c & 1) * kChunkM + k) * RF;
      const float4* qa = reinterpret_cast<const float4*>(r);
      const float4* qb = reinterpret_cast<const float4*>(r + 4 * NQ);
      const float* qj = r + 8 * NQ;
      const float* cd = r + 9 * NQ;
      // ---- panel base term in double-float
      df R[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        df s = two_sum(cd[d], -xr[d].hi);
        s.lo += cd[3 + d] - xr[d].lo;
        R[d] = fast_two_sum(s.hi, s.lo);
      }
      df r2 = two_prod(R[0].hi, R[0].hi);
      r2.lo = __fmaf_rn(2.f * R[0].hi, R[0].lo, r2.lo);
#pragma unroll
      for (int d = 1; d < 3; ++d) {
        df p = two_prod(R[d].hi, R[d].hi);
        p.lo = __fmaf_rn(2.f * R[d].hi, R[d].lo, p.lo);
        r2 = df_add_fast(r2, p);
      }
      const float y0 = rsqrtf(r2.hi);
      const df t = df_mul(r2, two_prod(y0, y0));
      const float ecor = (1.0f - t.hi) - t.lo;
      const df rinv = fast_two_sum(y0, 0.5f * y0 * ecor);
      const df ri3 = df_mul(df_mul(rinv, rinv), rinv);
      // R . nu in double-float: exact hi products, cross terms into the lo part
      df Rn;
      {
        const df p0 = two_prod(R[0].hi, cd[6]);
        const df p1 = two_prod(R[1].hi, cd[7]);
        const df p2 = two_prod(R[2].hi, cd[8]);
        df s01 = two_sum(p0.hi, p1.hi);
        df s = two_sum(s01.hi, p2.hi);
        float lo = s01.lo + s.lo + (p0.lo + p1.lo + p2.lo);
        lo = __fmaf_rn(R[0].hi, cd[9], __fmaf_rn(R[0].lo, cd[6], lo));
        lo = __fmaf_rn(R[1].hi, cd[10], __fmaf_rn(R[1].lo, cd[7], lo));
        lo = __fmaf_rn(R[2].hi, cd[11], __fmaf_rn(R[2].lo, cd[8], lo));
        Rn = fast_two_sum(s.hi, lo);
      }
      df gR = df_mul(Rn, ri3);
      gR.hi = -gR.hi;
      gR.lo = -gR.lo;
      // ---- per-point differences in FP32
      // with num = rc^2 - rq^2 = -(2 R_c.delta + |delta|^2):
      //   rc - rq = num / (rc + rq),  1/rq - 1/rc = (rc - rq) / (rq rc),
      //   (R.n)(-1/r^3) - (R_c.nu)(-1/rc^3)
      //     = rq^-3 [ (rc - rq)(rc^2 + rc rq + rq^2) (-(R_c.nu) / rc^3) - (R_c.(n - nu) + delta.n) ]
      const float Rcx = R[0].hi, Rcy = R[1].hi, Rcz = R[2].hi;
      const float rcinv = rinv.hi;
      const float rc2 = r2.hi;
      const float rc = rc2 * rcinv;
      const float K1 = -Rn.hi * ri3.hi;
      float ls0 = 0.f, ls1 = 0.f, ls2 = 0.f, ls3 = 0.f, ln0 = 0.f, ln1 = 0.f, ln2 = 0.f, ln3 = 0.f;
#pragma unroll
      for (int bq = 0; bq < Q1; ++bq) {
        // tensor-product accumulation: row sums over xi, then the two eta weights
        float st = 0.f, s1 = 0.f, nt = 0.f, n1 = 0.f;
#pragma unroll
        for (int aq = 0; aq < Q1; ++aq) {
          const int q = aq + Q1 * bq;
          const float4 A = qa[q];
          const float4 B = qb[q];
          const float J = qj[q];
          const float Rd = __fmaf_rn(Rcx, A.x, __fmaf_rn(Rcy, A.y, Rcz * A.z));
          const float num = -__fmaf_rn(2.f, Rd, A.w);
          const float rq2 = rc2 - num;
          const float rqinv = rsqrtf(rq2);
          const float rq = rq2 * rqinv;
          const float dr = __fdividef(num, rc + rq);
          const float u = rqinv * J;
          const float fs = dr * u;  // times 1/rc after the point sums
          const float tsum = __fmaf_rn(rc, rq, rc2) + rq2;
          const float t2 = __fmaf_rn(Rcx, B.x, __fmaf_rn(Rcy, B.y, __fmaf_rn(Rcz, B.z, B.w)));
          const float fn = (rqinv * rqinv) * u * __fmaf_rn(dr * tsum, K1, -t2);
          const float xa = c_qm.gpf[q][0];
          st += fs;
          s1 = __fmaf_rn(fs, xa, s1);
          nt += fn;
          n1 = __fmaf_rn(fn, xa, n1);
        }
        const float eb = c_qm.gpf[Q1 * bq][1];
        const float s0 = st - s1, n0 = nt - n1;
        ls0 = __fmaf_rn(s0, 1.f - eb, ls0);
        ls1 = __fmaf_rn(s1, 1.f - eb, ls1);
        ls2 = __fmaf_rn(s0, eb, ls2);
        ls3 = __fmaf_rn(s1, eb, ls3);
        ln0 = __fmaf_rn(n0, 1.f - eb, ln0);
        ln1 = __fmaf_rn(n1, 1.f - eb, ln1);
        ln2 = __fmaf_rn(n0, eb, ln2);
        ln3 = __fmaf_rn(n1, eb, ln3);
      }
      const float fnsum = (ln0 + ln1) + (ln2 + ln3);
      const float lsv[4] = {ls0 * rcinv, ls1 * rcinv, ls2 * rcinv, ls3 * rcinv};
      const float lnv[4] = {ln0, ln1, ln2, ln3};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t sl = (slots >> (8 * j)) & 255u;
        if (sl != 255u) {
          // acc += k(c) M_j + (FP32 point sum): exact hi product, one
          // two_sum into the accumulator, everything else into its lo part
          // (the pair is renormalised once, when it is written out)
          const float Mh = cd[12 + j], Ml = cd[16 + j];
          const int o = sl * LDA + tid;
          {
            const df p = two_prod(gR.hi, Mh);
            const float pl = __fmaf_rn(gR.hi, Ml, __fmaf_rn(gR.lo, Mh, p.lo));
            const df s2 = two_sum(aNh[o], p.hi);
            aNh[o] = s2.hi;
            aNl[o] = aNl[o] + (s2.lo + (pl + lnv[j]));
          }
          {
            const df p = two_prod(rinv.hi, Mh);
            const float pl = __fmaf_rn(rinv.hi, Ml, __fmaf_rn(rinv.lo, Mh, p.lo));
            const df s2 = two_sum(aDh[o], p.hi);
            aDh[o] = s2.hi;
            aDl[o] = aDl[o] + (s2.lo + (pl + lsv[j]));
          }
        }
      }
      if (owner) alpha_acc = df_add(alpha_acc, df_add_f(df_mul(gR, df{cd[20], cd[21]}), fnsum));
    }
    __syncthreads();
  }
  if (active) alpha_part[(size_t)tile * N + row] = df_to_double(alpha_acc);
  // the tile's columns: tile_ptr[gridDim.x + 1 + tile] .. (+ 1)
  const int col0 = tile_ptr[gridDim.x + 1 + tile], ncol = tile_ptr[gridDim.x + 2 + tile] - col0;
  for (int idx = tid; idx < RT * CT; idx += RT) {
    const int rr = idx / CT, cc = idx % CT;
    const int gr = row0 + rr, gc = col0 + cc;
    if (gr < N && cc < ncol) {
      const int o = cc * LDA + rr;
      const bool dj = so.sel[gc] != 0;
      const df en = two_sum(aNh[o], aNl[o]), ed = two_sum(aDh[o], aDl[o]);
      const float2 a = dj ? make_float2(-ed.hi, -ed.lo) : make_float2(en.hi, en.lo);
      const float2 b = dj ? make_float2(-en.hi, -en.lo) : make_float2(ed.hi, ed.lo);
      A2[(size_t)gr * N + gc] = a;
      B2[(size_t)gr * N + gc] = b;
      if (so.S) so.S[(size_t)gr * so.ld + gc] = a.x;
    }
  }
}

template <int Q1>
static cudaError_t launch_tile_mixed_t(int N, const double* X, const int* dnset, int n_tiles,
                                       const int* tile_ptr, const int2* tile_ent,
                                       const int4* cell_dofs, const float* rec,
                                       const float4* cellgeo, float2* A2, float2* B2,
                                       double* alpha_part, SysOut so, DevErr* err, cudaStream_t s) {
  constexpr int RF = mixed_rec_floats(Q1 * Q1);
  const size_t acc = (size_t)kColsPerTile * (kRowsPerTile + 1);
  const size_t smem = (size_t)2 * kChunkM * RF * 4 + 4 * acc * 4 + 16 +
                      2 * kChunkM * sizeof(ChunkMeta) + 2 * sizeof(uint64_t);
  cudaError_t e = cudaFuncSetAttribute(k_tile_mixed<Q1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(n_tiles, (N + kRowsPerTile - 1) / kRowsPerTile);
  k_tile_mixed<Q1><<<grid, kRowsPerTile, smem, s>>>(N, X, dnset, tile_ptr, tile_ent, cell_dofs, rec,
                                                    cellgeo, A2, B2, alpha_part, so, err);
  return cudaGetLastError();
}

// Near-field and singular contributions of a row are appended as items
// (column, dN, dD) in the order the reference adds them, so that the FP64
// kernels run beside the FP32 far-field kernel (they use different pipes)
// and k_merge_items adds them to the (hi, lo) entries afterwards.
constexpr int kNearItems = 1024;  // per row: 4 items per near panel (256 panels)
constexpr int kSingItems = 128;  // per row: 4 items per singular panel
constexpr int kItemCap = kNearItems + kSingItems;

__device__ __forceinline__ void add_entry(float2* A2, float2* B2, SysOut so, int N, int row, int col,
                                          double dn, double dd) {
  const size_t o = (size_t)row * N + col;
  const bool dj = so.sel[col] != 0;
  float2 v = A2[o];
  double s = (double)v.x + (double)v.y + (dj ? -dd : dn);
  float h = __double2float_rn(s);
  A2[o] = make_float2(h, __double2float_rn(s - (double)h));
  if (so.S) so.S[(size_t)row * so.ld + col] = h;
  v = B2[o];
  s = (double)v.x + (double)v.y + (dj ? -dn : dd);
  h = __double2float_rn(s);
  B2[o] = make_float2(h, __double2float_rn(s - (double)h));
}

// One thread per row: near items, then singular items, in order.
__global__ void k_merge_items(int N, const int* __restrict__ cnt, const int* __restrict__ dof,
                              const double2* __restrict__ val, float2* __restrict__ A2,
                              float2* __restrict__ B2, SysOut so) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= N) return;
  const size_t base = (size_t)row * kItemCap;
  const int nn = min(cnt[2 * row], kNearItems), ns = min(cnt[2 * row + 1], kSingItems);
  for (int k = 0; k < nn; ++k) {
    const double2 v = val[base + k];
    add_entry(A2, B2, so, N, row, dof[base + k], v.x, v.y);
  }
  for (int k = 0; k < ns; ++k) {
    const double2 v = val[base + kNearItems + k];
    add_entry(A2, B2, so, N, row, dof[base + kNearItems + k], v.x, v.y);
  }
}

// Candidate panels of the near field per block of kNearBlock consecutive
// rows (compact surface patches, see the internal dof order): those whose near sphere can
// reach any row of the block, |centre_block - centre_panel| < r_block +
// r_panel, in ascending panel order (ballot prefix sums, deterministic). A
// list that would overflow kNearCap is marked with cnt = -1 and its rows scan
// every panel instead.
constexpr int kNearBlock = 64;
constexpr int kNearCap = 2048;

__global__ void __launch_bounds__(256)
    k_near_candidates(int N, int C, const double* __restrict__ X, const float4* __restrict__ cellgeo,
                      int* __restrict__ cnt, int* __restrict__ list) {
  __shared__ float red[6][256];
  __shared__ int woff[8];
  __shared__ int total;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = blockIdx.x * kNearBlock;
  // bounding box of the block's rows
  float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  if (tid < kNearBlock && r0 + tid < N)
    for (int e = 0; e < 3; ++e) lo[e] = hi[e] = (float)X[3 * (size_t)(r0 + tid) + e];
  for (int e = 0; e < 3; ++e) {
    red[e][tid] = lo[e];
    red[3 + e][tid] = hi[e];
  }
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (tid < o)
      for (int e = 0; e < 3; ++e) {
        red[e][tid] = fminf(red[e][tid], red[e][tid + o]);
        red[3 + e][tid] = fmaxf(red[3 + e][tid], red[3 + e][tid + o]);
      }
    __syncthreads();
  }
  float cen[3], rb2 = 0.f;
  for (int e = 0; e < 3; ++e) {
    cen[e] = 0.5f * (red[e][0] + red[3 + e][0]);
    const float h = 0.5f * (red[3 + e][0] - red[e][0]);
    rb2 += h * h;
  }
  // margin for FP32 rounding of the coordinates and the radii
  const float rb = sqrtf(rb2) * 1.0001f + 1e-6f;
  if (tid == 0) total = 0;
  __syncthreads();
  for (int c0 = 0; c0 < C; c0 += 256) {
    const int c = c0 + tid;
    bool hit = false;
    if (c < C) {
      const float4 g = cellgeo[c];
      const float dx = g.x - cen[0], dy = g.y - cen[1], dz = g.z - cen[2];
      const float reach = sqrtf(g.w) * 1.0001f + rb;
      hit = dx * dx + dy * dy + dz * dz < reach * reach;
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) woff[warp] = __popc(m);
    __syncthreads();
    int base = total;
    for (int w = 0; w < warp; ++w) base += woff[w];
    const int pos = base + __popc(m & ((1u << lane) - 1));
    if (hit && pos < kNearCap) list[(size_t)blockIdx.x * kNearCap + pos] = c;
    __syncthreads();
    if (tid == 0)
      for (int w = 0; w < 8; ++w) total += woff[w];
    __syncthreads();
  }
  if (tid == 0) cnt[blockIdx.x] = total <= kNearCap ? total : -1;
}

// FP64 near field: one warp per row. The lanes test 32 candidate panels at a
// time against the near criterion (same test as the tile kernel); each near,
// non-singular panel is then integrated with the regular rule in FP64, one
// quadrature point per lane, and lane 0 appends its four contributions to the
// row's items in ascending panel order.
__global__ void __launch_bounds__(256)
    k_near_mixed(int N, int C, const double* __restrict__ X, const int* __restrict__ dnset,
                 const int4* __restrict__ cell_dofs, const float4* __restrict__ cellgeo,
                 const double* __restrict__ rec64, int* __restrict__ item_cnt,
                 int* __restrict__ item_dof, double2* __restrict__ item_val,
                 double* __restrict__ alpha_near, const int* __restrict__ ncnt,
                 const int* __restrict__ nlist, DevErr* err) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= N) return;
  const double xi = X[3 * (size_t)row], yi = X[3 * (size_t)row + 1], zi = X[3 * (size_t)row + 2];
  const float xf = __double2float_rn(xi), yf = __double2float_rn(yi), zf = __double2float_rn(zi);
  int set[kMaxSet];
#pragma unroll
  for (int k = 0; k < kMaxSet; ++k) set[k] = dnset[(size_t)row * kMaxSet + k];
  const int nq = c_qm.q1 * c_qm.q1;
  double asum = 0.0;
  int nitem = 0;
  // candidates of this row's block (ascending panel order), else every panel
  const int nc = ncnt[row / kNearBlock];
  const int* cl = nlist + (size_t)(row / kNearBlock) * kNearCap;
  const int ntot = nc >= 0 ? nc : C;
  for (int c0 = 0; c0 < ntot; c0 += 32) {
    const int c = c0 + lane < ntot ? (nc >= 0 ? cl[c0 + lane] : c0 + lane) : -1;
    bool nr = false;
    if (c >= 0 && near_test(xf, yf, zf, cellgeo[c])) {
      const int4 d = cell_dofs[c];
      nr = !(in_set_m(set, d.x) || in_set_m(set, d.y) || in_set_m(set, d.z) || in_set_m(set, d.w));
    }
    unsigned m = __ballot_sync(0xffffffffu, nr);
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1;
      const int cell = __shfl_sync(0xffffffffu, c, b);
      const double* r = rec64 + (size_t)cell * nq * 8;
      double ln[4] = {0, 0, 0, 0}, ld[4] = {0, 0, 0, 0};
      for (int q = lane; q < nq; q += 32) {
        const double Rx = r[8 * q] - xi, Ry = r[8 * q + 1] - yi, Rz = r[8 * q + 2] - zi;
        const double ri = rsqrt(fma(Rx, Rx, fma(Ry, Ry, Rz * Rz)));
        const double sq = ri * r[8 * q + 3];
        const double dq = -fma(Rx, r[8 * q + 4], fma(Ry, r[8 * q + 5], Rz * r[8 * q + 6])) * (ri * ri * ri);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          ln[j] = fma(dq, c_qm.phi[q][j], ln[j]);
          ld[j] = fma(sq, c_qm.phi[q][j], ld[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          ln[j] += __shfl_xor_sync(0xffffffffu, ln[j], o);
          ld[j] += __shfl_xor_sync(0xffffffffu, ld[j], o);
        }
      if (lane == 0) {
        const int4 d = cell_dofs[cell];
        const int id[4] = {d.x, d.y, d.z, d.w};
        for (int j = 0; j < 4; ++j) {
          if (nitem < kNearItems) {
            const size_t o = (size_t)row * kItemCap + nitem;
            item_dof[o] = id[j];
            item_val[o] = make_double2(ln[j], ld[j]);
          }
          ++nitem;
          asum += ln[j];
        }
      }
    }
  }
  if (lane == 0) {
    alpha_near[row] = asum;
    item_cnt[2 * row] = nitem;
    if (nitem > kNearItems) dev_fail(err, WBEM_ERR_NOMEM, 43, row, nitem);
  }
}

// FP64 vertex-singular panels (one thread per row), appended to the row's
// singular items.
__global__ void k_singular_mixed(int N, const double* __restrict__ X, const int* __restrict__ dnset,
                                 const int* __restrict__ sptr, const int* __restrict__ scell,
                                 const int4* __restrict__ cell_dofs, int* __restrict__ item_cnt,
                                 int* __restrict__ item_dof, double2* __restrict__ item_val,
                                 double* __restrict__ alpha_sing, DevErr* err) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= N) return;
  const double xi = X[3 * (size_t)row], yi = X[3 * (size_t)row + 1], zi = X[3 * (size_t)row + 2];
  int set[kMaxSet];
#pragma unroll
  for (int k = 0; k < kMaxSet; ++k) set[k] = dnset[(size_t)row * kMaxSet + k];
  const int nsp = c_qm.nsp;
  double asum = 0.0;
  int nitem = 0;
  for (int e = sptr[row]; e < sptr[row + 1]; ++e) {
    const int cell = scell[e];
    const int4 d = cell_dofs[cell];
    const int id[4] = {d.x, d.y, d.z, d.w};
    int v = -1;
    for (int j = 0; j < 4 && v < 0; ++j)
      if (in_set_m(set, id[j])) v = j;
    if (v < 0) {
      dev_fail(err, WBEM_ERR_ARG, 42, row, cell);
      continue;
    }
    double P[4][3];
    for (int k = 0; k < 4; ++k)
      for (int c = 0; c < 3; ++c) P[k][c] = X[3 * (size_t)id[k] + c];
    double ln[4] = {0, 0, 0, 0}, ld[4] = {0, 0, 0, 0};
    for (int q = 0; q < nsp; ++q) {
      const double s = c_qm.sp[v][q][0], t = c_qm.sp[v][q][1], w = c_qm.sp[v][q][2] * kInv4PiM;
      double x[3], cr[3];
      q1_geo(P, s, t, x, cr);
      const double det = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      const double Rx = x[0] - xi, Ry = x[1] - yi, Rz = x[2] - zi;
      const double ri = rsqrt(fma(Rx, Rx, fma(Ry, Ry, Rz * Rz)));
      const double sq = ri * det * w;
      const double dq = -(Rx * cr[0] + Ry * cr[1] + Rz * cr[2]) * (ri * ri * ri) * w;
      const double ph[4] = {(1 - s) * (1 - t), s * (1 - t), (1 - s) * t, s * t};
      for (int j = 0; j < 4; ++j) {
        ln[j] = fma(dq, ph[j], ln[j]);
        ld[j] = fma(sq, ph[j], ld[j]);
      }
    }
    for (int j = 0; j < 4; ++j) {
      if (nitem < kSingItems) {
        const size_t o = (size_t)row * kItemCap + kNearItems + nitem;
        item_dof[o] = id[j];
        item_val[o] = make_double2(ln[j], ld[j]);
      }
      ++nitem;
      asum += ln[j];
    }
  }
  alpha_sing[row] = asum;
  item_cnt[2 * row + 1] = nitem;
  if (nitem > kSingItems) dev_fail(err, WBEM_ERR_NOMEM, 44, row, nitem);
}

__global__ void k_alpha_mixed(int N, int n_tiles, const double* __restrict__ part,
                              const double* __restrict__ an, const double* __restrict__ as,
                              double* __restrict__ alpha) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double s = 0;
  for (int t = 0; t < n_tiles; ++t) s += part[(size_t)t * N + i];
  alpha[i] = -(s + an[i] + as[i]);
}

#define CUM WB_CU
#define CHKM WB_CHK

void free_mixed(wbem_context* h) {
  if (h->d_A2) { cudaFree(h->d_A2); h->d_A2 = nullptr; }
  if (h->d_B2) { cudaFree(h->d_B2); h->d_B2 = nullptr; }
  if (h->d_lu) { cudaFree(h->d_lu); h->d_lu = nullptr; }
  h->lu_elems = 0;
}

int ensure_system_buffer(wbem_context* h);
int system_ld(int N);

int assemble_mixed(wbem_context* h) {
  const int N = h->N, C = h->C;
  const wbem_options& o = h->opt;
  const int q1 = o.quadrature_order;
  if (q1 < 2 || q1 > 6) {
    h->err = "mixed form supports quadrature orders 2..6";
    return WBEM_ERR_ARG;
  }
  if (!(o.near_field_ratio >= 1.0)) {
    h->err = "near_field_ratio must be >= 1";
    return WBEM_ERR_ARG;
  }
  const size_t nn = (size_t)N * N;
  if (h->d_N) { cudaFree(h->d_N); h->d_N = nullptr; }
  if (h->d_D) { cudaFree(h->d_D); h->d_D = nullptr; }
  if (!h->d_A2 || h->mat_elems != nn) {
    CHKM(dev_alloc(h, &h->d_A2, nn));
    CHKM(dev_alloc(h, &h->d_B2, nn));
    h->mat_elems = nn;
  }
  if (!h->d_alpha) CHKM(dev_alloc(h, &h->d_alpha, (size_t)N));
  CHKM(dev_alloc(h, &h->d_alpha_part, (size_t)h->n_tiles * N));
  CHKM(dev_alloc(h, &h->d_alpha_near, (size_t)N));
  CHKM(dev_alloc(h, &h->d_alpha_sing, (size_t)N));
  const int nq = q1 * q1;
  const int RF = mixed_rec_floats(nq);
  CHKM(dev_alloc(h, &h->d_rec32, (size_t)C * RF));
  CHKM(dev_alloc(h, &h->d_cellgeo, (size_t)C * 4));
  CHKM(dev_alloc(h, &h->d_rec, (size_t)C * nq * 8));
  h->rec_cells = (size_t)C * nq;
  EvTimer tm(h->stream);
  CUM(launch_cell_records_fp64(C, h->d_X, h->d_cell_dofs, h->d_rec, q1, h->stream));
  k_cell_records_mixed<<<(C + 127) / 128, 128, 0, h->stream>>>(
      C, h->d_X, h->d_cell_dofs, h->d_rec32, reinterpret_cast<float4*>(h->d_cellgeo),
      (float)o.near_field_ratio);
  CUM(cudaGetLastError());
  h->stats.t_geometry_ms = tm.ms();
  const float4* geo = reinterpret_cast<const float4*>(h->d_cellgeo);
  // the FP32 system copy for the solvers, written alongside N and D
  // the column selection of A2 / B2: the current mask (none yet: Neumann)
  const bool new_sel = !h->d_selmask || h->sel_mask.size() != (size_t)N;
  h->sel_mask.assign(N, 0);
  if (h->have_mask)
    for (int i = 0; i < N; ++i) h->sel_mask[i] = h->mask[h->perm[i]];
  if (new_sel) CHKM(dev_alloc(h, &h->d_selmask, (size_t)N));
  CUM(cudaMemcpyAsync(h->d_selmask, h->sel_mask.data(), (size_t)N, cudaMemcpyHostToDevice, h->stream));
  SysOut so{nullptr, 0, h->d_selmask};
  if (h->have_mask && h->d_mask) {
    CHKM(ensure_system_buffer(h));
    so.S = h->d_lu;
    so.ld = system_ld(N);
  }
  h->s32_state = 0;
  // near field and singular panels (FP64) on the auxiliary stream, beside the
  // FP32 far-field kernel; their contributions are merged afterwards
  if (!h->aux_stream) {
    // high priority: its CTAs take the free slots beside the far-field CTAs
    // first, so the FP64 work hides under the FP32 kernel
    int lo = 0, hi = 0;
    CUM(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    CUM(cudaStreamCreateWithPriority(&h->aux_stream, cudaStreamNonBlocking, hi));
    CUM(cudaEventCreateWithFlags(&h->ev_aux_fork, cudaEventDisableTiming));
    CUM(cudaEventCreateWithFlags(&h->ev_aux_join, cudaEventDisableTiming));
  }
  if (h->item_rows < (size_t)N) {
    CHKM(dev_alloc(h, &h->d_item_val, (size_t)N * kItemCap));
    CHKM(dev_alloc(h, &h->d_item_dof, (size_t)N * kItemCap));
    CHKM(dev_alloc(h, &h->d_item_cnt, (size_t)2 * N));
    h->item_rows = N;
  }
  {
    const int nblk = (N + kNearBlock - 1) / kNearBlock;
    if (h->near_cap < nblk) {
      CHKM(dev_alloc(h, &h->d_near_cnt, (size_t)nblk));
      CHKM(dev_alloc(h, &h->d_near_cells, (size_t)nblk * kNearCap));
      h->near_cap = nblk;
    }
    cudaStream_t ax = h->aux_stream;
    CUM(cudaEventRecord(h->ev_aux_fork, h->stream));
    CUM(cudaStreamWaitEvent(ax, h->ev_aux_fork, 0));
    k_near_candidates<<<nblk, 256, 0, ax>>>(N, C, h->d_X, geo, h->d_near_cnt, h->d_near_cells);
    CUM(cudaGetLastError());
    k_near_mixed<<<(unsigned)(((size_t)N * 32 + 255) / 256), 256, 0, ax>>>(
        N, C, h->d_X, h->d_dnset, h->d_cell_dofs, geo, h->d_rec, h->d_item_cnt, h->d_item_dof,
        h->d_item_val, h->d_alpha_near, h->d_near_cnt, h->d_near_cells, h->d_err);
    CUM(cudaGetLastError());
    k_singular_mixed<<<(N + 63) / 64, 64, 0, ax>>>(N, h->d_X, h->d_dnset, h->d_sptr, h->d_scell,
                                                    h->d_cell_dofs, h->d_item_cnt, h->d_item_dof,
                                                    h->d_item_val, h->d_alpha_sing, h->d_err);
    CUM(cudaGetLastError());
    CUM(cudaEventRecord(h->ev_aux_join, ax));
  }
  cudaError_t e;
  switch (q1) {
    case 2: e = launch_tile_mixed_t<2>(N, h->d_X, h->d_dnset, h->n_tiles, h->d_tile_ptr, h->d_tile_ent, h->d_cell_dofs, h->d_rec32, geo, h->d_A2, h->d_B2, h->d_alpha_part, so, h->d_err, h->stream); break;
    case 3: e = launch_tile_mixed_t<3>(N, h->d_X, h->d_dnset, h->n_tiles, h->d_tile_ptr, h->d_tile_ent, h->d_cell_dofs, h->d_rec32, geo, h->d_A2, h->d_B2, h->d_alpha_part, so, h->d_err, h->stream); break;
    case 4: e = launch_tile_mixed_t<4>(N, h->d_X, h->d_dnset, h->n_tiles, h->d_tile_ptr, h->d_tile_ent, h->d_cell_dofs, h->d_rec32, geo, h->d_A2, h->d_B2, h->d_alpha_part, so, h->d_err, h->stream); break;
    case 5: e = launch_tile_mixed_t<5>(N, h->d_X, h->d_dnset, h->n_tiles, h->d_tile_ptr, h->d_tile_ent, h->d_cell_dofs, h->d_rec32, geo, h->d_A2, h->d_B2, h->d_alpha_part, so, h->d_err, h->stream); break;
    default: e = launch_tile_mixed_t<6>(N, h->d_X, h->d_dnset, h->n_tiles, h->d_tile_ptr, h->d_tile_ent, h->d_cell_dofs, h->d_rec32, geo, h->d_A2, h->d_B2, h->d_alpha_part, so, h->d_err, h->stream); break;
  }
  CUM(e);
  h->stats.t_assemble_ms = tm.ms();
  // join the near / singular work and add it to the far-field entries
  CUM(cudaStreamWaitEvent(h->stream, h->ev_aux_join, 0));
  k_merge_items<<<(N + 127) / 128, 128, 0, h->stream>>>(N, h->d_item_cnt, h->d_item_dof,
                                                         h->d_item_val, h->d_A2, h->d_B2, so);
  CUM(cudaGetLastError());
  h->stats.t_singular_ms = tm.ms();
  k_alpha_mixed<<<(N + 255) / 256, 256, 0, h->stream>>>(N, h->n_tiles, h->d_alpha_part,
                                                         h->d_alpha_near, h->d_alpha_sing,
                                                         h->d_alpha);
  CUM(cudaGetLastError());
  h->stats.t_alpha_ms = tm.ms();
  if (so.S) h->s32_state = 1;  // entries written; free term and constraints pending
  h->launches += 8;
  return check_device_error(h, "assemble (mixed)");
}

}  // namespace wbem
