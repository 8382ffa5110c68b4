// FP32 blocked LU (no pivoting) of the collocation system with TF32
// tensor-core trailing updates (tcgen05 + TMEM + TMA), and the FP32 block
// triangular solves used as the preconditioner of the FP64 GMRES refinement.
//
// The reference solves with GMRES(100) preconditioned by a direct LU of a
// band of the system (source/bem_problem.cc:821-895, 1107-1149). Here the
// preconditioner is the LU of the whole dense system, so the FP64 GMRES
// (iterative refinement) converges in a few steps. The collocation system of
// the mixed Dirichlet/Neumann problem is factored without pivoting: its
// diagonal (the free term alpha on Neumann columns, the single-layer self
// term on Dirichlet columns) dominates, and every pivot is checked (zero or
// non-finite -> WBEM_ERR_SINGULAR).
//
// Step k (block size kNB = 128), inside outer panels of kNB2 = 512 columns:
//   1. k_diag_block: LU of A_kk (one CTA, registers + shared memory), plus
//      the inverses of its unit-lower and upper factors;
//   2. k_panel_small: L_ik = A_ik inv(U_kk) and U_kj = inv(L_kk) A_kj (FP32
//      SIMT); then the panel's own trailing update A_ij -= L_ik U_kj (FP32,
//      K = 128). Both run first for the next block's 128 rows (the strip the
//      next diagonal block needs) and then, on a second stream, for the rows
//      below.
// Per outer panel P: U12 = inv(L11) A12 for the rest of its rows (FP32, with
// the earlier blocks' updates first; block row k as soon as A_kk is factored,
// on its own stream, writing an FP32 copy of U12^T), then the bulk trailing
// update A22 -= L21 U12 on the tensor cores, k_gemm_tc<true>: one TF32
// product (kind::tf32, L21 read in place from the LU buffer, U12^T from the
// copy) with FP32 accumulation in TMEM, K = 512, persistent 128 x 256 tiles.
// One TF32 product instead of three BF16 products (hi x hi + hi x lo +
// lo x hi) leaves the preconditioner about 20x coarser (residual 1e-4 of a
// vector instead of 5e-6) for one more GMRES iteration, and takes 8% off the
// update, which streams the same operand bytes per K step either way.
// The update is split between the next panel's columns (high-priority
// stream) and the remainder (low-priority stream). The panel kernels have a
// 13 KB footprint, so the next panel's chain runs beside the remainder's CTAs
// on every SM (look-ahead); a few SMs stay free for the 200 KB diagonal
// blocks.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include <atomic>
#include <vector>
#include "context.h"
#include "host_util.h"
#include "kernels.h"

namespace wbem {

constexpr int kNB = 128;   // inner LU block size (diagonal blocks, panels)
constexpr int kNB2 = 512;  // outer block: K of the tensor-core trailing update
constexpr int kLookaheadSMs = 4;  // SMs the bulk trailing update leaves to the panel work

// ------------------------------------------------------------------ input
// LU input: the system operator's pairs rounded to FP32 (A2: the boundary
// condition is already applied), alpha on Neumann diagonals, constrained
// rows replaced by e_i - sum_j c_ij e_j.
__global__ void __launch_bounds__(256)
    k_form_lu(int N, int ld, const float2* __restrict__ A2, const uint8_t* __restrict__ mask,
              const double* __restrict__ alpha, const uint8_t* __restrict__ cflag,
              float* __restrict__ A) {
  // one CTA per row, four consecutive columns per thread and step (two
  // 16-byte loads when the row start is 16-byte aligned)
  const int i = blockIdx.x;
  float* ar = A + (size_t)i * ld;
  if (cflag[i]) {
    for (int j = threadIdx.x; j < N; j += blockDim.x) ar[j] = (j == i) ? 1.f : 0.f;
    return;
  }
  const float2* pr = A2 + (size_t)i * N;
  const bool vec = (N & 1) == 0;
  const double di = mask[i] ? 0.0 : alpha[i];
  auto val = [&](int j, float2 v) -> float {
    double s = (double)v.x + (double)v.y;
    if (j == i) s += di;
    return (float)s;
  };
  for (int j = 4 * threadIdx.x; j < N; j += 4 * blockDim.x) {
    if (j + 3 < N) {
      float2 e[4];
      if (vec) {
        const float4* p = reinterpret_cast<const float4*>(pr + j);
        const float4 a = __ldcs(p), b = __ldcs(p + 1);
        e[0] = make_float2(a.x, a.y);
        e[1] = make_float2(a.z, a.w);
        e[2] = make_float2(b.x, b.y);
        e[3] = make_float2(b.z, b.w);
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u) e[u] = __ldcs(pr + j + u);
      }
      const float4 v = make_float4(val(j, e[0]), val(j + 1, e[1]), val(j + 2, e[2]), val(j + 3, e[3]));
      __stcs(reinterpret_cast<float4*>(ar + j), v);
    } else {
      for (int u = 0; j + u < N; ++u) ar[j + u] = val(j + u, __ldcs(pr + j + u));
    }
  }
}

// entries of the constrained rows (after k_form_lu wrote their identity part)
__global__ void k_lu_constraint_entries(int nrows, const int* __restrict__ crow,
                                        const int* __restrict__ cptr, const int* __restrict__ ccol,
                                        const double* __restrict__ cval, int N, float* __restrict__ A) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nrows) return;
  const int i = crow[k];
  for (int e = cptr[k]; e < cptr[k + 1]; ++e) A[(size_t)i * N + ccol[e]] -= (float)cval[e];
}

// ------------------------------------------------------------ diagonal block
// LU (no pivoting) of the kNB x kNB block at (k0, k0) and the inverses of its
// unit-lower and upper factors; writes the factors back to A, the inverses
// row-major (linv, uinv) and column-major (linvT, uinvT). One CTA, a
// register-resident unblocked elimination with one CTA barrier per pivot and
// every thread busy at every pivot. 1024 threads:
// thread (r, q) holds 16 entries of row r (columns 16q .. 16q+15) in
// registers:
//   * while r > k (row below the pivot) the combined row of the LU: the
//     working matrix right of the pivot, the row of inv(L) left of it (both
//     obey w_r -= l_rk * w_k), the pivot slot turning from a_rk into -l_rk;
//   * from r = k on, the row of Z = inv(U1), U = D U1 (D = diag(U)): the
//     column operations z_rj -= (u_kj / u_kk) z_rk, j > k, that take U to D.
// Each finished row is published to a row history in shared memory (U and
// inv(L) are read from it at the end), each column of Z to the upper
// triangle of the L array when it is final (later steps may leave garbage in
// register slots j <= k of a Z row, none of which is read again), and
// inv(U) = Z D^-1. The pivot loop is unrolled by 16 so every register slot is
// a compile-time index. Warp w takes column block q = w / 4 and row group g
// with g + q = w (mod 4): each scheduler (w mod 4) holds two warps of every
// row group and one of the four warps that own a pivot column.
constexpr int kDLD = kNB + 1;     // padded shared rows
constexpr int kDiagThreads = 1024;
constexpr int kDRowLD = 132;      // row history: 16-byte rows
constexpr size_t kDiagSmemBytes = ((size_t)kNB * kDLD + (size_t)kNB * kDRowLD + 2 * kNB + kNB) * sizeof(float);

__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void __launch_bounds__(kDiagThreads, 1)
    k_diag_block(int ld, int k0, int nb, float* __restrict__ A, float* __restrict__ linv,
                  float* __restrict__ uinv, float* __restrict__ linvT, float* __restrict__ uinvT,
                  DevErr* err) {
  extern __shared__ __align__(16) float dsm[];
  float* sLZ = dsm;                       // [128][129]: input; then L (strict lower), Z (upper)
  float* sRows = sLZ + kNB * kDLD;        // [128][132]: row history (inv(L) | U)
  float* sCol = sRows + kNB * kDRowLD;    // [2][128] pivot column of the rows below
  float* sInv = sCol + 2 * kNB;           // [128] 1 / u_kk
  __shared__ int bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int q = warp >> 2, g = ((warp & 3) - q) & 3;
  const int r = 32 * g + lane, c0 = 16 * q;
  for (int idx = tid; idx < kNB * kNB; idx += kDiagThreads) {
    const int rr = idx >> 7, cc = idx & 127;
    float* dst = sLZ + rr * kDLD + cc;
    if (rr < nb && cc < nb)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                   "l"(A + (size_t)(k0 + rr) * ld + k0 + cc));
    else
      *dst = rr == cc ? 1.f : 0.f;
  }
  asm volatile("cp.async.commit_group;\n cp.async.wait_group 0;" ::: "memory");
  if (tid == 0) bad = 0;
  __syncthreads();
  float w[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) w[i] = sLZ[r * kDLD + c0 + i];  // lanes are rows: distinct banks
  __syncthreads();
  // publish row 0 and column 0; row 0 continues as a Z row
  if (r == 0) {
#pragma unroll
    for (int i = 0; i < 16; i += 4)
      *reinterpret_cast<float4*>(sRows + c0 + i) = make_float4(w[i], w[i + 1], w[i + 2], w[i + 3]);
    if (q == 0) {
      const float p = w[0];
      if (!(fabsf(p) > 0.f && isfinite(p))) bad = 1;
      sInv[0] = rcp_approx(p);
      sLZ[0] = 1.f;
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) w[i] = 0.f;
  }
  if (q == 0 && r > 0) sCol[r] = w[0];
  __syncthreads();
#pragma unroll 1
  for (int kb = 0; kb < 8; ++kb) {
#pragma unroll
    for (int s = 0; s < 16; ++s) {
      if (s == 15 && kb == 7) break;  // the last pivot has nothing below it
      const int k = 16 * kb + s, k1 = k + 1;
      const int s1 = (s + 1) & 15, kb1 = kb + (s == 15 ? 1 : 0);
      const float* row = sRows + k * kDRowLD;
      const float* srcp = r > k ? sCol + (s & 1) * kNB + r : sLZ + r * kDLD + k;
      const float m = *srcp * sInv[k];
      // a warp whose rows are all Z rows and whose columns are all left of
      // the pivot holds only slots that are never read again: skip it
      if (32 * g + 31 > k || c0 + 15 > k) {
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          const float4 v = *reinterpret_cast<const float4*>(row + c0 + i);  // broadcast
          w[i] = __fmaf_rn(-m, v.x, w[i]);
          w[i + 1] = __fmaf_rn(-m, v.y, w[i + 1]);
          w[i + 2] = __fmaf_rn(-m, v.z, w[i + 2]);
          w[i + 3] = __fmaf_rn(-m, v.w, w[i + 3]);
        }
      }
      if (q == kb && r > k) {  // pivot slot of a row below: -l_rk; L keeps l_rk
        w[s] = -m;
        sLZ[r * kDLD + k] = m;
      }
      if (__any_sync(0xffffffffu, r == k1)) {  // warp-uniform: the warp holding row k+1
        if (r == k1) {  // row k+1 is final: publish it, continue as a Z row
          float* nrow = sRows + k1 * kDRowLD;
#pragma unroll
          for (int i = 0; i < 16; i += 4)
            *reinterpret_cast<float4*>(nrow + c0 + i) = make_float4(w[i], w[i + 1], w[i + 2], w[i + 3]);
          if (q == kb1) {
            const float p = w[s1];
            if (!(fabsf(p) > 0.f && isfinite(p))) bad = 1;
            sInv[k1] = rcp_approx(p);
            sLZ[k1 * kDLD + k1] = 1.f;  // z_kk
          }
#pragma unroll
          for (int i = 0; i < 16; ++i) w[i] = 0.f;
        }
      }
      if (q == kb1 && r != k1) {  // column k+1: multipliers below, final Z column above
        float* dst = r > k1 ? sCol + ((s + 1) & 1) * kNB + r : sLZ + r * kDLD + k1;
        *dst = w[s1];
      }
      __syncthreads();
    }
  }
  if (bad) {
    if (tid == 0) dev_fail(err, WBEM_ERR_SINGULAR, 51, k0, 0);
    return;  // uniform
  }
  for (int idx = tid; idx < kNB * kNB; idx += kDiagThreads) {
    const int rr = idx >> 7, cc = idx & 127;
    const float rowv = sRows[rr * kDRowLD + cc];
    if (rr < nb && cc < nb) A[(size_t)(k0 + rr) * ld + k0 + cc] = cc < rr ? sLZ[rr * kDLD + cc] : rowv;
    linv[idx] = cc < rr ? rowv : (cc == rr ? 1.f : 0.f);
    linvT[idx] = rr < cc ? sRows[cc * kDRowLD + rr] : (cc == rr ? 1.f : 0.f);
    uinv[idx] = rr <= cc ? sLZ[rr * kDLD + cc] * sInv[cc] : 0.f;
    uinvT[idx] = cc <= rr ? sLZ[cc * kDLD + rr] * sInv[rr] : 0.f;
  }
}

// ------------------------------------------------------------- panel GEMM
// BF16 hi/lo split of an FP32 value: hi = bf16(v), lo = bf16(v - hi).
__device__ __forceinline__ void split_bf16(float v, uint16_t* hi, uint16_t* lo) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
  *hi = __bfloat16_as_ushort(h);
  *lo = __bfloat16_as_ushort(l);
}

struct SplitOut {
  uint16_t* hi;   // BF16 hi part, row-major rows x ld
  uint16_t* lo;
  int row0;       // absolute matrix index of split row 0
  int ld;         // row length (K of the GEMM that consumes it)
  int coloff;     // column offset inside a row
  float* f32 = nullptr;  // instead of hi / lo: the FP32 values (TF32 operand copy)
};

// FP32 SIMT product of the panel work: out = Lft (rows x K) * Rgt (K x cols),
// K a multiple of 128, written (SET) or subtracted (SUB), optionally with
// BF16 hi/lo splits of the result. In-place use (out == Lft with cols == K,
// or out == Rgt with rows == K) is safe: a CTA reads all it needs before it
// writes, and no other CTA reads its rows (columns).
//   split rows: col_split == 0 -> split row = out row (column panel, L K-major)
//               col_split == 1 -> split row = out column (row panel, U^T K-major)
struct PanelArgs {
  const float* L;  // Lft(i, k) = L[i * ldl + k]
  int ldl;
  const float* R;  // Rgt(k, j) = R[k * ldr + j]
  int ldr;
  float* O;        // out(i, j) = O[i * ldo + j]
  int ldo;
  int rows, cols, K;
  int abs_row0, abs_col0;  // absolute matrix index of out row 0 / column 0 (splits)
  int sub;                 // 1: out -= product, 0: out = product
  int col_split;
};

// Writes (or subtracts) a thread's 4 x 4 quads of a panel product and the
// BF16 splits of the written values, 4 consecutive K entries per 8-byte store.
// Rows {ty*4 + u + 64 hu}, columns {tx*4 + v + 64 hv} of the CTA tile.
template <int RH, int CH>
__device__ __forceinline__ void panel_epilogue(const PanelArgs& pa, const SplitOut& s1,
                                               const SplitOut& s2, float (&acc)[4 * RH][4 * CH],
                                               int i0, int j0, int ty, int tx) {
#pragma unroll
  for (int hu = 0; hu < RH; ++hu)
#pragma unroll
    for (int hv = 0; hv < CH; ++hv) {
      const int ib = i0 + hu * 64 + ty * 4;  // first row of the quad
      const int jb = j0 + hv * 64 + tx * 4;  // first column of the quad
      if (ib >= pa.rows || jb >= pa.cols) continue;
      const int nu = min(4, pa.rows - ib), nv = min(4, pa.cols - jb);
      float r[4][4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) r[u][v] = acc[hu * 4 + u][hv * 4 + v];
      for (int u = 0; u < nu; ++u) {
        float* op = pa.O + (size_t)(ib + u) * pa.ldo + jb;
        if (nv == 4) {
          float4 o4 = make_float4(r[u][0], r[u][1], r[u][2], r[u][3]);
          if (pa.sub) {
            const float4 c = *reinterpret_cast<const float4*>(op);
            o4 = make_float4(c.x - o4.x, c.y - o4.y, c.z - o4.z, c.w - o4.w);
          }
          *reinterpret_cast<float4*>(op) = o4;
          r[u][0] = o4.x; r[u][1] = o4.y; r[u][2] = o4.z; r[u][3] = o4.w;
        } else {
          for (int v = 0; v < nv; ++v) {
            r[u][v] = pa.sub ? op[v] - r[u][v] : r[u][v];
            op[v] = r[u][v];
          }
        }
      }
      // BF16 splits, 4 consecutive K entries packed into one 8-byte store
      for (int w = 0; w < 2; ++w) {
        const SplitOut& so = w == 0 ? s1 : s2;
        if (!so.hi && !so.f32) continue;
        if (pa.col_split) {
          // split row = absolute column, K index = row (4 rows contiguous)
          for (int v = 0; v < nv; ++v) {
            const int aj = pa.abs_col0 + jb + v;
            if (aj < so.row0) continue;
            const size_t o = (size_t)(aj - so.row0) * so.ld + so.coloff + ib;
            if (so.f32) {
              if (nu == 4)
                *reinterpret_cast<float4*>(so.f32 + o) = make_float4(r[0][v], r[1][v], r[2][v], r[3][v]);
              else
                for (int u = 0; u < nu; ++u) so.f32[o + u] = r[u][v];
              continue;
            }
            uint16_t hh[4], ll[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) split_bf16(u < nu ? r[u][v] : 0.f, &hh[u], &ll[u]);
            if (nu == 4) {
              *reinterpret_cast<uint2*>(so.hi + o) = *reinterpret_cast<const uint2*>(hh);
              *reinterpret_cast<uint2*>(so.lo + o) = *reinterpret_cast<const uint2*>(ll);
            } else {
              for (int u = 0; u < nu; ++u) {
                so.hi[o + u] = hh[u];
                so.lo[o + u] = ll[u];
              }
            }
          }
        } else {
          // split row = absolute row, K index = column (4 columns contiguous)
          for (int u = 0; u < nu; ++u) {
            const int ai = pa.abs_row0 + ib + u;
            if (ai < so.row0) continue;
            const size_t o = (size_t)(ai - so.row0) * so.ld + so.coloff + jb;
            if (so.f32) {
              for (int v = 0; v < nv; ++v) so.f32[o + v] = r[u][v];
              continue;
            }
            uint16_t hh[4], ll[4];
#pragma unroll
            for (int v = 0; v < 4; ++v) split_bf16(v < nv ? r[u][v] : 0.f, &hh[v], &ll[v]);
            if (nv == 4) {
              *reinterpret_cast<uint2*>(so.hi + o) = *reinterpret_cast<const uint2*>(hh);
              *reinterpret_cast<uint2*>(so.lo + o) = *reinterpret_cast<const uint2*>(ll);
            } else {
              for (int v = 0; v < nv; ++v) {
                so.hi[o + v] = hh[v];
                so.lo[o + v] = ll[v];
              }
            }
          }
        }
      }
    }
}

// Panel products C = sign * Lft * Rgt (+ C) in FP32 with a 13 KB shared-memory
// footprint: K streams through shared memory 16 at a time (register prefetch
// of the next step),
// so these CTAs fit beside a persistent GEMM CTA (208 KB) on the same SM and
// the panel chain of the next outer panel runs while the bulk trailing update
// holds every SM.
//   TM x TN = 64 x 128 (column panels, full width) or 128 x 64 (row panels
//   and updates, full height); 256 threads, 32 outputs each.
template <int TM, int TN, bool ATRANS>
__global__ void __launch_bounds__(256) k_panel_small(PanelArgs pa, SplitOut s1, SplitOut s2) {
  constexpr int BK = 16;
  constexpr int RH = TM / 64, CH = TN / 64;
  __shared__ __align__(16) float As[BK][TM + 4];
  __shared__ __align__(16) float Bs[BK][TN];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int i0 = blockIdx.x * TM, j0 = blockIdx.y * TN;
  // staging: Lft TM x 16 (TM * 4 quads), Rgt 16 x TN (TN * 4 quads)
  constexpr int LQ = TM * BK / 4 / 256;  // quads per thread (1 or 2)
  constexpr int RQ = TN * BK / 4 / 256;
  float4 la[LQ], rb[RQ];
  auto load = [&](int kk) {
#pragma unroll
    for (int u = 0; u < LQ; ++u) {
      const int q = tid + 256 * u;
      if (ATRANS) {  // LT(k, i): rows of TM floats
        const int k = q / (TM / 4), c = (q % (TM / 4)) * 4;
        la[u] = i0 + c + 3 < pa.rows
                    ? __ldcg(reinterpret_cast<const float4*>(pa.L + (size_t)(kk + k) * pa.ldl + i0 + c))
                    : make_float4(0.f, 0.f, 0.f, 0.f);
      } else {       // L(i, k): rows of 16 floats
        const int i = q >> 2, c = (q & 3) * 4;
        la[u] = i0 + i < pa.rows
                    ? __ldcg(reinterpret_cast<const float4*>(pa.L + (size_t)(i0 + i) * pa.ldl + kk + c))
                    : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
#pragma unroll
    for (int u = 0; u < RQ; ++u) {
      const int q = tid + 256 * u;
      const int k = q / (TN / 4), c = (q % (TN / 4)) * 4;
      const int gj = j0 + c;
      const float* rp = pa.R + (size_t)(kk + k) * pa.ldr + gj;
      if (gj + 3 < pa.cols) {
        rb[u] = __ldcg(reinterpret_cast<const float4*>(rp));
      } else {
        rb[u].x = gj < pa.cols ? rp[0] : 0.f;
        rb[u].y = gj + 1 < pa.cols ? rp[1] : 0.f;
        rb[u].z = gj + 2 < pa.cols ? rp[2] : 0.f;
        rb[u].w = gj + 3 < pa.cols ? rp[3] : 0.f;
      }
    }
  };
  auto stage = [&]() {
#pragma unroll
    for (int u = 0; u < LQ; ++u) {
      const int q = tid + 256 * u;
      if (ATRANS) {
        const int k = q / (TM / 4), c = (q % (TM / 4)) * 4;
        *reinterpret_cast<float4*>(&As[k][c]) = la[u];
      } else {
        const int i = q >> 2, c = (q & 3) * 4;
        As[c + 0][i] = la[u].x;
        As[c + 1][i] = la[u].y;
        As[c + 2][i] = la[u].z;
        As[c + 3][i] = la[u].w;
      }
    }
#pragma unroll
    for (int u = 0; u < RQ; ++u) {
      const int q = tid + 256 * u;
      const int k = q / (TN / 4), c = (q % (TN / 4)) * 4;
      *reinterpret_cast<float4*>(&Bs[k][c]) = rb[u];
    }
  };
  float acc[4 * RH][4 * CH];
#pragma unroll
  for (int u = 0; u < 4 * RH; ++u)
#pragma unroll
    for (int v = 0; v < 4 * CH; ++v) acc[u][v] = 0.f;
  load(0);
  stage();
  __syncthreads();
  const int nk = pa.K / BK;
  for (int kt = 0; kt < nk; ++kt) {
    if (kt + 1 < nk) load((kt + 1) * BK);
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      float a[4 * RH], b[4 * CH];
#pragma unroll
      for (int h = 0; h < RH; ++h) {
        const float4 t = *reinterpret_cast<const float4*>(&As[k][h * 64 + ty * 4]);
        a[4 * h] = t.x; a[4 * h + 1] = t.y; a[4 * h + 2] = t.z; a[4 * h + 3] = t.w;
      }
#pragma unroll
      for (int h = 0; h < CH; ++h) {
        const float4 t = *reinterpret_cast<const float4*>(&Bs[k][h * 64 + tx * 4]);
        b[4 * h] = t.x; b[4 * h + 1] = t.y; b[4 * h + 2] = t.z; b[4 * h + 3] = t.w;
      }
#pragma unroll
      for (int u = 0; u < 4 * RH; ++u)
#pragma unroll
        for (int v = 0; v < 4 * CH; ++v) acc[u][v] = __fmaf_rn(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
    if (kt + 1 < nk) {
      stage();
      __syncthreads();
    }
  }
  panel_epilogue<RH, CH>(pa, s1, s2, acc, i0, j0, ty, tx);
}

template <int TM, int TN, bool ATRANS>
static cudaError_t run_panel_small(const PanelArgs& pa, const SplitOut& s1, const SplitOut& s2,
                                   cudaStream_t s) {
  dim3 g((pa.rows + TM - 1) / TM, (pa.cols + TN - 1) / TN);
  k_panel_small<TM, TN, ATRANS><<<g, 256, 0, s>>>(pa, s1, s2);
  return cudaGetLastError();
}

// ------------------------------------------------------- tcgen05 GEMM (BF16x3 or TF32)
// rows of padding after each split buffer and each padded test operand
constexpr int kSplitPad = 128;

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3}], [%4];" ::"r"(dst),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, "
      "%3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, "
      "%3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}


__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, uint32_t src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   map),
               "r"(x), "r"(y), "r"(src)
               : "memory");
}

// ------------------------------------------------- persistent tcgen05 GEMM
// C[crow0 + m, ccol0 + n] -= sum_k A[arow0 + m, k] B[brow0 + n, k], for the
// large trailing updates. Persistent CTAs (one per SM) walk 128 x 256 output
// tiles (M fastest, so the CTAs in flight share B tiles and stream A); warp
// roles:
//   warp 0     TMA producer: per K step of 32, BF16x3: A hi/lo (128 x 32) and
//              B hi/lo (256 x 32) with 64-byte swizzle; TF32: A and B in
//              FP32 with 128-byte swizzle; a 3-stage ring of 48 KB either way;
//   warp 1     TMEM owner and MMA issuer: per K step 6 kind::f16 tcgen05.mma
//              (M 128, N 256, K 16) or 4 kind::tf32 (K 8) into one of two
//              256-column FP32 accumulators;
//   warps 2-5, 6-9  two epilogue groups, one per accumulator (even / odd
//              tiles of the CTA): per 32-column chunk, the C chunk arrives by
//              TMA into one of the group's two 16 KB buffers (128-byte
//              swizzle), each thread subtracts its TMEM row (tcgen05.ld
//              32x32b.x32), one thread stores the chunk back by TMA and
//              refills the buffer two chunks ahead.
// Each group has two tiles' worth of MMA time for its epilogue, which is
// bound by the latency of the C round trip. Columns at or beyond Nc are neither read nor written (chunk
// granularity: Nc is a multiple of 32 or reaches the matrix edge); rows past
// the matrix edge are clipped by the tensor map.
constexpr int G3M = 128, G3N = 256, G3K = 32, G3S = 3;
constexpr int G3CB = 2;  // C chunk buffers per epilogue group
constexpr uint32_t kA3 = G3M * G3K * 2;                  // 8 KB
constexpr uint32_t kB3 = G3N * G3K * 2;                  // 16 KB
constexpr uint32_t kStage3 = 2 * kA3 + 2 * kB3;          // 48 KB
constexpr uint32_t kC3 = 128 * 32 * 4;                   // 16 KB C chunk
constexpr int kG3Threads = 320;

// K-major FP32 operand tile, 128-byte swizzle: rows of 128 B (32 TF32
// values), 8-row atoms of 1024 B (stride byte offset), layout type 2.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t saddr) {
  // K-major operand tile, 64-byte swizzle: rows of 64 B, 8-row atoms of
  // 512 B (stride byte offset), descriptor version 1 (tcgen05)
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

// Barrier of one epilogue group (named barrier 1 + group, 128 threads). The
// barrier form is warp-aligned: the warp is reconverged first (one lane of
// the group issues the C copies in branches of its own).
__device__ __forceinline__ void named_bar_epi(int g) {
  __syncwarp();
  asm volatile("bar.sync %0, 128;" ::"r"(1 + g) : "memory");
}
// The same barrier, also ORing a flag across the group, so every thread of
// the group takes the same branch after it.
__device__ __forceinline__ bool named_bar_epi_or(int g, bool v) {
  uint32_t r;
  __syncwarp();
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %2, 0;\n bar.red.or.pred q, %1, 128, p;\n selp.u32 %0, "
      "1, 0, q;\n}\n"
      : "=r"(r)
      : "r"(1 + g), "r"((uint32_t)v)
      : "memory");
  return r != 0;
}

// TF32: one kind::tf32 product per K step from FP32 operands (A through mAhi,
// B through mBhi, both 128-byte swizzled boxes of 32 K; A's K coordinates
// start at akoff); the stage holds A (16 KB) and B (32 KB), the same 48 KB.
template <bool TF32>
__global__ void __launch_bounds__(kG3Threads, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap mAhi, const __grid_constant__ CUtensorMap mAlo,
              const __grid_constant__ CUtensorMap mBhi, const __grid_constant__ CUtensorMap mBlo,
              const __grid_constant__ CUtensorMap mC, int crow0, int ccol0, int arow0, int brow0,
              int akoff, int M, int Nc, int K, DevErr* err) {
  extern __shared__ __align__(1024) uint8_t g3sm[];
  const uint32_t base_s = smem_u32(g3sm);
  const uint32_t pad = (1024 - (base_s & 1023)) & 1023;
  uint8_t* sm = g3sm + pad;                    // [G3S stages][Ahi Alo Bhi Blo]
  uint8_t* csm = sm + G3S * kStage3;           // [2 groups][G3CB] C chunk buffers, 1024-aligned
  uint64_t* full = reinterpret_cast<uint64_t*>(csm + 2 * G3CB * kC3);
  uint64_t* empty = full + G3S;
  uint64_t* tfull = empty + G3S;
  uint64_t* tempty = tfull + 2;
  uint64_t* cfull = tempty + 2;                // [2 groups][G3CB]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(cfull + 2 * G3CB);
  int* abort_flag = reinterpret_cast<int*>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_m = (M + G3M - 1) / G3M, tiles_n = (Nc + G3N - 1) / G3N;
  const int ntiles = tiles_m * tiles_n;
  const int nk = K / G3K;

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < G3S; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], 4);  // one arrival per warp of the epilogue group
    }
    for (int i = 0; i < 2 * G3CB; ++i) mbar_init(&cfull[i], 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  volatile int* vabort = abort_flag;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      for (int t = blockIdx.x; t < ntiles && !*vabort; t += gridDim.x) {
        const int m0 = (t % tiles_m) * G3M, n0 = (t / tiles_m) * G3N;
        for (int kb = 0; kb < nk; ++kb) {
          if (!mbar_wait_bounded(&empty[stage], phase ^ 1u)) {
            *vabort = 1;
            dev_fail(err, WBEM_ERR_TIMEOUT, 81, blockIdx.x, t);
            break;
          }
          const uint32_t st = smem_u32(sm + (size_t)stage * kStage3);
          mbar_arrive_expect_tx(&full[stage], kStage3);
          if (TF32) {
            tma_load_2d(st, &mAhi, akoff + kb * G3K, arow0 + m0, &full[stage]);
            tma_load_2d(st + 2 * kA3, &mBhi, kb * G3K, brow0 + n0, &full[stage]);
          } else {
            tma_load_2d(st, &mAhi, kb * G3K, arow0 + m0, &full[stage]);
            tma_load_2d(st + kA3, &mAlo, kb * G3K, arow0 + m0, &full[stage]);
            tma_load_2d(st + 2 * kA3, &mBhi, kb * G3K, brow0 + n0, &full[stage]);
            tma_load_2d(st + 2 * kA3 + kB3, &mBlo, kb * G3K, brow0 + n0, &full[stage]);
          }
          if (++stage == G3S) {
            stage = 0;
            phase ^= 1u;
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      // D f32, A/B bf16 (format 1) or tf32 (format 2), K-major both, N = 256, M = 128
      const uint32_t fmt = TF32 ? 2u : 1u;
      const uint32_t idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(G3N >> 3) << 17) |
                             ((uint32_t)(G3M >> 4) << 24);
      int stage = 0;
      uint32_t phase = 0;
      int acc = 0;
      uint32_t aphase = 0;
      for (int t = blockIdx.x; t < ntiles && !*vabort; t += gridDim.x) {
        if (!mbar_wait_bounded(&tempty[acc], aphase ^ 1u)) {
          *vabort = 1;
          dev_fail(err, WBEM_ERR_TIMEOUT, 82, blockIdx.x, t);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + (uint32_t)(acc * G3N);
        bool ok = true;
        for (int kb = 0; kb < nk; ++kb) {
          if (!mbar_wait_bounded(&full[stage], phase)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = smem_u32(sm + (size_t)stage * kStage3);
          if (TF32) {
            // A: 128 rows x 128 B at st, B: 256 rows x 128 B at st + 16 KB;
            // K = 8 TF32 (32 bytes) per instruction
            const uint64_t dA = smem_desc_sw128(st);
            const uint64_t dB = smem_desc_sw128(st + 2 * kA3);
#pragma unroll
            for (int kk = 0; kk < G3K / 8; ++kk) {
              const uint64_t adv = (uint64_t)(kk * 2);
              umma_tf32(d, dA + adv, dB + adv, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
            }
          } else {
            const uint64_t dAh = smem_desc_sw64(st);
            const uint64_t dAl = smem_desc_sw64(st + kA3);
            const uint64_t dBh = smem_desc_sw64(st + 2 * kA3);
            const uint64_t dBl = smem_desc_sw64(st + 2 * kA3 + kB3);
#pragma unroll
            for (int kk = 0; kk < G3K / 16; ++kk) {
              const uint64_t adv = (uint64_t)(kk * 2);  // 32 bytes along K, in 16-byte units
              umma_bf16(d, dAh + adv, dBh + adv, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
              umma_bf16(d, dAh + adv, dBl + adv, idesc, 1u);
              umma_bf16(d, dAl + adv, dBh + adv, idesc, 1u);
            }
          }
          umma_commit(&empty[stage]);
          if (++stage == G3S) {
            stage = 0;
            phase ^= 1u;
          }
        }
        if (!ok) {
          *vabort = 1;
          dev_fail(err, WBEM_ERR_TIMEOUT, 83, blockIdx.x, t);
          break;
        }
        umma_commit(&tfull[acc]);  // arrives once the tile's MMAs have completed
        if (++acc == 2) {
          acc = 0;
          aphase ^= 1u;
        }
      }
    }
  } else {
    // ------------------------------------------------ epilogue (warps 2..9)
    const int grp = (warp - 2) >> 2;    // group: accumulator and tile parity
    const int etid = tid - 64 - 128 * grp;  // 0..127 within the group
    const int q = warp & 3;             // TMEM lane quarter this warp may access
    const int r = q * 32 + lane;        // tile row = TMEM lane
    const uint32_t rsw = (uint32_t)(r & 7);
    const int acc = grp;
    uint32_t aphase = 0;
    uint32_t cph[2] = {0u, 0u};
    uint8_t* gcsm = csm + (size_t)grp * G3CB * kC3;
    uint64_t* gcfull = cfull + G3CB * grp;
    for (int t = blockIdx.x + grp * gridDim.x; t < ntiles; t += 2 * gridDim.x) {
      const int m0 = (t % tiles_m) * G3M, n0 = (t / tiles_m) * G3N;
      const int nch = min(G3N / 32, (Nc - n0 + 31) / 32);
      if (etid == 0) {
        for (int j = 0; j < G3CB && j < nch; ++j) {
          mbar_arrive_expect_tx(&gcfull[j], kC3);
          tma_load_2d(smem_u32(gcsm + j * kC3), &mC, ccol0 + n0 + 32 * j, crow0 + m0, &gcfull[j]);
        }
      }
      if (!mbar_wait_bounded(&tfull[acc], aphase)) {
        *vabort = 1;
        dev_fail(err, WBEM_ERR_TIMEOUT, 84, blockIdx.x, t);
      }
      if (named_bar_epi_or(grp, *vabort != 0)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      bool stop = false;
      for (int j = 0; j < nch; ++j) {
        const int b = j % G3CB;
        if (!mbar_wait_bounded(&gcfull[b], cph[b])) {
          *vabort = 1;
          dev_fail(err, WBEM_ERR_TIMEOUT, 85, blockIdx.x, t);
        }
        cph[b] ^= 1u;
        if (named_bar_epi_or(grp, *vabort != 0)) {
          stop = true;
          break;
        }
        uint32_t v[32];
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * G3N + 32 * j);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
            "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
            "%28, %29, %30, %31}, [%32];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
              "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
              "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
              "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
              "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
              "=r"(v[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        uint8_t* row = gcsm + b * kC3 + (size_t)r * 128;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          float4* p4 = reinterpret_cast<float4*>(row + (((uint32_t)c ^ rsw) << 4));
          float4 o = *p4;
          o.x -= __uint_as_float(v[4 * c + 0]);
          o.y -= __uint_as_float(v[4 * c + 1]);
          o.z -= __uint_as_float(v[4 * c + 2]);
          o.w -= __uint_as_float(v[4 * c + 3]);
          *p4 = o;
        }
        fence_proxy_async_smem();
        named_bar_epi(grp);
        if (etid == 0) {
          tma_store_2d(&mC, ccol0 + n0 + 32 * j, crow0 + m0, smem_u32(gcsm + b * kC3));
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
          // the buffer is refilled G3CB chunks ahead once the store has read it
          asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
          if (j + G3CB < nch) {
            mbar_arrive_expect_tx(&gcfull[b], kC3);
            tma_load_2d(smem_u32(gcsm + b * kC3), &mC, ccol0 + n0 + 32 * (j + G3CB), crow0 + m0,
                        &gcfull[b]);
          }
        }
      }
      if (stop) break;
      // accumulator read out: release it to the MMA warp
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[acc]);
      aphase ^= 1u;
    }
    if (etid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512)
                 : "memory");
}

static size_t gemm_smem() { return (size_t)G3S * kStage3 + 2 * G3CB * kC3 + 1024 + 256; }


// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library does not link libcuda directly, so it loads on hosts without a
// driver).
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

struct GemmMaps {
  CUtensorMap Ahi, Alo, Bhi, Blo;
};

// The four BF16 planes of a split buffer (A hi, A lo, B hi, B lo; each rows x
// kdim, K-major) as operands of k_gemm_bf16x3: boxes of 32 K x 128 rows (A) and
// 32 K x 256 rows (B), 64-byte swizzle.
static bool encode_ops3(GemmMaps* mp, const uint16_t* ahi, const uint16_t* alo, size_t rows_a,
                        const uint16_t* bhi, const uint16_t* blo, size_t rows_b, int kdim) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return false;
  auto one = [&](CUtensorMap* map, const uint16_t* b, size_t rows, int box_rows) {
    const cuuint64_t dims[2] = {(cuuint64_t)kdim, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)kdim * 2};
    const cuuint32_t box[2] = {(cuuint32_t)G3K, (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)b, dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  return one(&mp->Ahi, ahi, rows_a, G3M) && one(&mp->Alo, alo, rows_a, G3M) &&
         one(&mp->Bhi, bhi, rows_b, G3N) && one(&mp->Blo, blo, rows_b, G3N);
}

// FP32 matrix (rows x cols, leading dimension ld floats, ld % 4 == 0) seen by
// TMA in box_rows x 32 boxes with 128-byte swizzle (the C operand, and the
// TF32 A (128 rows) and B (256 rows) operands).
static bool encode_cmap(CUtensorMap* map, const float* base, int rows, int cols, int ld,
                        int box_rows = 128) {
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 4};
  const cuuint32_t box[2] = {32u, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc || (ld & 3)) return false;
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// C[crow0 + (0..M), ccol0 + (0..Nc)] -= A B^T, with A rows in (Ahi, Alo)
// [rowsA x K] and B rows in (Bhi, Blo) [rowsB x K], both K-major BF16; C
// row crow0 + i pairs with A row arow0 + i, C column ccol0 + j with B row
// brow0 + j. C is
// addressed through its tensor map; rows and columns past the map's extent are
// neither read (zero fill) nor written (clipped), so tiles may overhang M / Nc
// only where the region ends at the matrix edge.
// spare_sms: SMs left free of the persistent CTAs (for concurrent panel work)
template <bool TF32>
static cudaError_t run_gemm(const GemmMaps& mp, const CUtensorMap& cmap, int crow0, int ccol0,
                             int arow0, int brow0, int akoff, int M, int Nc, int K, DevErr* err,
                             cudaStream_t s, int spare_sms = 0) {
  // per device: the shared-memory attribute is set and the SM count read on
  // the first launch there (both idempotent, so racing first launches agree)
  static std::atomic<int> sms_of[kMaxDev];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= kMaxDev) return cudaErrorInvalidDevice;
  int sms = sms_of[dev].load(std::memory_order_acquire);
  if (sms == 0) {
    e = cudaFuncSetAttribute(k_gemm_tc<TF32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)gemm_smem());
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    sms_of[dev].store(sms, std::memory_order_release);
  }
  const int ntiles = ((M + G3M - 1) / G3M) * ((Nc + G3N - 1) / G3N);
  const int grid = std::min(ntiles, std::max(1, sms - spare_sms));
  k_gemm_tc<TF32><<<grid, kG3Threads, gemm_smem(), s>>>(mp.Ahi, mp.Alo, mp.Bhi, mp.Blo, cmap, crow0,
                                                       ccol0, arow0, brow0, akoff, M, Nc, K, err);
  return cudaGetLastError();
}


// ------------------------------------------------------------ triangular solves
// One cooperative launch per triangular sweep: CTA k owns block row k. It
// subtracts the contributions of the already solved blocks as they are
// published (flag[j] == epoch, bounded spin), applies the stored inverse of
// its diagonal block and publishes its own block. Modes:
//   0: L y = w (forward),   1: U x = y (backward),
//   2: U^T y = w (forward), 3: L^T x = y (backward).
// Rows of a block (modes 0/1) or columns (2/3) are read with coalesced loads.
constexpr int kTriThreads = 256;
// Block tile of one step in registers (64 floats per thread), loaded before
// the wait on the block's flag so that the DRAM latency overlaps the wait.
//   modes 0/1 (rows of block (k, j)): warp w holds rows 16 w .. +15, lane l
//       holds columns 4 l .. 4 l + 3 of each;
//   modes 2/3 (columns of block (j, k)): thread t holds column t % 128 of rows
//       t / 128, + 2, + 4, ...
__device__ __forceinline__ void tri_load(float t[64], int mode, const float* __restrict__ LU, int ld,
                                         int k0, int nb, int j0, int jn, bool vec4) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (mode <= 1) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int r = warp * 16 + i;
      const int c = 4 * lane;
      const float* p = LU + (size_t)(k0 + r) * ld + j0 + c;
      if (r < nb && c + 3 < jn && vec4) {
        const float4 v = __ldcs(reinterpret_cast<const float4*>(p));
        t[4 * i] = v.x; t[4 * i + 1] = v.y; t[4 * i + 2] = v.z; t[4 * i + 3] = v.w;
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u) t[4 * i + u] = (r < nb && c + u < jn) ? __ldcs(p + u) : 0.f;
      }
    }
  } else {
    const int c = tid & (kNB - 1), h = tid >> 7;
#pragma unroll
    for (int i = 0; i < 64; ++i) {
      const int r = h + 2 * i;
      t[i] = (c < nb && r < jn) ? __ldcs(LU + (size_t)(j0 + r) * ld + k0 + c) : 0.f;
    }
  }
}

__global__ void __launch_bounds__(kTriThreads)
    k_trsv_wave(int N, int ld, int nblk, int mode, const float* __restrict__ LU,
                const float* __restrict__ dinv, const float* __restrict__ in,
                float* __restrict__ out, unsigned* __restrict__ flags, unsigned epoch,
                DevErr* err) {
  extern __shared__ __align__(16) float tsm[];
  float* sInv = tsm;               // kNB x kNB: thread r reads sInv[c * kNB + r]
  float* acc = sInv + kNB * kNB;   // [kNB]
  float* v = acc + kNB;            // [kNB]
  float* part = v + kNB;           // [2][kNB]
  __shared__ int bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool fwd = (mode == 0 || mode == 2);
  const bool vec4 = (ld & 3) == 0;
  if (tid == 0) bad = 0;
  // A CTA takes the block rows blockIdx.x, blockIdx.x + gridDim.x, ... in
  // sweep order. Block row b waits only for rows earlier in that order, and
  // the owner of the earliest unfinished row has finished all of its earlier
  // rows, so the sweep progresses with any grid size that is co-resident.
  for (int b = blockIdx.x; b < nblk; b += gridDim.x) {
    const int k = fwd ? b : nblk - 1 - b;
    const int k0 = k * kNB, nb = min(kNB, N - k0);
    const float* Dk = dinv + (size_t)k * kNB * kNB;
    for (int idx = tid; idx < kNB * kNB; idx += kTriThreads) sInv[idx] = Dk[idx];
    if (tid < kNB) acc[tid] = (tid < nb) ? in[k0 + tid] : 0.f;
    const int jbeg = fwd ? 0 : nblk - 1, jend = k, jstep = fwd ? 1 : -1;
    float t[64];
    if (jbeg != jend) {
      const int j0 = jbeg * kNB;
      tri_load(t, mode, LU, ld, k0, nb, j0, min(kNB, N - j0), vec4);
    }
    __syncthreads();
    for (int j = jbeg; j != jend; j += jstep) {
      const int j0 = j * kNB, jn = min(kNB, N - j0);
      if (tid == 0 && !bad) {
        uint32_t it = 0;
        while (*((volatile unsigned*)&flags[j]) != epoch) {
          if (++it > (1u << 26)) {
            bad = 1;
            dev_fail(err, WBEM_ERR_TIMEOUT, 71, k, j);
            break;
          }
        }
        __threadfence();
      }
      __syncthreads();
      if (bad) break;
      if (tid < kNB) v[tid] = (tid < jn) ? __ldcg(out + j0 + tid) : 0.f;
      __syncthreads();
      if (mode <= 1) {
        const float4 vv = reinterpret_cast<const float4*>(v)[lane];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          float s2 = t[4 * i] * vv.x;
          s2 = __fmaf_rn(t[4 * i + 1], vv.y, s2);
          s2 = __fmaf_rn(t[4 * i + 2], vv.z, s2);
          s2 = __fmaf_rn(t[4 * i + 3], vv.w, s2);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
          if (lane == 0) acc[warp * 16 + i] -= s2;
        }
      } else {
        // four independent partial sums (the dot product is on the chain)
        const int c = tid & (kNB - 1), h = tid >> 7;
        float q0 = 0.f, q1 = 0.f, q2 = 0.f, q3 = 0.f;
#pragma unroll
        for (int i = 0; i < 64; i += 4) {
          q0 = __fmaf_rn(t[i], v[h + 2 * i], q0);
          q1 = __fmaf_rn(t[i + 1], v[h + 2 * i + 2], q1);
          q2 = __fmaf_rn(t[i + 2], v[h + 2 * i + 4], q2);
          q3 = __fmaf_rn(t[i + 3], v[h + 2 * i + 6], q3);
        }
        part[h * kNB + c] = (q0 + q1) + (q2 + q3);
      }
      // prefetch the next block while the next flag is pending
      const int jn2 = j + jstep;
      if (jn2 != jend) {
        const int j02 = jn2 * kNB;
        tri_load(t, mode, LU, ld, k0, nb, j02, min(kNB, N - j02), vec4);
      }
      __syncthreads();
      if (mode >= 2 && tid < kNB) acc[tid] -= part[tid] + part[kNB + tid];
      __syncthreads();
    }
    // diagonal block (four independent partial sums: this is on the chain)
    if (tid < kNB) {
      float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll 4
      for (int c = 0; c < kNB; c += 4) {
        s0 = __fmaf_rn(sInv[c * kNB + tid], acc[c], s0);
        s1 = __fmaf_rn(sInv[(c + 1) * kNB + tid], acc[c + 1], s1);
        s2 = __fmaf_rn(sInv[(c + 2) * kNB + tid], acc[c + 2], s2);
        s3 = __fmaf_rn(sInv[(c + 3) * kNB + tid], acc[c + 3], s3);
      }
      if (tid < nb) out[k0 + tid] = (s0 + s1) + (s2 + s3);
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      atomicExch(&flags[k], epoch);
    }
    if (bad) break;  // a wait gave up: the status word has it; stop this CTA
  }
}

__global__ void k_to_float(int N, const double* __restrict__ x, float* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) y[i] = (float)x[i];
}
__global__ void k_to_double(int N, const float* __restrict__ x, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) y[i] = (double)x[i];
}

// ------------------------------------------------------------ orchestration
int gmres_mixed_driver(wbem_context* h, const double* rhs, double* x, int transpose);

struct LuState {
  float* linv = nullptr;  // per block kNB x kNB, row-major
  float* uinv = nullptr;
  float* linvT = nullptr;  // column-major copies
  float* uinvT = nullptr;
  // the trailing update's TF32 operands: A = L21 in place in the LU buffer,
  // B = U12^T (K = kNB2 per row) in one of two FP32 copies: the trailing
  // update of outer panel P reads copy P % 2 while panel P + 1 writes the other
  float* u12t[2] = {nullptr, nullptr};
  GemmMaps maps2[2];
  // look-ahead: column work and the next panel's columns of the trailing
  // update on a high-priority stream, the row panel one block behind it on a
  // second one, the rest of the trailing update on a low-priority stream
  cudaStream_t s_panel = nullptr;
  cudaStream_t s_row = nullptr;
  cudaStream_t s_inrow = nullptr;      // in-panel row panel, beside the column panel
  cudaStream_t s_col2 = nullptr;       // column panel and in-panel update below the next block
  cudaStream_t s_trail = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_row = nullptr, ev_trail = nullptr, ev_join = nullptr;
  cudaEvent_t ev_next_rows = nullptr;  // bulk update of the next panel's rows done
  cudaEvent_t ev_blk = nullptr;        // diagonal block ready for its row panel
  cudaEvent_t ev_inrow = nullptr;      // in-panel row panel done
  cudaEvent_t ev_u12 = nullptr;        // row panel of the outer panel done
  cudaEvent_t ev_col2[2] = {nullptr, nullptr};  // s_col2 work of block k done (k % 2)
  float* w = nullptr;         // 2 x N ping-pong vectors
  unsigned* flags = nullptr;  // 4 x nblk publication flags
  unsigned epoch = 0;
  int N = 0;
  int ld = 0;       // leading dimension of the LU buffer (N rounded up to 32)
  CUtensorMap cmap; // the LU buffer as the GEMM's C operand
};

static LuState& lu_state(wbem_context* h) {
  if (!h->lu_state) h->lu_state = new LuState();
  return *static_cast<LuState*>(h->lu_state);
}

void free_lu(wbem_context* h) {
  if (!h->lu_state) return;
  LuState& L = *static_cast<LuState*>(h->lu_state);
  if (L.linv) cudaFree(L.linv);
  if (L.uinv) cudaFree(L.uinv);
  if (L.linvT) cudaFree(L.linvT);
  if (L.uinvT) cudaFree(L.uinvT);
  for (int b = 0; b < 2; ++b)
    if (L.u12t[b]) cudaFree(L.u12t[b]);
  if (L.s_panel) cudaStreamDestroy(L.s_panel);
  if (L.s_trail) cudaStreamDestroy(L.s_trail);
  if (L.s_row) cudaStreamDestroy(L.s_row);
  if (L.s_inrow) cudaStreamDestroy(L.s_inrow);
  if (L.s_col2) cudaStreamDestroy(L.s_col2);
  for (cudaEvent_t e : {L.ev_fork, L.ev_row, L.ev_trail, L.ev_join, L.ev_next_rows, L.ev_blk, L.ev_u12,
                        L.ev_inrow, L.ev_col2[0], L.ev_col2[1]})
    if (e) cudaEventDestroy(e);
  if (L.w) cudaFree(L.w);
  if (L.flags) cudaFree(L.flags);
  delete &L;
  h->lu_state = nullptr;
}

static int tri_sweep(wbem_context* h, LuState& L, int mode, const float* in, float* out) {
  const int N = h->N;
  const int nblk = (N + kNB - 1) / kNB;
  const float* dinv = (mode == 0) ? L.linvT : (mode == 1) ? L.uinvT : (mode == 2) ? L.uinv : L.linv;
  unsigned* flags = L.flags + (size_t)mode * nblk;
  unsigned epoch = ++L.epoch;
  const size_t smem = (size_t)(kNB * kNB + 4 * kNB) * sizeof(float);
  // per device: attribute and co-resident grid size on the first sweep there
  static std::atomic<int> grid_of[kMaxDev];
  int dev = 0;
  WB_CU(cudaGetDevice(&dev));
  if (dev >= kMaxDev) return fail(h, WBEM_ERR_CUDA, "triangular sweep: device index beyond 64");
  int cap = grid_of[dev].load(std::memory_order_acquire);
  if (cap == 0) {
    int sms = 0, per_sm = 0;
    WB_CU(cudaFuncSetAttribute(k_trsv_wave, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    WB_CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    WB_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_wave, kTriThreads, smem));
    cap = per_sm * sms;
    if (cap < 1) return fail(h, WBEM_ERR_CUDA, "triangular sweep: kernel does not fit on an SM");
    grid_of[dev].store(cap, std::memory_order_release);
  }
  // more block rows than co-resident CTAs: each CTA takes block rows
  // blockIdx.x, blockIdx.x + grid, ... in sweep order (no size limit)
  const int grid = std::min(nblk, cap);
  const float* LU = h->d_lu;
  DevErr* err = h->d_err;
  const int ld = L.ld;
  void* args[] = {(void*)&N, (void*)&ld, (void*)&nblk, (void*)&mode, (void*)&LU, (void*)&dinv,
                  (void*)&in, (void*)&out, (void*)&flags, (void*)&epoch, (void*)&err};
  if (h->profiling) h->prof_trsv.begin(h->stream);
  WB_CU(cudaLaunchCooperativeKernel((const void*)k_trsv_wave, dim3(grid), dim3(kTriThreads), args,
                                    smem, h->stream));
  if (h->profiling) h->prof_trsv.end(h->stream, 2.0 * (double)N * N);
  return WBEM_OK;
}

// The constrained system operator as one FP32 matrix in the LU buffer
// (row-major, leading dimension rounded up to 32 floats): the input of the
// LU, and the inner operator of the refinement solver.
int system_ld(int N) { return (N + 31) / 32 * 32; }

int build_constraint_structure(wbem_context* h);

int ensure_system_buffer(wbem_context* h) {
  const size_t nn = (size_t)h->N * system_ld(h->N);
  if (!h->d_lu || h->lu_elems != nn) {
    if (h->d_lu) {
      cudaFree(h->d_lu);
      h->d_lu = nullptr;
    }
    WB_CHK(dev_alloc(h, &h->d_lu, nn));
    h->lu_elems = nn;
    h->s32_state = 0;
  }
  return WBEM_OK;
}

// Completes the system matrix written by the assembly: the free term on the
// Neumann diagonal (hi of N_ii + alpha_i), and the constrained rows, which
// become e_i (their entries follow in k_lu_constraint_entries).
// The free term on the Neumann diagonals of the unconstrained rows, one
// thread per row (the assembly wrote every other entry).
__global__ void k_system_diag(int N, int ld, const float2* __restrict__ A2,
                              const uint8_t* __restrict__ mask, const double* __restrict__ alpha,
                              const uint8_t* __restrict__ cflag, float* __restrict__ A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || cflag[i] || mask[i]) return;
  const float2 n = A2[(size_t)i * N + i];  // N_ii on a Neumann column
  A[(size_t)i * ld + i] = (float)((double)n.x + (double)n.y + alpha[i]);
}

// Constrained rows: identity part, one CTA per constrained row.
__global__ void k_system_crows(int N, int ld, const int* __restrict__ crow, float* __restrict__ A) {
  const int i = crow[blockIdx.x];
  float* ar = A + (size_t)i * ld;
  for (int j = threadIdx.x; j < N; j += blockDim.x) ar[j] = (j == i) ? 1.f : 0.f;
}

int form_system_f32(wbem_context* h) {
  if (!h->d_cflag || !h->d_cptr_full || !h->d_A2 || !h->d_mask || !h->d_alpha)
    return fail(h, WBEM_ERR_STATE, "system matrix: assembly, mask or constraints missing");
  const int N = h->N;
  const int ld = system_ld(N);
  if (h->s32_state == 2) {
    h->stats.t_system_ms = 0.0;
    return WBEM_OK;
  }
  EvTimer tm(h->stream);
  if (h->s32_state == 1) {
    k_system_diag<<<(N + 255) / 256, 256, 0, h->stream>>>(N, ld, h->d_A2, h->d_mask, h->d_alpha,
                                                          h->d_cflag, h->d_lu);
    if (h->n_crows > 0) {
      WB_CU(cudaGetLastError());
      k_system_crows<<<h->n_crows, 256, 0, h->stream>>>(N, ld, h->d_crow, h->d_lu);
      h->launches++;
    }
  } else {
    WB_CHK(ensure_system_buffer(h));
    k_form_lu<<<N, 256, 0, h->stream>>>(N, ld, h->d_A2, h->d_mask, h->d_alpha, h->d_cflag, h->d_lu);
  }
  WB_CU(cudaGetLastError());
  h->launches++;
  if (h->n_crows > 0) {
    k_lu_constraint_entries<<<(h->n_crows + 127) / 128, 128, 0, h->stream>>>(
        h->n_crows, h->d_crow, h->d_cptr, h->d_ccol, h->d_cval, ld, h->d_lu);
    WB_CU(cudaGetLastError());
    h->launches++;
  }
  h->s32_state = 2;
  h->stats.t_system_ms = tm.ms();
  return WBEM_OK;
}

int factor_mixed(wbem_context* h) {
  const int N = h->N;
  const int ld = system_ld(N);
  if (h->lu_state && lu_state(h).N != N) free_lu(h);
  LuState& L = lu_state(h);
  L.N = N;
  L.ld = ld;
  WB_CHK(form_system_f32(h));
  h->s32_state = 0;  // the factorisation overwrites the system matrix
  if (!encode_cmap(&L.cmap, h->d_lu, N, N, ld))
    return fail(h, WBEM_ERR_CUDA, "cuTensorMapEncodeTiled (LU buffer) failed");
  const size_t rows_t = (size_t)N + kSplitPad;
  const int nblk = (N + kNB - 1) / kNB;
  const size_t rows = (size_t)N + kSplitPad;
  if (!L.linv) {
    WB_CHK(dev_alloc(h, &L.linv, (size_t)nblk * kNB * kNB));
    WB_CHK(dev_alloc(h, &L.uinv, (size_t)nblk * kNB * kNB));
    WB_CHK(dev_alloc(h, &L.linvT, (size_t)nblk * kNB * kNB));
    WB_CHK(dev_alloc(h, &L.uinvT, (size_t)nblk * kNB * kNB));
    WB_CHK(dev_alloc(h, &L.u12t[0], rows * kNB2));
    WB_CHK(dev_alloc(h, &L.u12t[1], rows * kNB2));
    WB_CHK(dev_alloc(h, &L.w, (size_t)2 * N));
    WB_CHK(dev_alloc(h, &L.flags, (size_t)4 * nblk));
    WB_CU(cudaMemsetAsync(L.flags, 0, sizeof(unsigned) * 4 * nblk, h->stream));
    L.epoch = 0;
    for (int b = 0; b < 2; ++b)
      WB_CU(cudaMemsetAsync(L.u12t[b], 0, sizeof(float) * rows * kNB2, h->stream));
    int lo = 0, hi = 0;
    WB_CU(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    WB_CU(cudaStreamCreateWithPriority(&L.s_panel, cudaStreamNonBlocking, hi));
    WB_CU(cudaStreamCreateWithPriority(&L.s_trail, cudaStreamNonBlocking, lo));
    WB_CU(cudaStreamCreateWithPriority(&L.s_row, cudaStreamNonBlocking, hi < lo ? hi + 1 : hi));
    WB_CU(cudaStreamCreateWithPriority(&L.s_inrow, cudaStreamNonBlocking, hi));
    WB_CU(cudaStreamCreateWithPriority(&L.s_col2, cudaStreamNonBlocking, hi));
    for (cudaEvent_t* e : {&L.ev_fork, &L.ev_row, &L.ev_trail, &L.ev_join, &L.ev_next_rows, &L.ev_blk,
                           &L.ev_u12, &L.ev_inrow, &L.ev_col2[0], &L.ev_col2[1]})
      WB_CU(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  }
  // the trailing update's operand maps: A = the LU buffer (L21 in place),
  // B = the U12^T copies (256-row boxes)
  for (int b = 0; b < 2; ++b) {
    GemmMaps& m2 = L.maps2[b];
    m2.Ahi = m2.Alo = L.cmap;
    if (!encode_cmap(&m2.Bhi, L.u12t[b], (int)rows_t, kNB2, kNB2, G3N))
      return fail(h, WBEM_ERR_CUDA, "cuTensorMapEncodeTiled (U12 copy) failed");
    m2.Blo = m2.Bhi;
  }
  EvTimer tm(h->stream);
  float* A = h->d_lu;
  const SplitOut none{nullptr, nullptr, 0, 0, 0};
  const size_t kDiagSmem = kDiagSmemBytes;
  WB_CU(cudaFuncSetAttribute(k_diag_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDiagSmem));
  // Right-looking LU over outer panels P = [p0, p1) of kNB2 columns, with
  // look-ahead.
  //   s_panel: the column work of P (diagonal blocks, column panels, inner
  //     updates; columns [p0, p1) only), then the trailing update of the next
  //     panel's columns [p1, p2).
  //   s_inrow: the in-panel row panel of block k (U_kj for the panel's
  //     columns right of the block), beside the column panel of block k.
  //   s_col2: the column panel and the in-panel update of block k for the
  //     rows below block k + 1, beside the diagonal block k + 1; s_panel
  //     does them for the rows of block k + 1 only (the strip the next
  //     diagonal block and the next strip need), so the chain of diagonal
  //     blocks does not wait for the full-height panel products. Block k's
  //     diagonal block needs the s_col2 work of block k - 2 (its rows lie
  //     below block k - 1), the strip of block k that of block k - 1.
  //   s_row: the row panel U12 of P (rows [p0, p1), columns [p1, N)), block
  //     row k as soon as diagonal block k is factored, beside the column work.
  //   s_trail: the trailing update of the columns [p2, N): first the next
  //     panel's rows [p1, p2), then the rows below, beside the column work
  //     of P + 1.
  // Ordering: the row panel of P waits for the first part of the trailing
  // update of P - 1 (its rows), the update of the next panel's columns for
  // the row panel of P and all of the trailing update of P - 1; the trailing
  // update of P waits for the update of the next panel's columns.
  // profiling: one stream, each launch bracketed by events
  const bool prof = h->profiling;
  cudaStream_t sp = prof ? h->stream : L.s_panel, st = prof ? h->stream : L.s_trail;
  cudaStream_t su = prof ? h->stream : L.s_row;
  cudaStream_t sr = prof ? h->stream : L.s_inrow;
  cudaStream_t sc = prof ? h->stream : L.s_col2;
  if (prof) {
    h->prof_gemm.reset();
    h->prof_diag.reset();
    h->prof_panel.reset();
    h->prof_matvec.reset();
    h->prof_trsv.reset();
  }
  auto pb = [&](ProfTimer& t, cudaStream_t s) {
    if (prof) t.begin(s);
  };
  auto pe = [&](ProfTimer& t, cudaStream_t s, double w) {
    if (prof) t.end(s, w);
  };
  auto gemm_flop = [](int M, int Nc, int K) { return 2.0 * M * (double)Nc * K; };
  WB_CU(cudaEventRecord(L.ev_fork, h->stream));
  WB_CU(cudaStreamWaitEvent(sp, L.ev_fork, 0));
  WB_CU(cudaStreamWaitEvent(st, L.ev_fork, 0));
  WB_CU(cudaStreamWaitEvent(su, L.ev_fork, 0));
  WB_CU(cudaStreamWaitEvent(sr, L.ev_fork, 0));
  WB_CU(cudaStreamWaitEvent(sc, L.ev_fork, 0));
  for (int e = 0; e < 2; ++e) WB_CU(cudaEventRecord(L.ev_col2[e], sc));
  bool trail_pending = false;  // a trailing update was queued on s_trail
  for (int p0 = 0; p0 < N; p0 += kNB2) {
    const int p1 = std::min(N, p0 + kNB2);
    const int buf = (p0 / kNB2) & 1;
    float* u12 = L.u12t[buf];
    const int n = N - p1;
    for (int k0 = p0; k0 < p1; k0 += kNB) {
      const int k = k0 / kNB, nb = std::min(kNB, N - k0), k1 = k0 + nb;
      const size_t bo = (size_t)k * kNB * kNB;
      WB_CU(cudaStreamWaitEvent(sp, L.ev_col2[k & 1], 0));  // s_col2 work of block k - 2
      pb(h->prof_diag, sp);
      k_diag_block<<<1, kDiagThreads, kDiagSmem, sp>>>(ld, k0, nb, A, L.linv + bo, L.uinv + bo,
                                                        L.linvT + bo, L.uinvT + bo, h->d_err);
      pe(h->prof_diag, sp, 0.0);
      h->launches++;
      WB_CU(cudaEventRecord(L.ev_blk, sp));
      if (k1 < p1) {
        // U_kj = inv(L_kk) A_kj for the panel's remaining columns, in place,
        // beside the column panel
        WB_CU(cudaStreamWaitEvent(sr, L.ev_blk, 0));
        const PanelArgs pr{L.linvT + bo, kNB, A + (size_t)k0 * ld + k1, ld, A + (size_t)k0 * ld + k1,
                           ld, kNB, p1 - k1, kNB, k0, k1, 0, 1};
        pb(h->prof_panel, sr);
        WB_CU((run_panel_small<128, 64, true>(pr, none, none, sr)));
        pe(h->prof_panel, sr, 0.0);
        WB_CU(cudaEventRecord(L.ev_inrow, sr));
        h->launches++;
      }
      if (p1 < N) {
        // ---- row panel block row k: A_kj -= L_k,[p0,k0) U_[p0,k0),j, then
        // U_kj = inv(L_kk) A_kj, for the columns right of the panel. L_k,[p0,k0)
        // comes from the column panels already queued on s_panel.
        WB_CU(cudaStreamWaitEvent(su, L.ev_blk, 0));
        if (k0 == p0 && trail_pending) WB_CU(cudaStreamWaitEvent(su, L.ev_next_rows, 0));
        pb(h->prof_panel, su);
        if (k0 > p0) {
          const PanelArgs pu{A + (size_t)k0 * ld + p0, ld, A + (size_t)p0 * ld + p1, ld,
                             A + (size_t)k0 * ld + p1, ld, kNB, n, k0 - p0, k0, p1, 1, 0};
          WB_CU((run_panel_small<128, 64, false>(pu, none, none, su)));
          h->launches++;
        }
        const SplitOut U12{nullptr, nullptr, p1, kNB2, k0 - p0, u12};
        const PanelArgs pr{L.linvT + bo, kNB, A + (size_t)k0 * ld + p1, ld, A + (size_t)k0 * ld + p1,
                           ld, kNB, n, kNB, k0, p1, 0, 1};
        WB_CU((run_panel_small<128, 64, true>(pr, U12, none, su)));
        pe(h->prof_panel, su, 0.0);
        h->launches++;
      }
      if (k1 >= N) break;
      const int m = N - k1;
      const int sh = std::min(kNB, m);  // the strip: rows of block k + 1
      const SplitOut l21 = none;  // the trailing update reads L21 in place
      // column panel L_ik = A_ik inv(U_kk), in place: the strip on s_panel
      // (after the s_col2 work of block k - 1, which updated these rows),
      // the rows below on s_col2
      WB_CU(cudaStreamWaitEvent(sp, L.ev_col2[(k + 1) & 1], 0));
      const PanelArgs pc{A + (size_t)k1 * ld + k0, ld, L.uinv + bo, kNB, A + (size_t)k1 * ld + k0,
                         ld, sh, kNB, kNB, k1, k0, 0, 0};
      pb(h->prof_panel, sp);
      WB_CU((run_panel_small<64, 128, false>(pc, none, l21, sp)));
      pe(h->prof_panel, sp, 0.0);
      h->launches++;
      if (m > sh) {
        WB_CU(cudaStreamWaitEvent(sc, L.ev_blk, 0));
        const int k2 = k1 + sh;
        const PanelArgs pc2{A + (size_t)k2 * ld + k0, ld, L.uinv + bo, kNB, A + (size_t)k2 * ld + k0,
                            ld, m - sh, kNB, kNB, k2, k0, 0, 0};
        pb(h->prof_panel, sc);
        WB_CU((run_panel_small<64, 128, false>(pc2, none, l21, sc)));
        pe(h->prof_panel, sc, 0.0);
        h->launches++;
      }
      if (k1 < p1) {
        const int w = p1 - k1;
        // in-panel update A[k1:, k1:p1] -= L_ik U_kj in FP32 (small footprint,
        // so it runs beside the previous outer panel's bulk update): the strip
        // on s_panel, the rows below on s_col2
        WB_CU(cudaStreamWaitEvent(sp, L.ev_inrow, 0));
        const PanelArgs pi{A + (size_t)k1 * ld + k0, ld, A + (size_t)k0 * ld + k1, ld,
                           A + (size_t)k1 * ld + k1, ld, sh, w, kNB, k1, k1, 1, 0};
        pb(h->prof_panel, sp);
        WB_CU((run_panel_small<64, 128, false>(pi, none, none, sp)));
        pe(h->prof_panel, sp, 0.0);
        h->launches++;
        if (m > sh) {
          const int k2 = k1 + sh;
          WB_CU(cudaStreamWaitEvent(sc, L.ev_inrow, 0));
          const PanelArgs pi2{A + (size_t)k2 * ld + k0, ld, A + (size_t)k0 * ld + k1, ld,
                              A + (size_t)k2 * ld + k1, ld, m - sh, w, kNB, k2, k1, 1, 0};
          pb(h->prof_panel, sc);
          WB_CU((run_panel_small<64, 128, false>(pi2, none, none, sc)));
          pe(h->prof_panel, sc, 0.0);
          h->launches++;
        }
      }
      WB_CU(cudaEventRecord(L.ev_col2[k & 1], sc));
      WB_CU(cudaGetLastError());
    }
    if (p1 >= N) break;
    // ---- trailing update A22 -= L21 U12 on the tensor cores (K = kNB2):
    // the next panel's columns on s_panel, the rest on s_trail
    const int p2 = std::min(N, p1 + kNB2);
    WB_CU(cudaEventRecord(L.ev_u12, su));
    WB_CU(cudaStreamWaitEvent(sp, L.ev_u12, 0));
    WB_CU(cudaEventRecord(L.ev_join, sc));  // every column panel's rows below the strips
    WB_CU(cudaStreamWaitEvent(sp, L.ev_join, 0));
    if (trail_pending) WB_CU(cudaStreamWaitEvent(sp, L.ev_trail, 0));
    pb(h->prof_gemm, sp);
    WB_CU(run_gemm<true>(L.maps2[buf], L.cmap, p1, p1, p1, 0, p0, n, p2 - p1, p1 - p0, h->d_err, sp));
    pe(h->prof_gemm, sp, gemm_flop(n, p2 - p1, p1 - p0));
    h->launches++;
    if (p2 < N) {
      WB_CU(cudaEventRecord(L.ev_row, sp));
      WB_CU(cudaStreamWaitEvent(st, L.ev_row, 0));
      // a few SMs stay free for the next panel's diagonal blocks (one
      // 200 KB CTA each); its panel kernels (13 KB CTAs) run beside this
      // update's CTAs on every SM. The next panel's rows [p1, p2) go first,
      // so that its row panel can start while the rows below are updated.
      const int spare = prof ? 0 : kLookaheadSMs;
      pb(h->prof_gemm, st);
      WB_CU(run_gemm<true>(L.maps2[buf], L.cmap, p1, p2, p1, p2 - p1, p0, p2 - p1, N - p2, p1 - p0,
                           h->d_err, st, spare));
      pe(h->prof_gemm, st, gemm_flop(p2 - p1, N - p2, p1 - p0));
      WB_CU(cudaEventRecord(L.ev_next_rows, st));
      pb(h->prof_gemm, st);
      WB_CU(run_gemm<true>(L.maps2[buf], L.cmap, p2, p2, p2, p2 - p1, p0, N - p2, N - p2, p1 - p0,
                           h->d_err, st, spare));
      pe(h->prof_gemm, st, gemm_flop(N - p2, N - p2, p1 - p0));
      WB_CU(cudaEventRecord(L.ev_trail, st));
      trail_pending = true;
      h->launches += 2;
    }
  }
  // join the streams back into the handle's stream
  WB_CU(cudaEventRecord(L.ev_join, sr));
  WB_CU(cudaStreamWaitEvent(h->stream, L.ev_join, 0));
  WB_CU(cudaEventRecord(L.ev_join, sc));
  WB_CU(cudaStreamWaitEvent(h->stream, L.ev_join, 0));
  WB_CU(cudaEventRecord(L.ev_join, su));
  WB_CU(cudaStreamWaitEvent(h->stream, L.ev_join, 0));
  WB_CU(cudaEventRecord(L.ev_join, sp));
  WB_CU(cudaStreamWaitEvent(h->stream, L.ev_join, 0));
  WB_CU(cudaEventRecord(L.ev_join, st));
  WB_CU(cudaStreamWaitEvent(h->stream, L.ev_join, 0));
  WB_CHK(check_device_error(h, "LU factorisation"));
  h->stats.t_factor_ms = tm.ms();
  return WBEM_OK;
}

// z = M^{-1} v with M = L U (FP32 factors), FP64 in/out.
int lu_apply(wbem_context* h, const double* v, double* z, int transpose) {
  LuState& L = lu_state(h);
  const int N = h->N;
  float* w0 = L.w;
  float* w1 = L.w + N;
  k_to_float<<<(N + 255) / 256, 256, 0, h->stream>>>(N, v, w0);
  WB_CU(cudaGetLastError());
  if (!transpose) {
    WB_CHK(tri_sweep(h, L, 0, w0, w1));  // L y = v
    WB_CHK(tri_sweep(h, L, 1, w1, w0));  // U z = y
  } else {
    WB_CHK(tri_sweep(h, L, 2, w0, w1));  // U^T y = v
    WB_CHK(tri_sweep(h, L, 3, w1, w0));  // L^T z = y
  }
  k_to_double<<<(N + 255) / 256, 256, 0, h->stream>>>(N, w0, z);
  WB_CU(cudaGetLastError());
  h->launches += 4;
  return WBEM_OK;
}

int solve_mixed(wbem_context* h, const double* d_rhs, double* d_x, int transpose) {
  return gmres_mixed_driver(h, d_rhs, d_x, transpose);
}

// ------------------------------------------------------ standalone GEMM test
// C (M x Nc, ld Nc) -= A (M x K) B^T (Nc x K) for FP32 A, B given row-major
// on the device, split to BF16 hi/lo inside. Used by the kernel tests.
__global__ void k_split_rows(int rows, int K, const float* __restrict__ X, uint16_t* __restrict__ hi,
                             uint16_t* __restrict__ lo) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < (size_t)rows * K) split_bf16(X[i], &hi[i], &lo[i]);
}

}  // namespace wbem

extern "C" int wbem_test_gemm_bf16x3(int M, int Nc, int K, const float* dA, const float* dB,
                                     float* dC) {
  using namespace wbem;
  if (M < 1 || Nc < 1 || K < G3K || K % G3K) return WBEM_ERR_ARG;
  const int rA = M + kSplitPad, rB = Nc + kSplitPad;
  uint16_t* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(uint16_t) * 2 * ((size_t)rA + rB) * K) != cudaSuccess) return WBEM_ERR_NOMEM;
  cudaMemset(buf, 0, sizeof(uint16_t) * 2 * ((size_t)rA + rB) * K);
  uint16_t* Ahi = buf;
  uint16_t* Alo = Ahi + (size_t)rA * K;
  uint16_t* Bhi = Alo + (size_t)rA * K;
  uint16_t* Blo = Bhi + (size_t)rB * K;
  k_split_rows<<<(unsigned)(((size_t)M * K + 255) / 256), 256>>>(M, K, dA, Ahi, Alo);
  k_split_rows<<<(unsigned)(((size_t)Nc * K + 255) / 256), 256>>>(Nc, K, dB, Bhi, Blo);
  GemmMaps mp;
  int st = WBEM_OK;
  if (!encode_ops3(&mp, Ahi, Alo, rA, Bhi, Blo, rB, K)) st = WBEM_ERR_CUDA;
  // C through a padded copy (TMA needs 16-byte aligned row strides)
  const int ldc = (Nc + 31) / 32 * 32;
  float* Cp = nullptr;
  if (st == WBEM_OK && cudaMalloc(&Cp, sizeof(float) * (size_t)M * ldc) != cudaSuccess) st = WBEM_ERR_NOMEM;
  CUtensorMap cmap;
  if (st == WBEM_OK) {
    cudaMemcpy2D(Cp, sizeof(float) * ldc, dC, sizeof(float) * Nc, sizeof(float) * Nc, M,
                 cudaMemcpyDeviceToDevice);
    if (!encode_cmap(&cmap, Cp, M, Nc, ldc)) st = WBEM_ERR_CUDA;
  }
  DevErr* err = nullptr;
  if (st == WBEM_OK && cudaMalloc(&err, sizeof(DevErr)) != cudaSuccess) st = WBEM_ERR_NOMEM;
  if (st == WBEM_OK) {
    cudaMemset(err, 0, sizeof(DevErr));
    if (run_gemm<false>(mp, cmap, 0, 0, 0, 0, 0, M, Nc, K, err, 0) != cudaSuccess) st = WBEM_ERR_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) st = WBEM_ERR_CUDA;
    DevErr de{};
    cudaMemcpy(&de, err, sizeof de, cudaMemcpyDeviceToHost);
    if (st == WBEM_OK && de.code) st = de.code;
    if (st == WBEM_OK)
      cudaMemcpy2D(dC, sizeof(float) * Nc, Cp, sizeof(float) * ldc, sizeof(float) * Nc, M,
                   cudaMemcpyDeviceToDevice);
  }
  if (err) cudaFree(err);
  if (Cp) cudaFree(Cp);
  cudaFree(buf);
  return st;
}

// C (M x Nc, ld Nc) -= A (M x K) B^T (Nc x K), FP32 A and B row-major on the
// device, one TF32 tensor-core product (the factorisation's trailing update).
extern "C" int wbem_test_gemm_tf32(int M, int Nc, int K, const float* dA, const float* dB, float* dC) {
  using namespace wbem;
  if (M < 1 || Nc < 1 || K < G3K || K % G3K) return WBEM_ERR_ARG;
  GemmMaps mp;
  int st = WBEM_OK;
  if (!encode_cmap(&mp.Ahi, dA, M, K, K, G3M) || !encode_cmap(&mp.Bhi, dB, Nc, K, K, G3N))
    st = WBEM_ERR_CUDA;
  mp.Alo = mp.Ahi;
  mp.Blo = mp.Bhi;
  const int ldc = (Nc + 31) / 32 * 32;
  float* Cp = nullptr;
  if (st == WBEM_OK && cudaMalloc(&Cp, sizeof(float) * (size_t)M * ldc) != cudaSuccess) st = WBEM_ERR_NOMEM;
  CUtensorMap cmap;
  if (st == WBEM_OK) {
    cudaMemcpy2D(Cp, sizeof(float) * ldc, dC, sizeof(float) * Nc, sizeof(float) * Nc, M,
                 cudaMemcpyDeviceToDevice);
    if (!encode_cmap(&cmap, Cp, M, Nc, ldc)) st = WBEM_ERR_CUDA;
  }
  DevErr* err = nullptr;
  if (st == WBEM_OK && cudaMalloc(&err, sizeof(DevErr)) != cudaSuccess) st = WBEM_ERR_NOMEM;
  if (st == WBEM_OK) {
    cudaMemset(err, 0, sizeof(DevErr));
    if (run_gemm<true>(mp, cmap, 0, 0, 0, 0, 0, M, Nc, K, err, 0) != cudaSuccess) st = WBEM_ERR_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) st = WBEM_ERR_CUDA;
    DevErr de{};
    cudaMemcpy(&de, err, sizeof de, cudaMemcpyDeviceToHost);
    if (st == WBEM_OK && de.code) st = de.code;
    if (st == WBEM_OK)
      cudaMemcpy2D(dC, sizeof(float) * Nc, Cp, sizeof(float) * ldc, sizeof(float) * Nc, M,
                   cudaMemcpyDeviceToDevice);
  }
  if (err) cudaFree(err);
  if (Cp) cudaFree(Cp);
  return st;
}

extern "C" int wbem_test_lu_factors(wbem_context* h, float* A_host, float* LU_host,
                                    int* perm_host) {
  using namespace wbem;
  if (!h) return WBEM_ERR_ARG;
  if (h->assembled_prec != WBEM_PREC_MIXED)
    return fail(h, WBEM_ERR_STATE, "wbem_test_lu_factors: assemble in mixed precision first");
  if (!h->have_mask) return fail(h, WBEM_ERR_STATE, "wbem_test_lu_factors: set the boundary conditions first");
  if (cudaSetDevice(h->device) != cudaSuccess)
    return fail(h, WBEM_ERR_CUDA, "wbem_test_lu_factors: cannot select the handle's device");
  const int N = h->N;
  const size_t ld = (size_t)system_ld(N);
  WB_CHK(build_constraint_structure(h));
  if (A_host) {
    WB_CHK(form_system_f32(h));
    WB_CU(cudaMemcpy2DAsync(A_host, sizeof(float) * N, h->d_lu, sizeof(float) * ld,
                            sizeof(float) * N, N, cudaMemcpyDeviceToHost, h->stream));
    WB_CU(cudaStreamSynchronize(h->stream));
  }
  WB_CHK(factor_mixed(h));
  h->factors_valid = true;
  h->factors_kind = WBEM_SOLVER_LU;
  if (LU_host) {
    WB_CU(cudaMemcpy2DAsync(LU_host, sizeof(float) * N, h->d_lu, sizeof(float) * ld,
                            sizeof(float) * N, N, cudaMemcpyDeviceToHost, h->stream));
    WB_CU(cudaStreamSynchronize(h->stream));
  }
  if (perm_host)
    for (int k = 0; k < N; ++k) perm_host[k] = h->perm[k];
  return WBEM_OK;
}

extern "C" int wbem_test_lu_apply(wbem_context* h, const double* v, double* z, int transpose) {
  using namespace wbem;
  if (!h || !v || !z) return WBEM_ERR_ARG;
  if (!h->factors_valid || h->factors_kind != WBEM_SOLVER_LU || !h->lu_state)
    return fail(h, WBEM_ERR_STATE, "wbem_test_lu_apply: no LU factors");
  if (cudaSetDevice(h->device) != cudaSuccess)
    return fail(h, WBEM_ERR_CUDA, "wbem_test_lu_apply: cannot select the handle's device");
  const int N = h->N;
  double* dv = nullptr;
  WB_CU(cudaMalloc(&dv, sizeof(double) * 2 * N));
  double* dz = dv + N;
  int st = WBEM_OK;
  if (cudaMemcpyAsync(dv, v, sizeof(double) * N, cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
    st = WBEM_ERR_CUDA;
  if (st == WBEM_OK) st = lu_apply(h, dv, dz, transpose);
  if (st == WBEM_OK &&
      cudaMemcpyAsync(z, dz, sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
    st = WBEM_ERR_CUDA;
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) st = WBEM_ERR_CUDA;
  cudaFree(dv);
  if (st == WBEM_OK) st = check_device_error(h, "wbem_test_lu_apply");
  return st;
}
