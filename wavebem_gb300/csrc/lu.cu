// FP32 blocked LU (no pivoting) of the collocation system with BF16x3
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
// Step k (block size kNB = 128):
//   1. k_diag_block: LU of A_kk in shared memory, plus the inverses of its
//      unit-lower and upper factors;
//   2. k_panel_gemm: U_kj = inv(L_kk) A_kj and L_ik = A_ik inv(U_kk) (FP32 SIMT),
//      also writing the BF16 hi/lo splits of both panels (K-major);
//   3. k_gemm_bf16x3: A_ij -= L_ik U_kj as Lhi Uhi + Lhi Ulo + Llo Uhi with
//      FP32 accumulation in TMEM (128 x 256 tile per CTA, K = 128 in two
//      64-wide TMA stages with 128B swizzle).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <vector>
#include "context.h"
#include "host_util.h"
#include "kernels.h"

namespace wbem {

constexpr int kNB = 128;  // LU block size (= GEMM K)

// ------------------------------------------------------------------ input
// LU input: hi part of the system operator, alpha on Neumann diagonals,
// constrained rows replaced by e_i - sum_j c_ij e_j.
__global__ void k_form_lu(int N, const float2* __restrict__ N2, const float2* __restrict__ D2,
                          const uint8_t* __restrict__ mask, const double* __restrict__ alpha,
                          const uint8_t* __restrict__ cflag, const int* __restrict__ cptr,
                          const int* __restrict__ ccol, const double* __restrict__ cval,
                          float* __restrict__ A) {
  const int i = blockIdx.y;
  float* ar = A + (size_t)i * N;
  if (cflag[i]) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x)
      ar[j] = (j == i) ? 1.f : 0.f;
    return;
  }
  const float2* nr = N2 + (size_t)i * N;
  const float2* dr = D2 + (size_t)i * N;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x) {
    float v;
    if (mask[j]) {
      const float2 d = dr[j];
      v = -(float)((double)d.x + (double)d.y);
    } else {
      const float2 n = nr[j];
      double s = (double)n.x + (double)n.y;
      if (j == i) s += alpha[i];
      v = (float)s;
    }
    ar[j] = v;
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
// LU (no pivoting) of the kNB x kNB block at (k0, k0) in shared memory;
// writes the factors back and inv(L) (unit lower), inv(U) to linv/uinv
// (row-major kNB x kNB).
__global__ void __launch_bounds__(kNB)
    k_diag_block(int N, int k0, int nb, float* __restrict__ A, float* __restrict__ linv,
                 float* __restrict__ uinv, DevErr* err) {
  extern __shared__ __align__(16) float sA[];  // [kNB][kNB+1]
  constexpr int LD = kNB + 1;
  const int r = threadIdx.x;
  for (int c = 0; c < kNB; ++c)
    sA[r * LD + c] = (r < nb && c < nb) ? A[(size_t)(k0 + r) * N + k0 + c] : (r == c ? 1.f : 0.f);
  __syncthreads();
  __shared__ int bad;
  if (r == 0) bad = 0;
  __syncthreads();
  for (int k = 0; k < kNB; ++k) {
    const float piv = sA[k * LD + k];
    if (r == 0 && (!(fabsf(piv) > 0.f) || !isfinite(piv))) bad = 1;
    __syncthreads();
    if (bad) break;
    if (r > k) {
      const float l = sA[r * LD + k] / piv;
      sA[r * LD + k] = l;
      for (int c = k + 1; c < kNB; ++c) sA[r * LD + c] = __fmaf_rn(-l, sA[k * LD + c], sA[r * LD + c]);
    }
    __syncthreads();
  }
  if (bad) {
    if (r == 0) dev_fail(err, WBEM_ERR_SINGULAR, 51, k0, 0);
    return;
  }
  if (r < nb)
    for (int c = 0; c < nb; ++c) A[(size_t)(k0 + r) * N + k0 + c] = sA[r * LD + c];
  // column r of inv(L): solve L x = e_r (forward); column r of inv(U): U y = e_r (backward)
  float* Li = linv;
  float* Ui = uinv;
  for (int i = 0; i < kNB; ++i) {
    float s = (i == r) ? 1.f : 0.f;
    for (int j = r; j < i; ++j) s = __fmaf_rn(-sA[i * LD + j], Li[j * kNB + r], s);
    Li[i * kNB + r] = (i < r) ? 0.f : s;
  }
  for (int i = kNB - 1; i >= 0; --i) {
    float s = (i == r) ? 1.f : 0.f;
    if (i <= r) {
      for (int j = i + 1; j <= r; ++j) s = __fmaf_rn(-sA[i * LD + j], Ui[j * kNB + r], s);
      s /= sA[i * LD + i];
    }
    Ui[i * kNB + r] = (i > r) ? 0.f : s;
  }
}

// ------------------------------------------------------------- panel GEMM
// out = Left (rows x 128) * Right (128 x cols), FP32 SIMT, 64 x 64 tiles,
// 256 threads (4 x 4 outputs each).
//   mode 0 (row panel):  Left = inv(L_kk), Right = A[k0:k0+128, c0:], out -> A same place,
//                        BF16 splits of out^T -> Uhi/Ulo[(c - c0)][k] (K-major)
//   mode 1 (col panel):  Left = A[r0:, k0:k0+128], Right = inv(U_kk), out -> A same place,
//                        BF16 splits -> Lhi/Llo[(r - r0)][k]
__device__ __forceinline__ void split_bf16(float v, uint16_t* hi, uint16_t* lo) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
  *hi = __bfloat16_as_ushort(h);
  *lo = __bfloat16_as_ushort(l);
}

__global__ void __launch_bounds__(256)
    k_panel_gemm(int N, int mode, int k0, int nrows, int ncols, float* __restrict__ A,
                 const float* __restrict__ inv, uint16_t* __restrict__ Shi,
                 uint16_t* __restrict__ Slo) {
  __shared__ float sL[64][33];
  __shared__ float sR[32][65];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int r0 = blockIdx.y * 64, c0 = blockIdx.x * 64;
  const int k1 = k0 + kNB;
  float acc[4][4] = {};
  for (int kk = 0; kk < kNB; kk += 32) {
    for (int t = threadIdx.x; t < 64 * 32; t += 256) {
      const int rr = t / 32, cc = t % 32;
      float v = 0.f;
      if (mode == 0) {
        v = (r0 + rr < kNB) ? inv[(r0 + rr) * kNB + kk + cc] : 0.f;
      } else if (r0 + rr < nrows) {
        v = A[(size_t)(k1 + r0 + rr) * N + k0 + kk + cc];
      }
      sL[rr][cc] = v;
    }
    for (int t = threadIdx.x; t < 32 * 64; t += 256) {
      const int rr = t / 64, cc = t % 64;
      float v = 0.f;
      if (mode == 0) {
        if (c0 + cc < ncols) v = A[(size_t)(k0 + kk + rr) * N + k1 + c0 + cc];
      } else if (c0 + cc < kNB) {
        v = inv[(kk + rr) * kNB + c0 + cc];
      }
      sR[rr][cc] = v;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
      float a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = sL[ty * 4 + u][k];
        b[u] = sR[k][tx * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = __fmaf_rn(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int rr = r0 + ty * 4 + u, cc = c0 + tx * 4 + v;
      if (mode == 0) {
        if (rr < kNB && cc < ncols) {
          A[(size_t)(k0 + rr) * N + k1 + cc] = acc[u][v];
          split_bf16(acc[u][v], &Shi[(size_t)cc * kNB + rr], &Slo[(size_t)cc * kNB + rr]);
        }
      } else {
        if (rr < nrows && cc < kNB) {
          A[(size_t)(k1 + rr) * N + k0 + cc] = acc[u][v];
          split_bf16(acc[u][v], &Shi[(size_t)rr * kNB + cc], &Slo[(size_t)rr * kNB + cc]);
        }
      }
    }
}

// ------------------------------------------------------- tcgen05 BF16x3 GEMM
constexpr int GM = 128, GN = 256, GK = 64;
constexpr uint32_t kStageBytes = (GM + GM + GN + GN) * GK * 2;  // Ahi Alo Bhi Blo: 96 KB

__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  // K-major operand tile, 128-byte swizzle: rows of 128 B, 8-row atoms of
  // 1024 B (stride byte offset), descriptor version 1 (tcgen05)
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

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

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__global__ void __launch_bounds__(128, 1)
    k_gemm_bf16x3(const __grid_constant__ CUtensorMap mAhi, const __grid_constant__ CUtensorMap mAlo,
                  const __grid_constant__ CUtensorMap mBhi, const __grid_constant__ CUtensorMap mBlo,
                  int M, int Nc, int K, float* __restrict__ Cm, int ldc, DevErr* err) {
  extern __shared__ __align__(1024) uint8_t gsm[];
  // 1024-byte aligned operand stages
  const uint32_t base_s = smem_u32(gsm);
  const uint32_t pad = (1024 - (base_s & 1023)) & 1023;
  uint8_t* sm = gsm + pad;
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + 2 * kStageBytes);
  uint64_t* empty = full + 2;
  uint64_t* done = full + 4;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(full + 5);
  int* fail_flag = reinterpret_cast<int*>(full + 6);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * GM, n0 = blockIdx.y * GN;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(256)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    mbar_init(&empty[0], 1);
    mbar_init(&empty[1], 1);
    mbar_init(done, 1);
    *fail_flag = 0;
    fence_mbar_init();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const int nk = K / GK;
  // instruction descriptor: D f32, A/B bf16, K-major both, N = 256, M = 128
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(GN >> 3) << 17) |
                         ((uint32_t)(GM >> 4) << 24);

  if (tid == 0) {
    auto stage_ptr = [&](int s) { return smem_u32(sm + (size_t)s * kStageBytes); };
    auto load = [&](int c) {
      const int s = c & 1;
      const uint32_t st = stage_ptr(s);
      mbar_arrive_expect_tx(&full[s], kStageBytes);
      tma_load_2d(st, &mAhi, c * GK, m0, &full[s]);
      tma_load_2d(st + GM * GK * 2, &mAlo, c * GK, m0, &full[s]);
      tma_load_2d(st + 2 * GM * GK * 2, &mBhi, c * GK, n0, &full[s]);
      tma_load_2d(st + 2 * GM * GK * 2 + GN * GK * 2, &mBlo, c * GK, n0, &full[s]);
    };
    bool ok = true;
    load(0);
    if (nk > 1) load(1);
    for (int c = 0; c < nk && ok; ++c) {
      const int s = c & 1;
      if (!mbar_wait_bounded(&full[s], (uint32_t)((c >> 1) & 1))) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t st = stage_ptr(s);
      const uint64_t dAh = smem_desc_sw128(st);
      const uint64_t dAl = smem_desc_sw128(st + GM * GK * 2);
      const uint64_t dBh = smem_desc_sw128(st + 2 * GM * GK * 2);
      const uint64_t dBl = smem_desc_sw128(st + 2 * GM * GK * 2 + GN * GK * 2);
#pragma unroll
      for (int kk = 0; kk < GK / 16; ++kk) {
        const uint64_t adv = (uint64_t)(kk * 2);  // 32 bytes along K, in 16-byte units
        umma_bf16(tmem, dAh + adv, dBh + adv, idesc, (c > 0 || kk > 0) ? 1u : 0u);
        umma_bf16(tmem, dAh + adv, dBl + adv, idesc, 1u);
        umma_bf16(tmem, dAl + adv, dBh + adv, idesc, 1u);
      }
      umma_commit(&empty[s]);
      if (c + 2 < nk) {
        if (!mbar_wait_bounded(&empty[s], (uint32_t)((c >> 1) & 1))) {
          ok = false;
          break;
        }
        load(c + 2);
      }
    }
    if (!ok) {
      *fail_flag = 1;
      dev_fail(err, WBEM_ERR_TIMEOUT, 61, blockIdx.x, blockIdx.y);
    }
    umma_commit(done);  // arrives once all issued MMAs have completed
  }
  __syncwarp();
  const bool ok_done = mbar_wait_bounded(done, 0u);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (ok_done && *fail_flag == 0) {
    const int row = m0 + warp * 32 + lane;
    float* crow = Cm + (size_t)row * ldc;
    for (int cc = 0; cc < GN; cc += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
          "%12, %13, %14, %15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
            "=r"(v[14]), "=r"(v[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < M) {
        const int col = n0 + cc;
        if (col + 16 <= Nc && ((ldc & 3) == 0)) {
          float4* p = reinterpret_cast<float4*>(crow + col);
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            float4 o = p[u];
            o.x -= __uint_as_float(v[4 * u + 0]);
            o.y -= __uint_as_float(v[4 * u + 1]);
            o.z -= __uint_as_float(v[4 * u + 2]);
            o.w -= __uint_as_float(v[4 * u + 3]);
            p[u] = o;
          }
        } else {
#pragma unroll
          for (int t = 0; t < 16; ++t)
            if (col + t < Nc) crow[col + t] -= __uint_as_float(v[t]);
        }
      }
    }
  } else if (!ok_done && tid == 0) {
    dev_fail(err, WBEM_ERR_TIMEOUT, 62, blockIdx.x, blockIdx.y);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256)
                 : "memory");
}

static size_t gemm_smem() { return 2 * (size_t)kStageBytes + 1024 + 64; }

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

static bool encode_map(CUtensorMap* map, const uint16_t* base, int rows, int kdim, int box_rows) {
  const cuuint64_t dims[2] = {(cuuint64_t)kdim, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kdim * 2};
  const cuuint32_t box[2] = {(cuuint32_t)GK, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return false;
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)base, dims,
                                      strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                      CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

struct GemmMaps {
  CUtensorMap Ahi, Alo, Bhi, Blo;
};

// C[M x Nc] (ldc) -= A B^T with A rows in (Ahi, Alo) [rowsA x K], B rows in
// (Bhi, Blo) [rowsB x K], both K-major BF16.
static cudaError_t run_gemm(const GemmMaps& mp, int M, int Nc, int K, float* Cm, int ldc,
                            DevErr* err, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_gemm_bf16x3, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)gemm_smem());
    if (e != cudaSuccess) return e;
    attr = true;
  }
  dim3 grid((M + GM - 1) / GM, (Nc + GN - 1) / GN);
  k_gemm_bf16x3<<<grid, 128, gemm_smem(), s>>>(mp.Ahi, mp.Alo, mp.Bhi, mp.Blo, M, Nc, K, Cm, ldc,
                                               err);
  return cudaGetLastError();
}

// ------------------------------------------------------------ triangular solves
// Blocked FP32 forward / backward substitution with the stored diagonal-block
// inverses. Work vector w (float, N). Forward (L, unit lower):
//   y_k = inv(L_kk) w_k ;  w_i -= L_ik y_k (i > k).
// Backward (U): x_k = inv(U_kk) w_k ; w_i -= U_ik x_k (i < k).
// Transposed solves (A^T = U^T L^T) use the row blocks instead of the column
// blocks: forward with U^T, backward with L^T.
__global__ void k_tri_diag(int N, int k0, int nb, const float* __restrict__ inv, int transpose,
                           float* __restrict__ w) {
  __shared__ float xs[kNB];
  const int r = threadIdx.x;
  xs[r] = (r < nb) ? w[k0 + r] : 0.f;
  __syncthreads();
  float s = 0.f;
  if (!transpose)
    for (int c = 0; c < kNB; ++c) s = __fmaf_rn(inv[r * kNB + c], xs[c], s);
  else
    for (int c = 0; c < kNB; ++c) s = __fmaf_rn(inv[c * kNB + r], xs[c], s);
  if (r < nb) w[k0 + r] = s;
}

// w[rows] -= M[rows, k0:k0+nb] x  (column-block update; ld = N), or for the
// transposed sweep w[cols] -= M[k0:k0+nb, cols]^T x (row-block update).
__global__ void k_tri_update(int N, int k0, int nb, int lo, int hi, const float* __restrict__ LU,
                             int rowblock, float* __restrict__ w) {
  __shared__ float xs[kNB];
  if (threadIdx.x < kNB) xs[threadIdx.x] = (threadIdx.x < nb) ? w[k0 + threadIdx.x] : 0.f;
  __syncthreads();
  if (!rowblock) {
    // one warp per row
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int i = lo + warp;
    if (i >= hi) return;
    const float* r = LU + (size_t)i * N + k0;
    float s = 0.f;
    for (int c = lane; c < nb; c += 32) s = __fmaf_rn(r[c], xs[c], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) w[i] -= s;
  } else {
    const int j = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= hi) return;
    float s = 0.f;
    for (int c = 0; c < nb; ++c) s = __fmaf_rn(LU[(size_t)(k0 + c) * N + j], xs[c], s);
    w[j] -= s;
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
  float* linv = nullptr;  // per block kNB x kNB
  float* uinv = nullptr;
  uint16_t* split = nullptr;  // Lhi, Llo, Uhi, Ulo: each N x kNB
  float* w = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // forward+backward, transposed
  int N = 0;
  GemmMaps maps;
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
  if (L.split) cudaFree(L.split);
  if (L.w) cudaFree(L.w);
  for (auto& g : L.graph)
    if (g) cudaGraphExecDestroy(g);
  delete &L;
  h->lu_state = nullptr;
}

static int enqueue_tri_solve(wbem_context* h, LuState& L, int transpose) {
  const int N = h->N;
  const int nblk = (N + kNB - 1) / kNB;
  const float* LU = h->d_lu;
  if (!transpose) {
    // L y = w (forward): diag with inv(L_kk), update rows below from column block k
    for (int k = 0; k < nblk; ++k) {
      const int k0 = k * kNB, nb = std::min(kNB, N - k0);
      k_tri_diag<<<1, kNB, 0, h->stream>>>(N, k0, nb, L.linv + (size_t)k * kNB * kNB, 0, L.w);
      const int lo = k0 + nb, hi = N;
      if (hi > lo) k_tri_update<<<(hi - lo + 7) / 8, 256, 0, h->stream>>>(N, k0, nb, lo, hi, LU, 0, L.w);
    }
    for (int k = nblk - 1; k >= 0; --k) {
      const int k0 = k * kNB, nb = std::min(kNB, N - k0);
      k_tri_diag<<<1, kNB, 0, h->stream>>>(N, k0, nb, L.uinv + (size_t)k * kNB * kNB, 0, L.w);
      if (k0 > 0) k_tri_update<<<(k0 + 7) / 8, 256, 0, h->stream>>>(N, k0, nb, 0, k0, LU, 0, L.w);
    }
  } else {
    // U^T y = w (forward): diag with inv(U_kk)^T, update columns right of k from row block k of U
    for (int k = 0; k < nblk; ++k) {
      const int k0 = k * kNB, nb = std::min(kNB, N - k0);
      k_tri_diag<<<1, kNB, 0, h->stream>>>(N, k0, nb, L.uinv + (size_t)k * kNB * kNB, 1, L.w);
      const int lo = k0 + nb, hi = N;
      if (hi > lo) k_tri_update<<<(hi - lo + 255) / 256, 256, 0, h->stream>>>(N, k0, nb, lo, hi, LU, 1, L.w);
    }
    // L^T x = y (backward): diag with inv(L_kk)^T, update columns left of k from row block k of L
    for (int k = nblk - 1; k >= 0; --k) {
      const int k0 = k * kNB, nb = std::min(kNB, N - k0);
      k_tri_diag<<<1, kNB, 0, h->stream>>>(N, k0, nb, L.linv + (size_t)k * kNB * kNB, 1, L.w);
      if (k0 > 0) k_tri_update<<<(k0 + 255) / 256, 256, 0, h->stream>>>(N, k0, nb, 0, k0, LU, 1, L.w);
    }
  }
  return cudaGetLastError() == cudaSuccess ? WBEM_OK : fail(h, WBEM_ERR_CUDA, "triangular solve launch");
}

int factor_mixed(wbem_context* h) {
  const int N = h->N;
  const size_t nn = (size_t)N * N;
  if (h->lu_state && lu_state(h).N != N) free_lu(h);
  LuState& L = lu_state(h);
  L.N = N;
  if (!h->d_lu || h->lu_elems != nn) {
    WB_CHK(dev_alloc(h, &h->d_lu, nn));
    h->lu_elems = nn;
  }
  const int nblk = (N + kNB - 1) / kNB;
  if (!L.linv) {
    WB_CHK(dev_alloc(h, &L.linv, (size_t)nblk * kNB * kNB));
    WB_CHK(dev_alloc(h, &L.uinv, (size_t)nblk * kNB * kNB));
    WB_CHK(dev_alloc(h, &L.split, (size_t)4 * ((size_t)N + GN) * kNB));
    WB_CHK(dev_alloc(h, &L.w, (size_t)N));
    WB_CU(cudaMemset(L.split, 0, sizeof(uint16_t) * 4 * ((size_t)N + GN) * kNB));
    uint16_t* Lhi = L.split;
    uint16_t* Llo = Lhi + ((size_t)N + GN) * kNB;
    uint16_t* Uhi = Llo + ((size_t)N + GN) * kNB;
    uint16_t* Ulo = Uhi + ((size_t)N + GN) * kNB;
    const int rows = N + GN;
    if (!encode_map(&L.maps.Ahi, Lhi, rows, kNB, GM) || !encode_map(&L.maps.Alo, Llo, rows, kNB, GM) ||
        !encode_map(&L.maps.Bhi, Uhi, rows, kNB, GN) || !encode_map(&L.maps.Blo, Ulo, rows, kNB, GN))
      return fail(h, WBEM_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  }
  uint16_t* Lhi = L.split;
  uint16_t* Llo = Lhi + ((size_t)N + GN) * kNB;
  uint16_t* Uhi = Llo + ((size_t)N + GN) * kNB;
  uint16_t* Ulo = Uhi + ((size_t)N + GN) * kNB;
  EvTimer tm(h->stream);
  {
    dim3 g(std::min(64, (N + 255) / 256), N);
    k_form_lu<<<g, 256, 0, h->stream>>>(N, h->d_N2, h->d_D2, h->d_mask, h->d_alpha, h->d_cflag,
                                        h->d_cptr_full, h->d_ccol_full, h->d_cval_full, h->d_lu);
    WB_CU(cudaGetLastError());
    if (h->n_crows > 0) {
      k_lu_constraint_entries<<<(h->n_crows + 127) / 128, 128, 0, h->stream>>>(
          h->n_crows, h->d_crow, h->d_cptr, h->d_ccol, h->d_cval, N, h->d_lu);
      WB_CU(cudaGetLastError());
    }
  }
  h->stats.t_system_ms = tm.ms();
  const size_t dsm = (size_t)kNB * (kNB + 1) * sizeof(float);
  WB_CU(cudaFuncSetAttribute(k_diag_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm));
  for (int k = 0; k < nblk; ++k) {
    const int k0 = k * kNB, nb = std::min(kNB, N - k0);
    const int k1 = k0 + nb, m = N - k1;
    k_diag_block<<<1, kNB, dsm, h->stream>>>(N, k0, nb, h->d_lu, L.linv + (size_t)k * kNB * kNB,
                                             L.uinv + (size_t)k * kNB * kNB, h->d_err);
    h->launches++;
    if (m <= 0) break;
    // row panel U_kj (128 x m) and column panel L_ik (m x 128)
    dim3 gr((m + 63) / 64, (kNB + 63) / 64);
    k_panel_gemm<<<gr, 256, 0, h->stream>>>(N, 0, k0, kNB, m, h->d_lu,
                                            L.linv + (size_t)k * kNB * kNB, Uhi, Ulo);
    dim3 gc((kNB + 63) / 64, (m + 63) / 64);
    k_panel_gemm<<<gc, 256, 0, h->stream>>>(N, 1, k0, m, kNB, h->d_lu,
                                            L.uinv + (size_t)k * kNB * kNB, Lhi, Llo);
    WB_CU(cudaGetLastError());
    WB_CU(run_gemm(L.maps, m, m, kNB, h->d_lu + (size_t)k1 * N + k1, N, h->d_err, h->stream));
    h->launches += 3;
  }
  WB_CHK(check_device_error(h, "LU factorisation"));
  h->stats.t_factor_ms = tm.ms();
  // capture the triangular sweeps as CUDA graphs (fixed launch sequence)
  for (int t = 0; t < 2; ++t) {
    if (L.graph[t]) {
      cudaGraphExecDestroy(L.graph[t]);
      L.graph[t] = nullptr;
    }
    cudaGraph_t g;
    WB_CU(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int st = enqueue_tri_solve(h, L, t);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (st != WBEM_OK) return st;
    WB_CU(e);
    WB_CU(cudaGraphInstantiate(&L.graph[t], g, 0));
    cudaGraphDestroy(g);
  }
  return WBEM_OK;
}

// z = M^{-1} v with M = L U (FP32 factors), FP64 in/out.
int lu_apply(wbem_context* h, const double* v, double* z, int transpose) {
  LuState& L = lu_state(h);
  const int N = h->N;
  k_to_float<<<(N + 255) / 256, 256, 0, h->stream>>>(N, v, L.w);
  WB_CU(cudaGetLastError());
  WB_CU(cudaGraphLaunch(L.graph[transpose ? 1 : 0], h->stream));
  k_to_double<<<(N + 255) / 256, 256, 0, h->stream>>>(N, L.w, z);
  WB_CU(cudaGetLastError());
  h->launches += 2 + 4 * ((N + kNB - 1) / kNB);
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
  if (M < 1 || Nc < 1 || K < GK || K % GK) return WBEM_ERR_ARG;
  const int rA = M + GM, rB = Nc + GN;
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
  if (!encode_map(&mp.Ahi, Ahi, rA, K, GM) || !encode_map(&mp.Alo, Alo, rA, K, GM) ||
      !encode_map(&mp.Bhi, Bhi, rB, K, GN) || !encode_map(&mp.Blo, Blo, rB, K, GN))
    st = WBEM_ERR_CUDA;
  DevErr* err = nullptr;
  if (st == WBEM_OK && cudaMalloc(&err, sizeof(DevErr)) != cudaSuccess) st = WBEM_ERR_NOMEM;
  if (st == WBEM_OK) {
    cudaMemset(err, 0, sizeof(DevErr));
    if (run_gemm(mp, M, Nc, K, dC, Nc, err, 0) != cudaSuccess) st = WBEM_ERR_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) st = WBEM_ERR_CUDA;
    DevErr de{};
    cudaMemcpy(&de, err, sizeof de, cudaMemcpyDeviceToHost);
    if (st == WBEM_OK && de.code) st = de.code;
  }
  if (err) cudaFree(err);
  cudaFree(buf);
  return st;
}
