// Library handle: host-side topology, device buffers and solver state.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "../../include/wbem.h"
#include "kernels.h"

constexpr int kNumVec = 10;
constexpr int kAssembledFma = 2;  // assembled_prec of the FMA method

// Event-bracketed intervals of one kernel class on one stream (kernel
// profiling mode): begin/end around each launch, summed after the work.
struct ProfTimer {
  std::vector<cudaEvent_t> a, b;
  size_t used = 0;
  double work = 0.0;  // flops or bytes of the bracketed launches
  void reset() {
    used = 0;
    work = 0.0;
  }
  void begin(cudaStream_t s) {
    if (used == a.size()) {
      cudaEvent_t x, y;
      cudaEventCreate(&x);
      cudaEventCreate(&y);
      a.push_back(x);
      b.push_back(y);
    }
    cudaEventRecord(a[used], s);
  }
  void end(cudaStream_t s, double w) {
    cudaEventRecord(b[used], s);
    ++used;
    work += w;
  }
  double total_ms() {
    double t = 0.0;
    for (size_t i = 0; i < used; ++i) {
      float ms = 0.f;
      cudaEventSynchronize(b[i]);
      cudaEventElapsedTime(&ms, a[i], b[i]);
      t += ms;
    }
    return t;
  }
  ~ProfTimer() {
    for (cudaEvent_t e : a) cudaEventDestroy(e);
    for (cudaEvent_t e : b) cudaEventDestroy(e);
  }
};

struct wbem_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  wbem_stats stats{};
  wbem_options opt{};
  // the regular Gauss-Legendre line rule on [0,1] of the last quadrature
  // set-up (the tensor rule of the panels is its product)
  int gauss_n = 0;
  double gauss_x[8] = {}, gauss_w[8] = {};

  // ---- host topology (caller order)
  int N = 0, C = 0;
  std::vector<double> X;
  std::vector<int> cells;
  std::vector<int> dn_ptr, dn_idx;
  std::vector<unsigned char> mask;
  bool have_mask = false;
  // internal order: perm[internal] = caller dof, iperm[caller] = internal dof
  std::vector<int> perm, iperm;
  int n_tiles = 0;

  // ---- device topology / geometry (internal order)
  double* d_X = nullptr;        // N x 3
  int4* d_cell_dofs = nullptr;  // C
  int* d_dnset = nullptr;       // N x kMaxSet
  int* d_tile_ptr = nullptr;    // n_tiles + 1 (+ the tiles' first columns)
  int2* d_tile_ent = nullptr;
  int n_tiles64 = 0;            // FP64 column tiles: groups of consecutive patches
  int* d_tile_ptr64 = nullptr;
  int2* d_tile_ent64 = nullptr;
  int* d_sptr = nullptr;        // singular panels per row (CSR)
  int* d_scell = nullptr;
  int* d_perm = nullptr;        // internal -> caller
  int* d_iperm = nullptr;       // caller -> internal
  int* d_ncptr = nullptr;       // node -> (cell, local vertex) CSR, internal nodes
  int* d_ncent = nullptr;
  uint8_t* d_mask = nullptr;
  double* d_rec = nullptr;      // FP64 panel records
  float* d_rec32 = nullptr;     // mixed panel records
  double* d_cellc = nullptr;    // mixed: panel centre / normal / moments (double-float source)
  float* d_cellgeo = nullptr;   // mixed: centre (float), radius^2 for the near test
  size_t rec_cells = 0;

  // ---- matrices (internal order)
  double* d_N = nullptr;
  double* d_D = nullptr;
  // mixed form: (hi, lo) float pairs of the two operators, the boundary-
  // condition selection applied per column (so each mat-vec streams one
  // contiguous matrix): A2 = sel_j ? -D_ij : N_ij (system operator, vmult),
  // B2 = sel_j ? -N_ij : D_ij (right-hand side, compute_rhs)
  float2* d_A2 = nullptr;
  float2* d_B2 = nullptr;
  std::vector<uint8_t> sel_mask;  // internal order: the column mask A2 / B2 are selected for
  uint8_t* d_selmask = nullptr;
  int* d_flips = nullptr;         // columns to reselect after a mask change
  size_t flips_cap = 0;
  double* d_alpha = nullptr;
  double* d_alpha_part = nullptr;
  double* d_alpha_near = nullptr;
  double* d_alpha_sing = nullptr;
  // mixed assembly: near-field and singular contributions appended per row
  // (on aux_stream, beside the far-field kernel) and merged afterwards
  double2* d_item_val = nullptr;  // (dN, dD) per item
  int* d_item_dof = nullptr;
  int* d_item_cnt = nullptr;      // per row: near items, singular items
  size_t item_rows = 0;
  cudaStream_t aux_stream = nullptr;
  cudaEvent_t ev_aux_fork = nullptr, ev_aux_join = nullptr;
  // right-hand side computed on rhs_stream (lowest priority: it fills the
  // SMs the factorisation leaves idle) beside the factorisation; the Krylov
  // solve waits for ev_rhs when rhs_pending
  cudaStream_t rhs_stream = nullptr;
  cudaEvent_t ev_rhs = nullptr;
  bool rhs_pending = false;
  int* d_near_cnt = nullptr;
  int* d_near_cells = nullptr;
  int near_cap = 0;
  size_t mat_elems = 0;       // allocated N*N (fp64 or float2)
  int assembled_prec = -1;    // precision of the current assembly, -1 = none
  // kernel profiling mode: the factorisation runs on one stream and the
  // launches of each kernel class are bracketed by events
  bool profiling = false;
  ProfTimer prof_gemm, prof_diag, prof_panel, prof_matvec, prof_trsv;
  bool factors_valid = false;  // preconditioner of factors_kind ready for this assembly
  int factors_kind = 0;        // WBEM_SOLVER_* it was prepared for

  // ---- constraints (internal order)
  int n_crows = 0;
  int* d_crow = nullptr;
  int* d_cptr = nullptr;
  int* d_ccol = nullptr;
  double* d_cval = nullptr;
  double* d_cinh = nullptr;
  uint8_t* d_cflag = nullptr;
  int* d_cptr_full = nullptr;
  int* d_ccol_full = nullptr;
  double* d_cval_full = nullptr;
  int* d_tptr = nullptr;   // transposed constraint entries (by column)
  int* d_tsrc = nullptr;
  double* d_tval = nullptr;
  // host copy of the constraint structure last uploaded: a solve whose lines
  // and entries are unchanged uploads only the inhomogeneities
  std::vector<int> c_crow, c_cptr, c_ccol;
  std::vector<double> c_cval;

  // ---- solver workspaces
  double* d_binv = nullptr;
  double* d_V = nullptr;   // (restart + 1) x N Krylov basis
  int V_cap = 0;
  double* d_vec[kNumVec] = {};  // N-vectors: [0..2] GMRES, [7] transposed operator, [8..9] refinement
  double* d_part = nullptr;
  double* d_small = nullptr;
  float* d_lu = nullptr;   // mixed: FP32 system matrix, then its LU factors
  // state of d_lu: 0 = neither, 1 = system entries from the assembly (free
  // term and constraint rows pending), 2 = complete system matrix
  int s32_state = 0;
  uint16_t* d_split = nullptr;
  float* d_lutmp = nullptr;
  int* d_info = nullptr;
  size_t lu_elems = 0;
  // last solution (internal order), kept for the adjoint
  double* d_sol = nullptr;
  double* d_rhs = nullptr;
  double* d_b = nullptr;   // known data (internal order)
  bool have_solution = false;
  std::vector<double> sol_b;  // known data (tmp_rhs) of the last solve, caller order

  // FMA method (fma.cu): octree, near field and expansion buffers; rebuilt
  // when the nodes or the order change
  void* fma_state = nullptr;
  bool fma_geometry_stale = true;
  wbem::QuadTables quad{};  // the quadrature tables of the last set-up

  wbem::DevErr* d_err = nullptr;
  int launches = 0;
  void* lu_state = nullptr;  // mixed LU workspaces (lu.cu)
};
