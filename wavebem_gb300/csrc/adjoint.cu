// Hull force evaluation and the adjoint of assemble + solve + force.
#include <cuda_runtime.h>
#include <vector>
#include "context.h"

namespace wbem {
cudaError_t upload_quadrature_force(const QuadTables& t);
static __constant__ QuadTables c_qa;
cudaError_t upload_quadrature_adjoint(const QuadTables& t) {
  cudaError_t e = cudaMemcpyToSymbol(c_qa, &t, sizeof(QuadTables));
  if (e != cudaSuccess) return e;
  return upload_quadrature_force(t);
}
int ensure_vectors(wbem_context* h, int restart);

static int hull_dofs_upload(wbem_context* h, const int* hull_cells, int n_hull, int4** out) {
  std::vector<int4> hd(n_hull > 0 ? n_hull : 1);
  for (int k = 0; k < n_hull; ++k) {
    const int c = hull_cells[k];
    if (c < 0 || c >= h->C) {
      h->err = "hull cell index out of range";
      return WBEM_ERR_ARG;
    }
    const int* v = &h->cells[4 * (size_t)c];
    hd[k] = make_int4(h->iperm[v[0]], h->iperm[v[1]], h->iperm[v[2]], h->iperm[v[3]]);
  }
  if (cudaMalloc(out, sizeof(int4) * hd.size()) != cudaSuccess) {
    h->err = "cudaMalloc failed";
    return WBEM_ERR_NOMEM;
  }
  cudaMemcpyAsync(*out, hd.data(), sizeof(int4) * hd.size(), cudaMemcpyHostToDevice, h->stream);
  cudaStreamSynchronize(h->stream);
  return WBEM_OK;
}

int hull_force_dev(wbem_context* h, const int* hull_cells, int n_hull, const double* U, int dir,
                   const double* d_phi, const double* d_dphi, double* force) {
  int4* hd = nullptr;
  int st = hull_dofs_upload(h, hull_cells, n_hull, &hd);
  if (st) return st;
  double* part = nullptr;
  if (cudaMalloc(&part, sizeof(double) * (n_hull + 1)) != cudaSuccess) {
    cudaFree(hd);
    h->err = "cudaMalloc failed";
    return WBEM_ERR_NOMEM;
  }
  cudaError_t e = launch_hull_force(n_hull, hd, h->d_X, U, dir, d_phi, d_dphi, part, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(force, part + n_hull, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(part);
  cudaFree(hd);
  if (e != cudaSuccess) {
    h->err = cudaGetErrorString(e);
    return WBEM_ERR_CUDA;
  }
  return WBEM_OK;
}

int adjoint_force(wbem_context* h, const int*, int, const double*, int, const double*, double*,
                  double*) {
  h->err = "adjoint not available";
  return WBEM_ERR_ARG;
}
}  // namespace wbem
