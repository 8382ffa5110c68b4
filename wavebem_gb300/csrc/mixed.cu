// Mixed-precision form (placeholder until the kernels land).
#include <cuda_runtime.h>
#include "context.h"

namespace wbem {
static __constant__ QuadTables c_qm;
cudaError_t upload_quadrature_mixed(const QuadTables& t) {
  return cudaMemcpyToSymbol(c_qm, &t, sizeof(QuadTables));
}
int assemble_mixed(wbem_context* h) {
  h->err = "mixed precision form not available";
  return WBEM_ERR_ARG;
}
int factor_mixed(wbem_context* h) {
  h->err = "mixed precision form not available";
  return WBEM_ERR_ARG;
}
int solve_mixed(wbem_context* h, const double*, double*, int) {
  h->err = "mixed precision form not available";
  return WBEM_ERR_ARG;
}
void free_mixed(wbem_context*) {}
}  // namespace wbem
