// Hull force on device-resident fields, without any device allocation.
//
// wbem_hull_force allocates a small buffer for its per-panel partial sums on
// every call and frees it again. Freeing device memory synchronises the whole
// device, and allocating goes around whatever memory pool the caller runs
// with. A time-stepping caller that evaluates the force after every Newton
// iteration, on a stream of its own and with device memory handed out by
// another framework's caching allocator, cannot afford either. This variant
// takes device pointers only and keeps its partial sums in a fixed array in
// the library's own device memory, so it never calls the allocator.
#include <cuda_runtime.h>
#include <atomic>
#include <cmath>
#include <mutex>
#include <string>
#include "context.h"

namespace {

// Largest number of hull panels one call accepts: the per-panel partial
// sums live in a file-scope device array of this many doubles (512 KB). Every
// GPU that loads the library holds it until the process exits.
constexpr int kNoAllocMaxPanels = 65536;
constexpr int kMaxDevices = 64;

struct GaussLine {
  int n;
  double x[8];
  double w[8];
};

}  // namespace

// Partial sums of the last call (shared by every call on a device).
static __device__ __align__(256) double g_hull_partials[kNoAllocMaxPanels];

// Host-side copies of the device address of g_hull_partials, one per device.
// The name g_hull_partials in host code is only a stand-in for the device
// symbol, so the address is looked up once per device with that device
// current and passed to the kernels. The lookup is serialised by a mutex;
// later calls read the cached address without locking. A device reset
// (cudaDeviceReset) invalidates the cached addresses: reload the library
// after one.
static std::atomic<double*> s_partials[kMaxDevices];
static std::mutex s_partials_lock;

// Device address of g_hull_partials on the current device `dev`.
static cudaError_t partials_address(int dev, double** out) {
  double* p = s_partials[dev].load(std::memory_order_acquire);
  if (!p) {
    std::lock_guard<std::mutex> g(s_partials_lock);
    p = s_partials[dev].load(std::memory_order_relaxed);
    if (!p) {
      void* q = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&q, g_hull_partials);
      if (e != cudaSuccess) return e;
      if (!q) return cudaErrorInvalidSymbol;
      p = static_cast<double*>(q);
      s_partials[dev].store(p, std::memory_order_release);
    }
  }
  *out = p;
  return cudaSuccess;
}

// Makes `dev` current for the lifetime of the guard and gives the caller's
// current device back on every return path.
struct DeviceScope {
  int prev = -1;
  bool ok = false;
  explicit DeviceScope(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) return;
    ok = prev == dev || cudaSetDevice(dev) == cudaSuccess;
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// One thread per hull panel: F_panel = sum_q p n_dir JxW with
// p = -(U . grad phi + |grad phi|^2 / 2), grad phi = tangential gradient of
// the Q1 interpolant of phi + (interpolated dphi/dn) n. Panel indices and the
// fields are in the caller's numbering; an out-of-range panel gives NaN.
__global__ void k_hull_partials_noalloc(int nh, int C, const int* __restrict__ hull_cells,
                                        const int4* __restrict__ cell_dofs,
                                        const int* __restrict__ perm,
                                        const double* __restrict__ X, double U0, double U1,
                                        double U2, int dir, const double* __restrict__ phi,
                                        const double* __restrict__ dphi, GaussLine g,
                                        double* __restrict__ partials) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nh) return;
  const int cell = hull_cells[k];
  if (cell < 0 || cell >= C) {
    partials[k] = nan("");
    return;
  }
  const int4 d = cell_dofs[cell];
  const int id[4] = {d.x, d.y, d.z, d.w};
  double P[4][3], ph[4], pn[4];
  for (int v = 0; v < 4; ++v) {
    for (int e = 0; e < 3; ++e) P[v][e] = X[3 * (size_t)id[v] + e];
    ph[v] = phi[perm[id[v]]];
    pn[v] = dphi[perm[id[v]]];
  }
  const double U[3] = {U0, U1, U2};
  double F = 0.0;
  for (int b = 0; b < g.n; ++b)
    for (int a = 0; a < g.n; ++a) {
      const double s = g.x[a], t = g.x[b], w = g.w[a] * g.w[b];
      const double Nv[4] = {(1 - s) * (1 - t), s * (1 - t), (1 - s) * t, s * t};
      const double Ns[4] = {-(1 - t), (1 - t), -t, t};
      const double Nt[4] = {-(1 - s), -s, (1 - s), s};
      double jx[3] = {0, 0, 0}, je[3] = {0, 0, 0}, gs = 0, gt = 0, dn = 0;
      for (int v = 0; v < 4; ++v) {
        for (int e = 0; e < 3; ++e) {
          jx[e] += Ns[v] * P[v][e];
          je[e] += Nt[v] * P[v][e];
        }
        gs += Ns[v] * ph[v];
        gt += Nt[v] * ph[v];
        dn += Nv[v] * pn[v];
      }
      const double g11 = jx[0] * jx[0] + jx[1] * jx[1] + jx[2] * jx[2];
      const double g12 = jx[0] * je[0] + jx[1] * je[1] + jx[2] * je[2];
      const double g22 = je[0] * je[0] + je[1] * je[1] + je[2] * je[2];
      const double det = g11 * g22 - g12 * g12;
      const double c1 = (g22 * gs - g12 * gt) / det, c2 = (-g12 * gs + g11 * gt) / det;
      const double cr[3] = {jx[1] * je[2] - jx[2] * je[1], jx[2] * je[0] - jx[0] * je[2],
                            jx[0] * je[1] - jx[1] * je[0]};
      const double A = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      double G[3];
      for (int e = 0; e < 3; ++e) G[e] = c1 * jx[e] + c2 * je[e] + dn * cr[e] / A;
      const double p = -(U[0] * G[0] + U[1] * G[1] + U[2] * G[2] +
                         0.5 * (G[0] * G[0] + G[1] * G[1] + G[2] * G[2]));
      F += p * cr[dir] * w;
    }
  partials[k] = F;
}

// Fixed-order sum of the partials into *out (one block).
__global__ void k_sum_partials_noalloc(int nh, const double* __restrict__ partials,
                                       double* __restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < nh; i += blockDim.x) s += partials[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

extern "C" int wbem_hull_force_noalloc(wbem_handle h, const int* hull_cells, int n_hull,
                                       const double* U, int dir, const double* phi,
                                       const double* dphi_dn, double* force, void* stream) {
  if (!h) return WBEM_ERR_ARG;
  if (!U || !force || (n_hull > 0 && (!hull_cells || !phi || !dphi_dn)) || dir < 0 || dir > 2) {
    h->err = "wbem_hull_force_noalloc: bad argument";
    return WBEM_ERR_ARG;
  }
  if (n_hull < 0 || n_hull > kNoAllocMaxPanels) {
    h->err = "wbem_hull_force_noalloc: n_hull must be in [0, 65536] (size of the static scratch "
             "array); use wbem_hull_force for larger hulls";
    return WBEM_ERR_ARG;
  }
  if (h->N == 0 || !h->d_cell_dofs) {
    h->err = "wbem_hull_force_noalloc: set the geometry first";
    return WBEM_ERR_STATE;
  }
  if (h->device < 0 || h->device >= kMaxDevices) {
    h->err = "wbem_hull_force_noalloc: device index beyond the library's table of 64";
    return WBEM_ERR_CUDA;
  }
  if (h->gauss_n < 1 || h->gauss_n > 8) {
    h->err = "wbem_hull_force_noalloc: no quadrature rule (set the geometry first)";
    return WBEM_ERR_STATE;
  }
  // the handle's device is current from here on; the caller's is restored
  DeviceScope scope(h->device);
  if (!scope.ok) {
    h->err = "wbem_hull_force_noalloc: cannot select the handle's device";
    return WBEM_ERR_CUDA;
  }
  // one-time set-up per device (the first call on a device)
  double* partials = nullptr;
  {
    const cudaError_t e = partials_address(h->device, &partials);
    if (e != cudaSuccess) {
      h->err = std::string("wbem_hull_force_noalloc: cudaGetSymbolAddress failed: ") +
               cudaGetErrorString(e);
      return WBEM_ERR_CUDA;
    }
  }
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : h->stream;
  // the same line rule as the panels' tensor rule of the allocating path
  GaussLine g{};
  g.n = h->gauss_n;
  for (int a = 0; a < g.n; ++a) {
    g.x[a] = h->gauss_x[a];
    g.w[a] = h->gauss_w[a];
  }
  if (n_hull > 0)
    k_hull_partials_noalloc<<<(n_hull + 127) / 128, 128, 0, s>>>(
        n_hull, h->C, hull_cells, h->d_cell_dofs, h->d_perm, h->d_X, U[0], U[1], U[2], dir, phi,
        dphi_dn, g, partials);
  k_sum_partials_noalloc<<<1, 256, 0, s>>>(n_hull, partials, force);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    h->err = std::string("wbem_hull_force_noalloc: launch failed: ") + cudaGetErrorString(e);
    return WBEM_ERR_CUDA;
  }
  return WBEM_OK;
}
