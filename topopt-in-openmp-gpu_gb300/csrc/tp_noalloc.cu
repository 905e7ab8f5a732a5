// Density-filter adjoint v <- H (v / Hs) for callers that cannot allocate
// device memory. Some host applications own all of the GPU's memory: they
// reserve one arena or pool at start-up and hand out pieces of it themselves,
// and they forbid the libraries they link from calling cudaMalloc or cudaFree,
// because an outside allocation can exhaust or fragment the arena and a
// cudaFree waits for the whole device. Others run this step inside a loop
// with a fixed time budget, where an allocation's latency is not acceptable.
// The caller passes v in memory of its own; the intermediate v/Hs lives in a
// file-scope __device__ array of fixed size, so no call allocates anything.
//
// The array (kNoAllocMaxElements doubles, 16 MiB) is part of this library's
// module: every GPU that loads the library holds it until the process exits.
// All calls share it and it keeps the last call's contents; every entry a call
// reads is written by that same call first, so nothing needs clearing. Calls
// whose kernels overlap on the GPU (different streams, or different host
// threads) race on the array and must be serialised by the caller.
//
// Host code cannot name the array directly: its name in host code is only a
// host-side stand-in, not a device address. The first call on each device
// therefore asks the runtime for the array's device address
// (cudaGetSymbolAddress, with that device current), checks the result and
// caches it; make that first call before any stream capture. The result is
// the same as the context-based tp_filter_T (stencil_optimization.c:290-395).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>

#include "topopt_gb300.h"

namespace {

constexpr long kNoAllocMaxElements = 1L << 21;
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_filter_scratch[kNoAllocMaxElements];

double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

__device__ __forceinline__ void nbox(int i, int n, int cr, int& lo, int& hi) {
  lo = max(i - (cr - 1), 0);
  hi = min(i + cr + 1, n);
}

// tmp_e = v_e / Hs_e, with Hs_e the filter row sum summed in the reference's
// x, z, y order
__global__ void noalloc_div_kernel(int ex, int ey, int ez, int cr, double rmin, const double* __restrict__ v,
                                   double* __restrict__ tmp) {
  const long ne = (long)ex * ey * ez;
  for (long e = blockIdx.x * 256L + threadIdx.x; e < ne; e += (long)gridDim.x * 256) {
    const int j = e % ey, k = (e / ey) % ez, i = e / ((long)ey * ez);
    int i0, i1, k0, k1, j0, j1;
    nbox(i, ex, cr, i0, i1);
    nbox(k, ez, cr, k0, k1);
    nbox(j, ey, cr, j0, j1);
    double hs = 0.0;
    for (int i2 = i0; i2 < i1; i2++)
      for (int k2 = k0; k2 < k1; k2++)
        for (int j2 = j0; j2 < j1; j2++) {
          const unsigned d2 = (unsigned)((i - i2) * (i - i2) + (j - j2) * (j - j2) + (k - k2) * (k - k2));
          hs += fmax(0.0, rmin - sqrt((double)d2));
        }
    tmp[e] = v[e] / hs;
  }
}

// v_e = sum_e2 w(e, e2) tmp_e2
__global__ void noalloc_sum_kernel(int ex, int ey, int ez, int cr, double rmin, const double* __restrict__ tmp,
                                   double* __restrict__ v) {
  const long ne = (long)ex * ey * ez;
  for (long e = blockIdx.x * 256L + threadIdx.x; e < ne; e += (long)gridDim.x * 256) {
    const int j = e % ey, k = (e / ey) % ez, i = e / ((long)ey * ez);
    int i0, i1, k0, k1, j0, j1;
    nbox(i, ex, cr, i0, i1);
    nbox(k, ez, cr, k0, k1);
    nbox(j, ey, cr, j0, j1);
    double s = 0.0;
    for (int i2 = i0; i2 < i1; i2++)
      for (int k2 = k0; k2 < k1; k2++)
        for (int j2 = j0; j2 < j1; j2++) {
          const unsigned d2 = (unsigned)((i - i2) * (i - i2) + (j - j2) * (j - j2) + (k - k2) * (k - k2));
          s += fmax(0.0, rmin - sqrt((double)d2)) * tmp[((long)i2 * ez + k2) * ey + j2];
        }
    v[e] = s;
  }
}

}  // namespace

extern "C" {

long tp_filter_T_noalloc_max_elements(void) { return kNoAllocMaxElements; }

tp_status tp_filter_T_noalloc(int nelx, int nely, int nelz, double rmin, double* v_dev, void* stream) {
  if (nelx < 1 || nely < 1 || nelz < 1 || !(rmin > 0) || !std::isfinite(rmin) || !v_dev) return TP_ERR_ARG;
  const long ne = (long)nelx * nely * nelz;
  if (ne > kNoAllocMaxElements) {
    std::fprintf(stderr,
                 "tp_filter_T_noalloc: %ld elements exceed the fixed scratch of %ld elements; "
                 "use tp_filter_T on a context instead\n",
                 ne, kNoAllocMaxElements);
    return TP_ERR_ARG;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TP_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return TP_ERR_ARG;
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_filter_scratch);
      if (e != cudaSuccess || !p) return TP_ERR_CUDA;
      g_scratch_addr[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch_addr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // a radius past the grid's largest extent reaches every element: the box
  // [i - (cr - 1), i + cr] clipped to the grid is then the whole axis, so the
  // box half-width is capped there (and stays an int for any finite rmin)
  const int span = std::max(nelx, std::max(nely, nelz)) + 1;
  const int cr = rmin >= (double)span ? span : (int)std::ceil(rmin);
  long nb = (ne + 255) / 256;
  if (nb > 4096) nb = 4096;
  // launched through cudaLaunchKernel so that each launch's own status is
  // read from its return value: an error the caller left pending from its
  // own work is neither reported here nor cleared
  int ax = nelx, ay = nely, az = nelz, acr = cr;
  double ar = rmin;
  double* av = v_dev;
  double* at = scratch;
  void* a1[] = {&ax, &ay, &az, &acr, &ar, &av, &at};
  void* a2[] = {&ax, &ay, &az, &acr, &ar, &at, &av};
  const dim3 grid((unsigned)nb), block(256);
  if (cudaLaunchKernel((const void*)noalloc_div_kernel, grid, block, a1, 0, s) != cudaSuccess) return TP_ERR_CUDA;
  if (cudaLaunchKernel((const void*)noalloc_sum_kernel, grid, block, a2, 0, s) != cudaSuccess) return TP_ERR_CUDA;
  return TP_OK;
}

}  // extern "C"
