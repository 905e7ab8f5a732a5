// CG vector updates and reductions (stencil_solvers.c:259-397,
// stencil_solvers.h:36-58). Every reduction is two-pass and order-fixed:
// blocks write partial sums, one block adds them in index order, so results
// are bit-reproducible from run to run. The CG scalars (rho, alpha, beta,
// relres) stay in device memory; the host reads relres once per iteration.
#include "tp_internal.h"

namespace tp {

int grid_for(long n, int threads) {
  long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  return (int)b;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// sum of a block of 256 threads, valid in thread 0
__device__ __forceinline__ double block_sum256(double v) {
  __shared__ double sh[8];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < 8; w++) s += sh[w];
  return s;
}

constexpr int kDotBlocks = 2048;

// grid-stride dot with a fixed number of blocks -> partials[0..gridDim)
__global__ void dot_kernel(long n, const double* __restrict__ a, const double* __restrict__ b,
                           double* __restrict__ partials) {
  double s = 0.0;
  for (long i = blockIdx.x * 256L + threadIdx.x; i < n; i += (long)gridDim.x * 256) s += a[i] * b[i];
  s = block_sum256(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

void dot_partials(tp_ctx* c, long n, const double* a, const double* b, int* nblocks) {
  ProfScope ps(c, P_VECTOR);
  int nb = (int)((n + 255) / 256);
  if (nb > kDotBlocks) nb = kDotBlocks;
  if (nb < 1) nb = 1;
  dot_kernel<<<nb, 256, 0, c->s>>>(n, a, b, c->d_red);
  TP_CHECK_LAUNCH(c, "dot");
  *nblocks = nb;
}

// op 0: sum; op 1: max
__global__ void finish_kernel(const double* __restrict__ partials, int nb, double* __restrict__ out, int op) {
  __shared__ double sh[256];
  double s = (op == 1) ? 0.0 : 0.0;
  // each thread folds a contiguous chunk, in order
  const int per = (nb + 255) / 256;
  const int b0 = threadIdx.x * per;
  for (int i = b0; i < b0 + per && i < nb; i++) s = (op == 1) ? fmax(s, partials[i]) : s + partials[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = sh[0];
    for (int i = 1; i < 256; i++) t = (op == 1) ? fmax(t, sh[i]) : t + sh[i];
    *out = t;
  }
}

void finish_sum(tp_ctx* c, int nblocks, int slot, int op) {
  ProfScope ps(c, P_VECTOR);
  finish_kernel<<<1, 256, 0, c->s>>>(c->d_red, nblocks, c->d_scal + slot, op);
  TP_CHECK_LAUNCH(c, "finish");
}

template <typename A, typename B>
__global__ void cast_kernel(long n, const A* __restrict__ a, B* __restrict__ b) {
  const long i = blockIdx.x * 256L + threadIdx.x;
  if (i < n) b[i] = (B)a[i];
}
void cast_d2f(tp_ctx* c, long n, const double* a, float* b) {
  ProfScope ps(c, P_VECTOR);
  cast_kernel<double, float><<<grid_for(n, 256), 256, 0, c->s>>>(n, a, b);
  TP_CHECK_LAUNCH(c, "cast_d2f");
}
void cast_f2d(tp_ctx* c, long n, const float* a, double* b) {
  ProfScope ps(c, P_VECTOR);
  cast_kernel<float, double><<<grid_for(n, 256), 256, 0, c->s>>>(n, a, b);
  TP_CHECK_LAUNCH(c, "cast_f2d");
}

// out = omega * a * b (the first Jacobi sweep from a zero initial guess:
// K*0 = 0, so u1 = omega*invD*b exactly)
template <typename T>
__global__ void vscale_kernel(long n, const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ out, T omega) {
  const long i = blockIdx.x * 256L + threadIdx.x;
  if (i < n) out[i] = omega * a[i] * (b[i] - T(0));
}
template <typename T>
void vscale(tp_ctx* c, long n, const T* a, const T* b, T* out, T omega) {
  ProfScope ps(c, P_VECTOR);
  vscale_kernel<T><<<grid_for(n, 256), 256, 0, c->s>>>(n, a, b, out, omega);
  TP_CHECK_LAUNCH(c, "vscale");
}
template void vscale<double>(tp_ctx*, long, const double*, const double*, double*, double);
template void vscale<float>(tp_ctx*, long, const float*, const float*, float*, float);

// p = z (first iteration) or p = beta*p + z, beta = rho/rhoold from the device
__global__ void pupdate_kernel(long n, const double* __restrict__ z, double* __restrict__ p,
                               const double* __restrict__ scal, int first) {
  const long i = blockIdx.x * 256L + threadIdx.x;
  if (i >= n) return;
  if (first)
    p[i] = z[i];
  else
    p[i] = scal[S_BETA] * p[i] + z[i];
}
void cg_pupdate(tp_ctx* c, long n, const double* z, double* p, int first) {
  ProfScope ps(c, P_VECTOR);
  pupdate_kernel<<<grid_for(n, 256), 256, 0, c->s>>>(n, z, p, c->d_scal, first);
  TP_CHECK_LAUNCH(c, "cg_pupdate");
}

// u += alpha p ; r -= alpha q ; partials of <r, r>
__global__ void xr_kernel(long n, double* __restrict__ u, double* __restrict__ r,
                          const double* __restrict__ p, const double* __restrict__ q,
                          const double* __restrict__ scal, double* __restrict__ partials) {
  const double alpha = scal[S_ALPHA];
  double s = 0.0;
  for (long i = blockIdx.x * 256L + threadIdx.x; i < n; i += (long)gridDim.x * 256) {
    u[i] += alpha * p[i];
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    s += ri * ri;
  }
  s = block_sum256(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}
void cg_xr_update(tp_ctx* c, long n, double* u, double* r, const double* p, const double* q, int* nblocks) {
  ProfScope ps(c, P_VECTOR);
  int nb = (int)((n + 255) / 256);
  if (nb > kDotBlocks) nb = kDotBlocks;
  xr_kernel<<<nb, 256, 0, c->s>>>(n, u, r, p, q, c->d_scal, c->d_red);
  TP_CHECK_LAUNCH(c, "cg_xr_update");
  *nblocks = nb;
}

// what 0: beta = rho/rhoold (before the p update)
// what 1: alpha = rho/dpr, rhoold = rho
// what 2: relres = sqrt(rnorm2)/sqrt(bnorm2)
__global__ void scalars_kernel(double* s, int what) {
  if (what == 0) s[S_BETA] = s[S_RHO] / s[S_RHOOLD];
  if (what == 1) {
    s[S_ALPHA] = s[S_RHO] / s[S_DPR];
    s[S_RHOOLD] = s[S_RHO];
  }
  if (what == 2) s[S_RELRES] = sqrt(s[S_RNORM2]) / sqrt(s[S_BNORM2]);
}
void cg_scalars(tp_ctx* c, int what) {
  ProfScope ps(c, P_VECTOR);
  scalars_kernel<<<1, 1, 0, c->s>>>(c->d_scal, what);
  TP_CHECK_LAUNCH(c, "cg_scalars");
}

}  // namespace tp
