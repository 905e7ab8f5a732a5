// CG vector updates and reductions (stencil_solvers.c:259-397,
// stencil_solvers.h:36-58). Every reduction is two-pass and order-fixed:
// blocks write partial sums, one block adds them in index order, so results
// are bit-reproducible from run to run. The CG scalars (rho, alpha, beta,
// relres) stay in device memory.
//
// Several right-hand sides (load cases sharing one operator) are handled as
// nr columns of length n stored one after the other; column r keeps its own
// scalars at d_scal[r * S_COUNT + slot] and its own reduction partials. A
// column whose relative residual has dropped below the tolerance is frozen
// (alpha = beta = 0), so the columns still iterating do not disturb it.
#include <math_constants.h>

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

static int dot_blocks(long n) {
  int nb = (int)((n + 255) / 256);
  if (nb > kDotBlocks) nb = kDotBlocks;
  if (nb < 1) nb = 1;
  return nb;
}

// grid-stride dot per column with a fixed number of blocks -> partials[r * gridDim.x + block];
// b may be FP32 (the mixed V-cycle's output, widened exactly)
template <typename TB>
__global__ void dot_kernel(long n, const double* __restrict__ a, const TB* __restrict__ b,
                           double* __restrict__ partials) {
  const long off = (long)blockIdx.y * n;
  double s = 0.0;
  for (long i = blockIdx.x * 256L + threadIdx.x; i < n; i += (long)gridDim.x * 256)
    s += a[off + i] * (double)b[off + i];
  s = block_sum256(s);
  if (threadIdx.x == 0) partials[(long)blockIdx.y * gridDim.x + blockIdx.x] = s;
}

template <typename TB>
void dot_partials(tp_ctx* c, long n, const double* a, const TB* b, int* nblocks, int nr) {
  ProfScope ps(c, P_VECTOR);
  const int nb = dot_blocks(n);
  dot_kernel<TB><<<dim3(nb, nr), 256, 0, c->s>>>(n, a, b, c->d_red);
  TP_CHECK_LAUNCH(c, "dot");
  *nblocks = nb;
}
template void dot_partials<double>(tp_ctx*, long, const double*, const double*, int*, int);
template void dot_partials<float>(tp_ctx*, long, const double*, const float*, int*, int);

// op 0: sum; op 1: max. Column r (blockIdx.x) folds partials[r*nb .. r*nb + nb)
// into out[r * S_COUNT].
__global__ void finish_kernel(const double* __restrict__ partials, int nb, double* __restrict__ out, int op) {
  __shared__ double sh[256];
  partials += (long)blockIdx.x * nb;
  double s = 0.0;
  // each thread folds a contiguous chunk, in order
  const int per = (nb + 255) / 256;
  const int b0 = threadIdx.x * per;
  for (int i = b0; i < b0 + per && i < nb; i++) s = (op == 1) ? fmax(s, partials[i]) : s + partials[i];
  const double t = fold256(s, op == 1, sh);
  if (threadIdx.x == 0) out[(long)blockIdx.x * S_COUNT] = t;
}

void finish_sum(tp_ctx* c, int nblocks, int slot, int op, int nr) {
  ProfScope ps(c, P_VECTOR);
  finish_kernel<<<nr, 256, 0, c->s>>>(c->d_red, nblocks, c->d_scal + slot, op);
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
// K*0 = 0, so u1 = omega*invD*b exactly); a (invD) has one column, b and out nr
template <typename T>
__global__ void vscale_kernel(long n, const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ out,
                              T omega) {
  const long i = blockIdx.x * 256L + threadIdx.x;
  const long o = (long)blockIdx.y * n;  // column
  if (i < n) out[o + i] = omega * a[i] * (b[o + i] - T(0));
}
template <typename T>
void vscale(tp_ctx* c, long n, const T* a, const T* b, T* out, T omega, int nr) {
  ProfScope ps(c, P_VECTOR);
  vscale_kernel<T><<<dim3(grid_for(n, 256), nr), 256, 0, c->s>>>(n, a, b, out, omega);
  TP_CHECK_LAUNCH(c, "vscale");
}
template void vscale<double>(tp_ctx*, long, const double*, const double*, double*, double, int);
template void vscale<float>(tp_ctx*, long, const float*, const float*, float*, float, int);

// p = z (first iteration) or p = beta*p + z, beta of the column from the
// device; first = -1: the first iteration is the device counter's zero. z
// may be FP32 (the mixed V-cycle's output, widened exactly).
template <typename TZ>
__global__ void pupdate_kernel(long n, const TZ* __restrict__ z, double* __restrict__ p,
                               const double* __restrict__ scal, int first) {
  const long i = blockIdx.x * 256L + threadIdx.x;
  if (i >= n) return;
  const long o = (long)blockIdx.y * n;  // column
  if (first < 0) first = scal[S_IT] == 0.0;
  const double zi = (double)z[o + i];
  if (first)
    p[o + i] = zi;
  else
    p[o + i] = scal[blockIdx.y * S_COUNT + S_BETA] * p[o + i] + zi;
}
template <typename TZ>
void cg_pupdate(tp_ctx* c, long n, const TZ* z, double* p, int first, int nr) {
  ProfScope ps(c, P_VECTOR);
  pupdate_kernel<TZ><<<dim3(grid_for(n, 256), nr), 256, 0, c->s>>>(n, z, p, c->d_scal, first);
  TP_CHECK_LAUNCH(c, "cg_pupdate");
}
template void cg_pupdate<double>(tp_ctx*, long, const double*, double*, int, int);
template void cg_pupdate<float>(tp_ctx*, long, const float*, double*, int, int);

// u += alpha p ; r -= alpha q ; partials of <r, r>, per column; with rf, also
// rf = (float) r, the next mixed V-cycle's input (the cast it would start with)
__global__ void xr_kernel(long n, double* __restrict__ u, double* __restrict__ r, float* __restrict__ rf,
                          const double* __restrict__ p, const double* __restrict__ q,
                          const double* __restrict__ scal, double* __restrict__ partials) {
  const long off = (long)blockIdx.y * n;
  const double alpha = scal[blockIdx.y * S_COUNT + S_ALPHA];
  double s = 0.0;
  for (long i = off + blockIdx.x * 256L + threadIdx.x; i < off + n; i += (long)gridDim.x * 256) {
    u[i] += alpha * p[i];
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    if (rf) rf[i] = (float)ri;
    s += ri * ri;
  }
  s = block_sum256(s);
  if (threadIdx.x == 0) partials[(long)blockIdx.y * gridDim.x + blockIdx.x] = s;
}
void cg_xr_update(tp_ctx* c, long n, double* u, double* r, const double* p, const double* q, int* nblocks, int nr,
                  float* rf) {
  ProfScope ps(c, P_VECTOR);
  const int nb = dot_blocks(n);
  xr_kernel<<<dim3(nb, nr), 256, 0, c->s>>>(n, u, r, rf, p, q, c->d_scal, c->d_red);
  TP_CHECK_LAUNCH(c, "cg_xr_update");
  *nblocks = nb;
}

// Per column r (thread r):
// what 0: beta = rho/rhoold (before the p update), 0 once converged
// what 1: alpha = rho/dpr, rhoold = rho; 0 once converged
// what 2: relres = sqrt(rnorm2)/sqrt(bnorm2) (0 for a zero load); a column
//         below tol is marked converged at iteration `iter`. Thread 0 also
//         keeps the largest relres of the columns in S_MAXRR of column 0.
__global__ void scalars_kernel(double* scal, int what, int nr, double tol, int iter) {
  const int r = threadIdx.x;
  if (iter < 0) iter = (int)scal[S_IT];
  if (r < nr) {
    double* s = scal + (long)r * S_COUNT;
    const bool done = s[S_CONV] > 0.0;
    if (what == 0) s[S_BETA] = done ? 0.0 : s[S_RHO] / s[S_RHOOLD];
    if (what == 1) {
      s[S_ALPHA] = done ? 0.0 : s[S_RHO] / s[S_DPR];
      s[S_RHOOLD] = s[S_RHO];
    }
    if (what == 2 && !done) {
      // a non-finite load or residual norm gives a NaN relres (never "below
      // tol"), so the loop stops and reports it instead of converging
      const double bn = s[S_BNORM2], rn = s[S_RNORM2];
      if (!isfinite(bn) || !isfinite(rn))
        s[S_RELRES] = CUDART_NAN;
      else
        s[S_RELRES] = bn > 0.0 ? sqrt(rn) / sqrt(bn) : 0.0;
      if (s[S_RELRES] < tol) {
        s[S_CONV] = 1.0;
        s[S_ITER] = iter;
      }
    }
  }
  __syncwarp();
  if (what == 2 && r == 0) {
    double m = 0.0;
    for (int q = 0; q < nr; q++) {
      const double v = scal[(long)q * S_COUNT + S_RELRES];
      m = (v > m || v != v) ? v : m;  // a NaN column makes the maximum NaN
      if (m != m) break;
    }
    scal[S_MAXRR] = m;
  }
}
void cg_scalars(tp_ctx* c, int what, int nr, double tol, int iter) {
  ProfScope ps(c, P_VECTOR);
  scalars_kernel<<<1, 32, 0, c->s>>>(c->d_scal, what, nr, tol, iter);
  TP_CHECK_LAUNCH(c, "cg_scalars");
}

// clears the converged marks of the nr columns before a solve
__global__ void cg_reset_kernel(double* scal, int nr) {
  const int r = threadIdx.x;
  if (r < nr) {
    scal[(long)r * S_COUNT + S_CONV] = 0.0;
    scal[(long)r * S_COUNT + S_ITER] = -1.0;
    scal[(long)r * S_COUNT + S_RELRES] = 0.0;
  }
}
void cg_reset(tp_ctx* c, int nr) {
  cg_reset_kernel<<<1, 32, 0, c->s>>>(c->d_scal, nr);
  TP_CHECK_LAUNCH(c, "cg_reset");
}

}  // namespace tp
