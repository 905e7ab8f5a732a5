// Coarsest-level direct solver in FP64, replacing the reference's host
// CHOLMOD factor/solve (stencil_assembly.c:366-503).
//
// The coarsest operator (fixed rows and columns zeroed, unit diagonal,
// stencil_assembly.c:226-259) is banded in the natural node order: half
// bandwidth bw = 3*(nz*ny + ny + 1) + 2. Its lower band is stored
// column-major with leading dimension bw -- entry (r, c), 0 <= r - c <= bw,
// sits at c*bw + r -- so any rectangle inside the band is a dense
// column-major block.
//   factor : right-looking blocked band Cholesky, panel width NB:
//            POTRF of the NB x NB diagonal block (one CTA), TRSM of the panel
//            below it (one thread per row), SYRK update of the trailing band
//            triangle (32x32 tiles). A non-positive pivot sets *info and is
//            replaced by 1 so the factor completes; the host reports
//            TP_ERR_NOT_SPD.
//   solve  : L y = b and L^T x = y by blocks of NBS rows; the inverse of each
//            diagonal block is formed once per factorisation, so each block
//            step is two matrix-vector products.
#include <algorithm>

#include "tp_internal.h"

namespace tp {

constexpr int NB = 32;    // factor panel width
constexpr int NBS = 128;  // solve block size

__host__ __device__ __forceinline__ long lmax(long a, long b) { return a > b ? a : b; }
__host__ __device__ __forceinline__ long lmin(long a, long b) { return a < b ? a : b; }

__device__ __forceinline__ double bget(const double* B, long bw, long r, long c) {
  const long d = r - c;
  return (d >= 0 && d <= bw) ? B[c * bw + r] : 0.0;
}

// ----------------------------------------------------------------------------
// band assembly from the coarsest FP64 stencil (BCs already applied there)
__global__ void band_scatter_kernel(int nx, int ny, int nz, long nnodes, long bw,
                                    const double* __restrict__ st, double* __restrict__ B) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= nnodes * 27) return;
  const long n = t % nnodes;
  const int m = (int)(t / nnodes);
  const int j = n % ny;
  const int k = (n / ny) % nz;
  const int i = n / ((long)ny * nz);
  const int mx = m / 9 - 1, mz = (m / 3) % 3 - 1, my = m % 3 - 1;
  const int mi = i + mx, mk = k + mz, mj = j + my;
  if (mi < 0 || mi >= nx || mk < 0 || mk >= nz || mj < 0 || mj >= ny) return;
  const long nm = ((long)mi * nz + mk) * ny + mj;
  for (int c = 0; c < 3; c++)
    for (int d = 0; d < 3; d++) {
      const long r = 3 * n + c, col = 3 * nm + d;
      if (col <= r && r - col <= bw) B[col * bw + r] = st[(long)(m * 9 + 3 * c + d) * nnodes + n];
    }
}

void coarse_alloc(tp_ctx* c) {
  Coarse& C = c->coarse;
  const Level& L = c->L[c->nl - 1];
  C.n = L.ndof;
  C.bw = 3L * ((long)L.nz * L.ny + L.ny + 1) + 2;
  if (C.bw > C.n - 1) C.bw = std::max(1L, C.n - 1);
  C.band_elems = (size_t)C.n * (C.bw + 1) + 1;
  cudaMalloc(&C.band, C.band_elems * sizeof(double));
  C.nbs = NBS;
  C.nblk = (int)((C.n + NBS - 1) / NBS);
  cudaMalloc(&C.dinv, (size_t)C.nblk * NBS * NBS * 2 * sizeof(double));
  cudaMalloc(&C.vec, (size_t)C.n * 2 * sizeof(double));
  cudaMalloc(&C.info, sizeof(int));
  c->mem_bytes += (long)(C.band_elems + (size_t)C.nblk * NBS * NBS * 2 + C.n * 2) * 8;
}

void coarse_free(tp_ctx* c) {
  Coarse& C = c->coarse;
  cudaFree(C.band);
  cudaFree(C.dinv);
  cudaFree(C.vec);
  cudaFree(C.info);
  C = Coarse();
}

void coarse_assemble(tp_ctx* c) {
  ProfScope ps(c, P_COARSE_FACTOR);
  Coarse& C = c->coarse;
  const int l = c->nl - 1;
  const Level& L = c->L[l];
  cudaMemsetAsync(C.band, 0, C.band_elems * sizeof(double), c->s);
  const long work = L.nnodes * 27;
  band_scatter_kernel<<<grid_for(work, 256), 256, 0, c->s>>>(L.nx, L.ny, L.nz, L.nnodes, C.bw, c->st[l], C.band);
  TP_CHECK_LAUNCH(c, "band_scatter");
}

// ----------------------------------------------------------------------------
__global__ void potrf_kernel(double* __restrict__ B, long bw, long k, int nb, int* info) {
  __shared__ double S[NB][NB + 1];
  const int tid = threadIdx.x;
  for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
    const int r = idx % NB, cc = idx / NB;
    S[r][cc] = (r < nb && cc < nb && r >= cc) ? bget(B, bw, k + r, k + cc) : 0.0;
  }
  __syncthreads();
  for (int j = 0; j < nb; j++) {
    if (tid == 0) {
      double d = S[j][j];
      if (!(d > 0.0)) {
        atomicCAS(info, 0, (int)(k + j + 1));
        d = 1.0;
      }
      S[j][j] = sqrt(d);
    }
    __syncthreads();
    for (int r = j + 1 + tid; r < nb; r += blockDim.x) S[r][j] /= S[j][j];
    __syncthreads();
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
      const int r = idx % NB, cc = idx / NB;
      if (cc > j && r >= cc && r < nb) S[r][cc] -= S[r][j] * S[cc][j];
    }
    __syncthreads();
  }
  for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
    const int r = idx % NB, cc = idx / NB;
    if (r < nb && cc < nb && r >= cc && r - cc <= bw) B[(k + cc) * bw + (k + r)] = S[r][cc];
  }
}

// rows R0..R1 of panel columns k..k+nb-1: solve x L_kk^T = a, one thread per row
__global__ void trsm_kernel(double* __restrict__ B, long bw, long k, int nb, long R0, long R1) {
  __shared__ double S[NB][NB + 1];
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int r = idx % NB, cc = idx / NB;
    S[r][cc] = (r < nb && cc < nb && r >= cc) ? B[(k + cc) * bw + (k + r)] : 0.0;
  }
  __syncthreads();
  const long r = R0 + blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (r > R1) return;
  double x[NB];
  const long t0 = lmax(0L, r - k - bw);  // columns before t0 lie outside the band
#pragma unroll
  for (int t = 0; t < NB; t++) {
    if (t >= nb) break;
    double v = 0.0;
    if (t >= t0) {
      v = B[(k + t) * bw + r];
      for (int tt = (int)t0; tt < t; tt++) v -= x[tt] * S[t][tt];
      v /= S[t][t];
      B[(k + t) * bw + r] = v;
    }
    x[t] = v;
  }
}

// A(r,c) -= sum_t L(r,k+t) L(c,k+t), R0 <= c <= r <= R1, 32x32 tiles
__global__ void syrk_kernel(double* __restrict__ B, long bw, long k, int nb, long R0, long R1) {
  __shared__ double Lr[NB][33], Lc[NB][33];
  // blockIdx.x -> lower-triangular tile (tr, tc)
  const long b = blockIdx.x;
  long tr = (long)((sqrt(8.0 * (double)b + 1.0) - 1.0) / 2.0);
  while ((tr + 1) * (tr + 2) / 2 <= b) tr++;
  while (tr * (tr + 1) / 2 > b) tr--;
  const long tc = b - tr * (tr + 1) / 2;
  const long rb = R0 + tr * 32, cb = R0 + tc * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 256 threads
  for (int t = ty; t < NB; t += 8) {
    const long r = rb + tx, cc = cb + tx;
    Lr[t][tx] = (t < nb && r <= R1) ? bget(B, bw, r, k + t) : 0.0;
    Lc[t][tx] = (t < nb && cc <= R1) ? bget(B, bw, cc, k + t) : 0.0;
  }
  __syncthreads();
  const long r = rb + tx;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int cy = ty + 8 * q;
    const long cc = cb + cy;
    double s = 0.0;
#pragma unroll
    for (int t = 0; t < NB; t++) s += Lr[t][tx] * Lc[t][cy];
    if (r <= R1 && cc <= R1 && cc <= r && r - cc <= bw) B[cc * bw + r] -= s;
  }
}

// inverse of each diagonal block: thread per column, forward substitution;
// writes both column-major (dinv) and row-major (dinv + nblk*NBS*NBS) copies
__global__ void dinv_kernel(const double* __restrict__ B, long bw, long n, int nblk, double* __restrict__ D) {
  const int blk = blockIdx.y;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const long b0 = (long)blk * NBS;
  const int s = (int)lmin((long)NBS, n - b0);
  if (j >= NBS) return;
  double* Dc = D + (long)blk * NBS * NBS;
  double* Dr = D + (long)nblk * NBS * NBS + (long)blk * NBS * NBS;
  for (int i = 0; i < NBS; i++) {
    Dc[(long)j * NBS + i] = 0.0;
    Dr[(long)i * NBS + j] = 0.0;
  }
  if (j >= s) return;
  Dc[(long)j * NBS + j] = 1.0 / B[(b0 + j) * bw + (b0 + j)];
  for (int i = j + 1; i < s; i++) {
    double v = 0.0;
    for (int t = j; t < i; t++) v += bget(B, bw, b0 + i, b0 + t) * Dc[(long)j * NBS + t];
    Dc[(long)j * NBS + i] = -v / B[(b0 + i) * bw + (b0 + i)];
  }
  for (int i = j; i < s; i++) Dr[(long)i * NBS + j] = Dc[(long)j * NBS + i];
}

void coarse_factor(tp_ctx* c) {
  ProfScope ps(c, P_COARSE_FACTOR);
  Coarse& C = c->coarse;
  cudaMemsetAsync(C.info, 0, sizeof(int), c->s);
  for (long k = 0; k < C.n; k += NB) {
    const int nb = (int)std::min((long)NB, C.n - k);
    potrf_kernel<<<1, 256, 0, c->s>>>(C.band, C.bw, k, nb, C.info);
    const long R0 = k + nb, R1 = std::min(C.n - 1, k + nb - 1 + C.bw);
    if (R0 <= R1) {
      const long m = R1 - R0 + 1;
      trsm_kernel<<<grid_for(m, 64), 64, 0, c->s>>>(C.band, C.bw, k, nb, R0, R1);
      const long T = (m + 31) / 32;
      syrk_kernel<<<(unsigned)(T * (T + 1) / 2), 256, 0, c->s>>>(C.band, C.bw, k, nb, R0, R1);
    }
  }
  dinv_kernel<<<dim3(NBS / 64, C.nblk), 64, 0, c->s>>>(C.band, C.bw, C.n, C.nblk, C.dinv);
  TP_CHECK_LAUNCH(c, "coarse_factor");
}

// ----------------------------------------------------------------------------
// forward: t_r = b_r - sum_{c<b0} L(r,c) y_c for the rows of block blk (warp per row)
__global__ void fwd_rows_kernel(const double* __restrict__ B, long bw, long n, int blk,
                                const double* __restrict__ b, const double* __restrict__ y,
                                double* __restrict__ t) {
  const long b0 = (long)blk * NBS;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const long r = b0 + w;
  if (w >= NBS || r >= n) return;
  const long c0 = lmax(0L, r - bw);
  double s = 0.0;
  for (long cc = c0 + lane; cc < b0; cc += 32) s += B[cc * bw + r] * y[cc];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) t[r] = b[r] - s;
}

// y_blk = Dinv_blk t_blk (column-major Dinv, thread per output row)
__global__ void fwd_diag_kernel(const double* __restrict__ D, long n, int blk, const double* __restrict__ t,
                                double* __restrict__ y) {
  __shared__ double ts[NBS];
  const long b0 = (long)blk * NBS;
  const int i = threadIdx.x;
  ts[i] = (b0 + i < n) ? t[b0 + i] : 0.0;
  __syncthreads();
  if (b0 + i >= n) return;
  const double* Dc = D + (long)blk * NBS * NBS;
  double s = 0.0;
  for (int j = 0; j <= i; j++) s += Dc[(long)j * NBS + i] * ts[j];
  y[b0 + i] = s;
}

// backward: t_r = y_r - sum_{c>=b1} L(c,r) x_c (warp per row)
__global__ void bwd_rows_kernel(const double* __restrict__ B, long bw, long n, int blk,
                                const double* __restrict__ y, const double* __restrict__ x,
                                double* __restrict__ t) {
  const long b0 = (long)blk * NBS, b1 = lmin(n, b0 + NBS);
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const long r = b0 + w;
  if (w >= NBS || r >= n) return;
  const long c1 = lmin(n - 1, r + bw);
  double s = 0.0;
  for (long cc = b1 + lane; cc <= c1; cc += 32) s += B[r * bw + cc] * x[cc];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) t[r] = y[r] - s;
}

// x_blk = Dinv_blk^T t_blk (row-major copy, thread per output)
__global__ void bwd_diag_kernel(const double* __restrict__ D, long n, int nblk, int blk,
                                const double* __restrict__ t, double* __restrict__ x) {
  __shared__ double ts[NBS];
  const long b0 = (long)blk * NBS;
  const int i = threadIdx.x;
  ts[i] = (b0 + i < n) ? t[b0 + i] : 0.0;
  __syncthreads();
  if (b0 + i >= n) return;
  const double* Dr = D + (long)nblk * NBS * NBS + (long)blk * NBS * NBS;
  const int s = (int)lmin((long)NBS, n - b0);
  double acc = 0.0;
  for (int j = i; j < s; j++) acc += Dr[(long)j * NBS + i] * ts[j];
  x[b0 + i] = acc;
}

void coarse_solve(tp_ctx* c, const double* rhs, double* x) {
  ProfScope ps(c, P_COARSE_SOLVE);
  Coarse& C = c->coarse;
  double* y = C.vec;
  double* t = C.vec + C.n;
  for (int b = 0; b < C.nblk; b++) {
    fwd_rows_kernel<<<NBS / 8, 256, 0, c->s>>>(C.band, C.bw, C.n, b, rhs, y, t);
    fwd_diag_kernel<<<1, NBS, 0, c->s>>>(C.dinv, C.n, b, t, y);
  }
  for (int b = C.nblk - 1; b >= 0; b--) {
    bwd_rows_kernel<<<NBS / 8, 256, 0, c->s>>>(C.band, C.bw, C.n, b, y, x, t);
    bwd_diag_kernel<<<1, NBS, 0, c->s>>>(C.dinv, C.n, C.nblk, b, t, x);
  }
  TP_CHECK_LAUNCH(c, "coarse_solve");
}

}  // namespace tp
