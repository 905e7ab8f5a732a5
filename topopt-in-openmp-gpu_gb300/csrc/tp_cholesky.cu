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
//            below it (one warp per row), SYRK update of the trailing band
//            triangle (32x32 tiles). A non-positive pivot sets *info and is
//            replaced by 1 so the factor completes; the host reports
//            TP_ERR_NOT_SPD.
//   solve  : L y = b and L^T x = y by blocks of NBS rows; the inverse of each
//            diagonal block is formed once per factorisation, so each block
//            step is two matrix-vector products. Both sweeps run as one
//            cooperative launch with grid barriers between the half steps
//            (or, where that launch plan does not apply, as two launches per
//            block step).
#include <algorithm>

#include "tp_internal.h"

namespace tp {

constexpr int NB = 32;    // factor panel width
constexpr int NBS = 512;  // solve block size (largest)

__host__ __device__ __forceinline__ long lmax(long a, long b) { return a > b ? a : b; }
__host__ __device__ __forceinline__ long lmin(long a, long b) { return a < b ? a : b; }

__device__ __forceinline__ double bget(const double* B, long bw, long r, long c) {
  const long d = r - c;
  return (d >= 0 && d <= bw) ? B[c * bw + r] : 0.0;
}

static void ps_plan(tp_ctx* c);

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
  C.nbs = (int)std::min((long)NBS, ((C.n + 31) / 32) * 32);
  C.nblk = (int)((C.n + C.nbs - 1) / C.nbs);
  const size_t dsz = (size_t)C.nblk * C.nbs * C.nbs;
  const size_t lsz = (size_t)C.nblk * C.nbs * C.bw;
  cudaMalloc(&C.dinv, dsz * sizeof(double));
  cudaMalloc(&C.dinvT, dsz * sizeof(double));
  cudaMalloc(&C.lrow, lsz * sizeof(double));
  // work columns: y and t, kSolveCols each, then rhs and sol of a single solve
  cudaMalloc(&C.vec, (size_t)C.n * (2 * 8 + 2) * sizeof(double));
  C.rhs = C.vec + 16 * C.n;
  C.sol = C.vec + 17 * C.n;
  cudaMalloc(&C.info, sizeof(int));
  cudaMalloc(&C.linv, (NB * NB + NB) * sizeof(double));  // current diagonal block of L and 1/L(j,j)
  cudaStreamCreateWithFlags(&C.s2, cudaStreamNonBlocking);
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  C.prio_high = hi;
  cudaEventCreateWithFlags(&C.ev_panel, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&C.ev_rest, cudaEventDisableTiming);
  c->mem_bytes += (long)(C.band_elems + 2 * dsz + lsz + C.n * 18) * 8;
  int* flags = nullptr;  // barrier counter, status word, exit counter
  if (cudaMalloc(&flags, 3 * sizeof(int)) == cudaSuccess) {
    cudaMemsetAsync(flags, 0, 3 * sizeof(int), c->s);
    C.bar = reinterpret_cast<unsigned*>(flags);
    C.serr = flags + 1;
  }
  ps_plan(c);
}

void coarse_free(tp_ctx* c) {
  Coarse& C = c->coarse;
  cudaFree(C.band);
  cudaFree(C.dinv);
  cudaFree(C.dinvT);
  cudaFree(C.lrow);
  cudaFree(C.vec);
  if (C.graph_exec) cudaGraphExecDestroy(C.graph_exec);
  if (C.factor_exec) cudaGraphExecDestroy(C.factor_exec);
  cudaFree(C.info);
  cudaFree(C.linv);
  if (C.s2) cudaStreamDestroy(C.s2);
  if (C.ev_panel) cudaEventDestroy(C.ev_panel);
  if (C.ev_rest) cudaEventDestroy(C.ev_rest);
  cudaFree(C.bar);  // C.serr shares its allocation
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
// Factor the nb x nb diagonal block held (updated, lower part, zero above the
// diagonal) in S with the 256 threads of the CTA: L into S and into the band,
// and into lblk_out (row-major 32x32, zero above the diagonal, followed by
// the 32 reciprocals 1/L(j,j)). A non-positive pivot sets *info (first
// column + 1) and is replaced by 1 so that the factor completes.
//
// This block lies on the factorisation's critical path (one per 32 columns),
// and FP64 issue per SM is scarce on this part, so the work is spread over
// all warps and the serial chain per column is kept to one multiply-add and
// one reciprocal square root: thread (i, g) owns row i, columns g, g+8, g+16,
// g+24; column j is updated unscaled (with 1/L(j,j)^2) and scaled one step
// later; the owner of (j+1, j+1) forms the next pivot right after its last
// update. (No inverse is formed: the panel solve below substitutes with L
// directly, which keeps this block -- the part of each 32-column step that
// no other CTA can share -- short.)
__device__ __forceinline__ void diag_pivot(double (*S)[NB + 1], double* rp, int j, long k, int* info) {
  double d = S[j][j];
  if (!(d > 0.0)) {
    atomicCAS(info, 0, (int)(k + j + 1));
    d = 1.0;
  }
  const double r = rsqrt(d);
  rp[j] = r;
  rp[NB + j] = r * r;  // 1/d for the unscaled column update
  S[j][j] = d * r;
}

__device__ void factor_diag_block(double* __restrict__ B, long bw, long k, int nb, double (*S)[NB + 1],
                                  double* __restrict__ lblk_out, int* info) {
  __shared__ double rp[2 * NB];  // 1/L(j,j), then 1/L(j,j)^2
  const int tid = threadIdx.x;
  const int i = tid >> 3, g = tid & 7;
  if (tid == 0) diag_pivot(S, rp, 0, k, info);
  __syncthreads();
  for (int j = 0; j < nb; j++) {
    const double r2 = rp[NB + j];
    if (j >= 1 && g == 0 && i >= j && i < nb) S[i][j - 1] *= rp[j - 1];
    if (i > j && i < nb) {
      const double sij = S[i][j] * r2;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int t = g + 8 * q;
        if (t > j && t <= i) S[i][t] -= sij * S[t][j];
      }
    }
    if (j + 1 < nb && i == j + 1 && g == ((j + 1) & 7)) diag_pivot(S, rp, j + 1, k, info);
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int r = idx % NB, cc = idx / NB;
    const bool in = r < nb && cc < nb && r >= cc;
    if (in && r - cc <= bw) B[(k + cc) * bw + (k + r)] = S[r][cc];
    lblk_out[r * NB + cc] = in ? S[r][cc] : 0.0;
  }
  if (threadIdx.x < NB) lblk_out[NB * NB + threadIdx.x] = threadIdx.x < nb ? rp[threadIdx.x] : 0.0;
}

// the first diagonal block (later ones are factored inside syrk_kernel)
__global__ void potrf_kernel(double* __restrict__ B, long bw, long k, int nb, double* __restrict__ linv, int* info) {
  __shared__ double S[NB][NB + 1];
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int r = idx % NB, cc = idx / NB;
    S[r][cc] = (r < nb && cc < nb && r >= cc) ? bget(B, bw, k + r, k + cc) : 0.0;
  }
  __syncthreads();
  factor_diag_block(B, bw, k, nb, S, linv, info);
}

// panel rows R0..R1 of columns k..k+nb-1: solve x L_kk^T = a for each row,
// one warp per row, lane t holding x_t: at step p lane p finishes
// x_p = acc_p / L(p,p) and broadcasts it, lanes t > p subtract L(t,p) x_p
__global__ void trsm_kernel(double* __restrict__ B, long bw, long k, int nb, long R0, long R1,
                            const double* __restrict__ lblk) {
  __shared__ double Lb[NB][NB + 1], rp[NB];
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) Lb[idx / NB][idx % NB] = lblk[idx];
  if (threadIdx.x < NB) rp[threadIdx.x] = lblk[NB * NB + threadIdx.x];
  __syncthreads();
  const int w = threadIdx.x >> 5, t = threadIdx.x & 31;
  const long r = R0 + (long)blockIdx.x * (blockDim.x >> 5) + w;
  if (r > R1) return;
  double acc = (t < nb) ? bget(B, bw, r, k + t) : 0.0;
  double x = 0.0;
#pragma unroll
  for (int p = 0; p < NB; p++) {
    const double xp = __shfl_sync(0xffffffffu, acc * rp[p], p);
    if (t == p) x = xp;
    if (t > p) acc -= Lb[t][p] * xp;
  }
  if (t < nb && r - (k + t) <= bw) B[(k + t) * bw + r] = x;
}

// A(r,c) -= sum_t L(r,k+t) L(c,k+t), R0 <= c <= r <= R1, 32x32 tiles (tr, tc)
// of the trailing triangle. part 1: the first tile column only (tc = 0, the
// next panel), whose tile (0,0) -- the next diagonal block -- is then
// factored by its CTA for the next step; part 2: the other tiles (tc >= 1).
__global__ void syrk_kernel(double* __restrict__ B, long bw, long n, long k, int nb, long R0, long R1,
                            double* __restrict__ linv, int* info, int part) {
  __shared__ double Lr[NB][33], Lc[NB][33];
  __shared__ double S[NB][NB + 1];
  long tr, tc;
  if (part == 1) {
    tr = blockIdx.x;
    tc = 0;
  } else {  // blockIdx.x -> lower-triangular tile among those with tc >= 1
    const long b = blockIdx.x;
    long q = (long)((sqrt(8.0 * (double)b + 1.0) - 1.0) / 2.0);
    while ((q + 1) * (q + 2) / 2 <= b) q++;
    while (q * (q + 1) / 2 > b) q--;
    tr = q + 1;
    tc = b - q * (q + 1) / 2 + 1;
  }
  const long rb = R0 + tr * 32, cb = R0 + tc * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 256 threads
  for (int t = ty; t < NB; t += 8) {
    const long r = rb + tx, cc = cb + tx;
    Lr[t][tx] = (t < nb && r <= R1) ? bget(B, bw, r, k + t) : 0.0;
    Lc[t][tx] = (t < nb && cc <= R1) ? bget(B, bw, cc, k + t) : 0.0;
  }
  __syncthreads();
  const bool diag_next = part == 1 && tr == 0;
  const long r = rb + tx;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int cy = ty + 8 * q;
    const long cc = cb + cy;
    double s = 0.0;
#pragma unroll
    for (int t = 0; t < NB; t++) s += Lr[t][tx] * Lc[t][cy];
    double v = 0.0;
    const bool upd = r <= R1 && cc <= R1 && cc <= r && r - cc <= bw;
    if (upd) {
      v = B[cc * bw + r] - s;
      B[cc * bw + r] = v;
    }
    // entries of the next diagonal block that this step leaves alone keep their value
    if (diag_next) S[tx][cy] = upd ? v : ((cc <= r && r < n) ? bget(B, bw, r, cc) : 0.0);
  }
  if (diag_next) {
    __syncthreads();
    const int nb2 = (int)lmin((long)NB, n - R0);
    factor_diag_block(B, bw, R0, nb2, S, linv, info);
  }
}

// Inverse of each diagonal NBSxNBS block of L, one CTA per (block, 32-column
// chunk): the chunk's columns X of L_bb^{-1} are found by blocked forward
// substitution over 32-row chunks R,
//   acc = E_R - sum_{S<R} L_RS X_S,    X_R = L_RR^{-1} acc (substitution),
// with X kept in shared memory. Writes D (row-major) and D^T (row-major).
constexpr int kDinvThreads = 256;

__global__ void __launch_bounds__(kDinvThreads)
    dinv_kernel(const double* __restrict__ B, long bw, long n, int nbs, double* __restrict__ D,
                double* __restrict__ DT) {
  extern __shared__ double smem[];
  double* X = smem;                    // nbs x 33
  double* Lt = X + (long)nbs * 33;     // 32 x 33
  double* Acc = Lt + 32 * 33;          // 32 x 33
  const int blk = blockIdx.y, cc = blockIdx.x, tid = threadIdx.x;
  const long b0 = (long)blk * nbs;
  const int s = (int)lmin((long)nbs, n - b0);
  const int j0 = cc * 32;
  double* Db = D + (long)blk * nbs * nbs;
  double* DTb = DT + (long)blk * nbs * nbs;
  const int a = tid >> 3, q0 = (tid & 7) * 4;
  const int nR = (s + 31) / 32;
  for (int R = cc; R < nR; R++) {
    double acc[4];
#pragma unroll
    for (int q = 0; q < 4; q++) acc[q] = (R == cc && a == q0 + q) ? 1.0 : 0.0;
    for (int S = cc; S < R; S++) {
      for (int idx = tid; idx < 1024; idx += kDinvThreads) {
        const int ra = idx & 31, cs = idx >> 5;
        const long r = b0 + R * 32 + ra, col = b0 + S * 32 + cs;
        Lt[ra * 33 + cs] = (R * 32 + ra < s) ? bget(B, bw, r, col) : 0.0;
      }
      __syncthreads();
#pragma unroll 4
      for (int t = 0; t < 32; t++) {
        const double l = Lt[a * 33 + t];
        const double* xr = X + (long)(S * 32 + t) * 33 + q0;
#pragma unroll
        for (int q = 0; q < 4; q++) acc[q] -= l * xr[q];
      }
      __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 4; q++) Acc[a * 33 + q0 + q] = acc[q];
    for (int idx = tid; idx < 1024; idx += kDinvThreads) {
      const int ra = idx & 31, cs = idx >> 5;
      const long r = b0 + R * 32 + ra, col = b0 + R * 32 + cs;
      Lt[ra * 33 + cs] = (R * 32 + ra < s && R * 32 + cs < s && ra >= cs) ? bget(B, bw, r, col) : 0.0;
    }
    __syncthreads();
    if (tid < 32) {
      const int col = tid;
      for (int ra = 0; ra < 32; ra++) {
        double v = Acc[ra * 33 + col];
        for (int t = 0; t < ra; t++) v -= Lt[ra * 33 + t] * X[(long)(R * 32 + t) * 33 + col];
        const double d = Lt[ra * 33 + ra];
        X[(long)(R * 32 + ra) * 33 + col] = (R * 32 + ra < s && d != 0.0) ? v / d : 0.0;
      }
    }
    __syncthreads();
  }
  // D[r][j0+col] for r in [0, nbs): zero above the diagonal chunk and past s
  for (int idx = tid; idx < nbs * 32; idx += kDinvThreads) {
    const int r = idx >> 5, col = idx & 31;
    const double v = (r >= j0 && r < s && j0 + col < s) ? X[(long)r * 33 + col] : 0.0;
    Db[(long)r * nbs + j0 + col] = v;
  }
  for (int idx = tid; idx < nbs * 32; idx += kDinvThreads) {
    const int col = idx / nbs, r = idx % nbs;
    const double v = (r >= j0 && r < s && j0 + col < s) ? X[(long)r * 33 + col] : 0.0;
    DTb[(long)(j0 + col) * nbs + r] = v;
  }
}

// row-major copy of the band rows of each block left of the block:
// Lrow[blk][i][t] = L(b0 + i, b0 - bw + t), zero outside the band or the matrix
__global__ void lrow_kernel(const double* __restrict__ B, long bw, long n, int nbs, double* __restrict__ Lrow) {
  __shared__ double tile[32][33];
  const int blk = blockIdx.z;
  const long b0 = (long)blk * nbs;
  const int i0 = blockIdx.y * 32, t0 = blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int k = ty; k < 32; k += 8) {
    const long r = b0 + i0 + tx, col = b0 - bw + t0 + k;
    double v = 0.0;
    if (i0 + tx < nbs && r < n && col >= 0 && t0 + k < bw) v = bget(B, bw, r, col);
    tile[k][tx] = v;
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int i = i0 + k, t = t0 + tx;
    if (i < nbs && t < bw) Lrow[((long)blk * nbs + i) * bw + t] = tile[tx][k];
  }
}

// Lookahead over two streams. Per 32-column step k: the panel solve T_k, then
// on the main stream the update of the next panel's tile column with the
// factorisation of the next diagonal block (the chain every step waits on),
// and on the second stream the rest of the trailing update, which overlaps
// that chain and the next step's panel solve. The next step's first-column
// update waits for this step's rest, which writes the same tiles.
static void coarse_factor_launches(tp_ctx* c, size_t dinv_smem) {
  Coarse& C = c->coarse;
  cudaStream_t s = c->s, s2 = C.s2;
  cudaMemsetAsync(C.info, 0, sizeof(int), s);
  potrf_kernel<<<1, 256, 0, s>>>(C.band, C.bw, 0, (int)std::min((long)NB, C.n), C.linv, C.info);
  bool rest_pending = false;
  for (long k = 0; k < C.n; k += NB) {
    const int nb = (int)std::min((long)NB, C.n - k);
    const long R0 = k + nb, R1 = std::min(C.n - 1, k + nb - 1 + C.bw);
    if (R0 <= R1) {
      const long m = R1 - R0 + 1;
      // the chain's kernels run at the highest priority, so that their CTAs
      // take the SMs first as the trailing update's CTAs retire
      cudaLaunchAttribute pri[1];
      pri[0].id = cudaLaunchAttributePriority;
      pri[0].val.priority = C.prio_high;
      cudaLaunchConfig_t cfg = {};
      cfg.blockDim = dim3(256);
      cfg.stream = s;
      cfg.attrs = pri;
      cfg.numAttrs = 1;
      cfg.gridDim = dim3((unsigned)((m + 7) / 8));
      double* band = C.band;
      const long bw = C.bw, n = C.n;
      const double* lc = C.linv;
      cudaLaunchKernelEx(&cfg, trsm_kernel, band, bw, k, nb, R0, R1, lc);
      const long T = (m + 31) / 32;
      if (T > 1) {
        cudaEventRecord(C.ev_panel, s);
        cudaStreamWaitEvent(s2, C.ev_panel, 0);
      }
      if (rest_pending) cudaStreamWaitEvent(s, C.ev_rest, 0);
      cfg.gridDim = dim3((unsigned)T);
      cudaLaunchKernelEx(&cfg, syrk_kernel, band, bw, n, k, nb, R0, R1, C.linv, C.info, 1);
      rest_pending = false;
      if (T > 1) {
        syrk_kernel<<<(unsigned)(T * (T - 1) / 2), 256, 0, s2>>>(C.band, C.bw, C.n, k, nb, R0, R1, C.linv, C.info, 2);
        cudaEventRecord(C.ev_rest, s2);
        rest_pending = true;
      }
    }
  }
  if (rest_pending) cudaStreamWaitEvent(s, C.ev_rest, 0);
  dinv_kernel<<<dim3(C.nbs / 32, C.nblk), kDinvThreads, dinv_smem, c->s>>>(C.band, C.bw, C.n, C.nbs, C.dinv, C.dinvT);
  lrow_kernel<<<dim3((unsigned)((C.bw + 31) / 32), C.nbs / 32, C.nblk), dim3(32, 8), 0, c->s>>>(C.band, C.bw, C.n,
                                                                                               C.nbs, C.lrow);
}

// The launch sequence (about 2 per 32 columns) is captured once into a CUDA
// graph on the context's stream and replayed at every design iteration.
void coarse_factor(tp_ctx* c) {
  ProfScope ps(c, P_COARSE_FACTOR);
  Coarse& C = c->coarse;
  const size_t smem = ((size_t)C.nbs * 33 + 2 * 32 * 33) * sizeof(double);
  if (!C.factor_exec) {
    cudaFuncSetAttribute(dinv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      coarse_factor_launches(c, smem);
      if (cudaStreamEndCapture(c->s, &g) == cudaSuccess && g) {
        if (cudaGraphInstantiate(&C.factor_exec, g, cudaGraphInstantiateFlagUseNodePriority) != cudaSuccess)
          C.factor_exec = nullptr;
        cudaGraphDestroy(g);
      }
    }
    cudaGetLastError();
  }
  if (C.factor_exec)
    cudaGraphLaunch(C.factor_exec, c->s);
  else
    coarse_factor_launches(c, smem);
  TP_CHECK_LAUNCH(c, "coarse_factor");
}

// ----------------------------------------------------------------------------
// Block triangular solves, NBS rows per block, warp per row, coalesced:
//   forward   t = b_k - Lrow_k y,   y_k = D_k t
//   backward  t = y_k - L_{.,k}^T x (band columns are contiguous), x_k = D_k^T t
// Up to kSolveCols right-hand sides (columns n apart) share each load of L.
constexpr int kSolveCols = 8;

__device__ __forceinline__ double wsum(double s) {
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  return s;
}

template <int NR>
__global__ void fwd_rows_kernel(const double* __restrict__ Lrow, long bw, long n, int nbs, int blk,
                                const double* __restrict__ b, const double* __restrict__ y,
                                double* __restrict__ t) {
  const long b0 = (long)blk * nbs;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const long r = b0 + i;
  if (i >= nbs || r >= n) return;
  const long tlo = lmax(lmax(0L, bw - b0), (long)i);  // columns >= 0 and inside the band
  const double* L = Lrow + ((long)blk * nbs + i) * bw;
  const double* yy = y + (b0 - bw);
  double s[NR] = {};
  for (long q = tlo + lane; q < bw; q += 32) {
    const double l = L[q];
#pragma unroll
    for (int v = 0; v < NR; v++)
      s[v] += l * yy[v * n + q];
  }
#pragma unroll
  for (int v = 0; v < NR; v++)
    {
      const double sv = wsum(s[v]);
      if (lane == 0) t[v * n + r] = b[v * n + r] - sv;
    }
}

template <int NR>
__global__ void fwd_diag_kernel(const double* __restrict__ D, long n, int nbs, int blk,
                                const double* __restrict__ t, double* __restrict__ y) {
  const long b0 = (long)blk * nbs;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= nbs || b0 + i >= n) return;
  const double* Dr = D + ((long)blk * nbs + i) * nbs;
  const double* tt = t + b0;
  double s[NR] = {};
  for (int j = lane; j <= i; j += 32) {
    const double d = Dr[j];
#pragma unroll
    for (int v = 0; v < NR; v++)
      s[v] += d * tt[v * n + j];
  }
#pragma unroll
  for (int v = 0; v < NR; v++)
    {
      const double sv = wsum(s[v]);
      if (lane == 0) y[v * n + b0 + i] = sv;
    }
}

template <int NR>
__global__ void bwd_rows_kernel(const double* __restrict__ B, long bw, long n, int nbs, int blk,
                                const double* __restrict__ y, const double* __restrict__ x,
                                double* __restrict__ t) {
  const long b0 = (long)blk * nbs, b1 = lmin(n, b0 + nbs);
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const long r = b0 + i;
  if (i >= nbs || r >= n) return;
  const long c1 = lmin(n - 1, r + bw);
  double s[NR] = {};
  for (long cc = b1 + lane; cc <= c1; cc += 32) {
    const double l = B[r * bw + cc];
#pragma unroll
    for (int v = 0; v < NR; v++)
      s[v] += l * x[v * n + cc];
  }
#pragma unroll
  for (int v = 0; v < NR; v++)
    {
      const double sv = wsum(s[v]);
      if (lane == 0) t[v * n + r] = y[v * n + r] - sv;
    }
}

template <int NR>
__global__ void bwd_diag_kernel(const double* __restrict__ DT, long n, int nbs, int blk,
                                const double* __restrict__ t, double* __restrict__ x) {
  const long b0 = (long)blk * nbs;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= nbs || b0 + i >= n) return;
  const int s = (int)lmin((long)nbs, n - b0);
  const double* Dr = DT + ((long)blk * nbs + i) * nbs;
  const double* tt = t + b0;
  double acc[NR] = {};
  for (int j = i + lane; j < s; j += 32) {
    const double d = Dr[j];
#pragma unroll
    for (int v = 0; v < NR; v++)
      acc[v] += d * tt[v * n + j];
  }
#pragma unroll
  for (int v = 0; v < NR; v++)
    {
      const double sv = wsum(acc[v]);
      if (lane == 0) x[v * n + b0 + i] = sv;
    }
}

// ----------------------------------------------------------------------------
// The same block triangular solves as ONE cooperative launch: every half step
// of the forward and the backward sweep (Lrow product, D_k product, L^T
// product, D_k^T product) is a phase, and the CTAs meet at a grid barrier
// between phases instead of at a kernel boundary. CTA b owns rows
// b*R .. b*R+R-1 of every block; each row is split into P = 8/R fixed parts,
// one warp each, so every sum is formed in the same order on every call.
// While a CTA works on phase h (and waits at the barrier after it), the
// matrix rows of phase h+1 -- constant during the solve -- arrive in shared
// memory by cp.async; the vectors written by other CTAs are read through L2
// (ld.global.cg). Each barrier wait is bounded: a CTA that gives up sets the
// status word and every CTA leaves at its next barrier; the host reads (and
// clears) the word after the solve and reports TP_ERR_TIMEOUT.
constexpr int kPsWarps = 8;
constexpr long kBarrierSpin = 1L << 22;  // polls of the barrier counter (about a second)

struct PsArgs {
  const double* lrow;
  const double* band;
  const double* D;
  const double* DT;
  long bw, n;
  int nbs, nblk, R, P, seg;
  const double* rhs;
  double* y;
  double* t;
  double* x;
  unsigned* bar;  // barrier counter; bar[2] counts the CTAs out
  int* err;
  long spin;         // polls before a barrier wait gives up
  unsigned missing;  // arrivals each barrier waits for beyond the grid (0; 1 only in the failure test)
};

enum { PH_FA = 0, PH_FB, PH_BA, PH_BB };

// phase h -> (kind, block): forward FB_0, FA_1, FB_1, ..., FB_{m-1}, then
// backward BB_{m-1}, BA_{m-2}, BB_{m-2}, ..., BB_0 (m = nblk)
__device__ __forceinline__ void ps_phase(const PsArgs& a, int h, int& kind, int& k) {
  const int nf = 2 * a.nblk - 1;
  if (h < nf) {
    k = (h + 1) / 2;
    kind = (h & 1) ? PH_FA : PH_FB;
  } else {
    const int q = h - nf;
    k = a.nblk - 1 - (q + 1) / 2;
    kind = (q & 1) ? PH_BA : PH_BB;
  }
}

// Row i of block k in phase kind: the matrix entry at position e is m[e], the
// vector entry of column v at vb[v*n + voff + e], for lo <= e < hi. This
// warp's part of the row is [a0, a1).
struct PsRow {
  const double* m;
  const double* vb;
  long voff, a0, a1;
};

__device__ __forceinline__ bool ps_row(const PsArgs& a, int kind, int k, int i, int p, PsRow& r) {
  const long b0 = (long)k * a.nbs;
  const int s = (int)lmin((long)a.nbs, a.n - b0);
  if (i >= s) return false;
  long lo, hi;
  if (kind == PH_FA) {  // t = b - Lrow_k y over columns b0-bw+e, e in [max(0, bw-b0, i), bw)
    r.m = a.lrow + ((long)k * a.nbs + i) * a.bw;
    r.vb = a.y;
    r.voff = b0 - a.bw;
    lo = lmax(lmax(0L, a.bw - b0), (long)i);
    hi = a.bw;
  } else if (kind == PH_FB) {  // y_k = D_k t_k, lower triangle
    r.m = a.D + ((long)k * a.nbs + i) * a.nbs;
    r.vb = k == 0 ? a.rhs : a.t;
    r.voff = b0;
    lo = 0;
    hi = i + 1;
  } else if (kind == PH_BA) {  // t = y - L(b1.., r)^T x: band column r is contiguous
    const long rr = b0 + i, b1 = lmin(a.n, b0 + a.nbs);
    r.m = a.band + rr * a.bw;
    r.vb = a.x;
    r.voff = 0;
    lo = b1;
    hi = lmin(a.n - 1, rr + a.bw) + 1;
  } else {  // x_k = D_k^T t_k, upper triangle
    r.m = a.DT + ((long)k * a.nbs + i) * a.nbs;
    r.vb = k == a.nblk - 1 ? a.y : a.t;
    r.voff = b0;
    lo = i;
    hi = s;
  }
  const long len = lmax(0L, hi - lo), cs = (len + a.P - 1) / a.P;  // cs <= seg
  r.a0 = lo + p * cs;
  r.a1 = lmin(hi, r.a0 + cs);
  return true;
}

__device__ __forceinline__ void cp_async8(double* dst, const double* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// stage this warp's part of phase h's matrix row; lane l copies (and later
// reads) positions a0 + l, a0 + l + 32, ...
__device__ __forceinline__ void ps_stage(const PsArgs& a, int h, double* wbuf, int i, int p, int lane) {
  int kind, k;
  ps_phase(a, h, kind, k);
  PsRow r;
  if (!ps_row(a, kind, k, i, p, r)) return;
  for (long e = r.a0 + lane; e < r.a1; e += 32) cp_async8(wbuf + (e - r.a0), r.m + e);
}

// Grid barrier number h (targets h * gridDim.x arrivals), at most spin polls;
// false if this or another CTA gave up.
__device__ __forceinline__ bool ps_barrier(unsigned* bar, int* err, unsigned target, long spin) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    atomicAdd(bar, 1u);
    for (long it = 0;; it++) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(bar) : "memory");
      if (v >= target) break;
      if (*(volatile int*)err != 0) {
        ok = 0;
        break;
      }
      if (it >= spin) {
        atomicExch(err, 1);
        ok = 0;
        break;
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <int NR>
__global__ void __launch_bounds__(kPsWarps * 32) ps_solve_kernel(PsArgs a) {
  extern __shared__ double sm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rl = w / a.P, p = w % a.P;
  const int i = blockIdx.x * a.R + rl;
  auto buf = [&](int b) { return sm + (long)(b * kPsWarps + w) * a.seg; };  // stage b of this warp
  double* part = sm + 2L * kPsWarps * a.seg;  // [warp][NR]
  const int nph = 4 * a.nblk - 2;
  ps_stage(a, 0, buf(0), i, p, lane);
  cp_commit();
  for (int h = 0; h < nph; h++) {
    if (h + 1 < nph) {
      ps_stage(a, h + 1, buf((h + 1) & 1), i, p, lane);
      cp_commit();
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    int kind, k;
    ps_phase(a, h, kind, k);
    PsRow r;
    double acc[NR];
#pragma unroll
    for (int v = 0; v < NR; v++) acc[v] = 0.0;
    if (ps_row(a, kind, k, i, p, r)) {
      const double* mb = buf(h & 1);
      for (long e = r.a0 + lane; e < r.a1; e += 32) {
        const double mv = mb[e - r.a0];
        const long ve = r.voff + e;  // >= 0
#pragma unroll
        for (int v = 0; v < NR; v++) acc[v] += mv * __ldcg(r.vb + (v * a.n + ve));
      }
    }
#pragma unroll
    for (int v = 0; v < NR; v++) {
      const double sv = wsum(acc[v]);
      if (lane == 0) part[w * NR + v] = sv;
    }
    __syncthreads();
    if (threadIdx.x < a.R * NR) {
      const int rr = threadIdx.x / NR, v = threadIdx.x % NR;
      const long b0 = (long)k * a.nbs;
      const long row = blockIdx.x * a.R + rr;
      if (row < lmin((long)a.nbs, a.n - b0)) {
        double sum = 0.0;
        for (int q = 0; q < a.P; q++) sum += part[(rr * a.P + q) * NR + v];
        const long o = v * a.n + b0 + row;
        if (kind == PH_FA)
          a.t[o] = a.rhs[o] - sum;
        else if (kind == PH_FB)
          a.y[o] = sum;
        else if (kind == PH_BA)
          a.t[o] = __ldcg(a.y + o) - sum;
        else
          a.x[o] = sum;
      }
    }
    if (h + 1 < nph && !ps_barrier(a.bar, a.err, (unsigned)(h + 1) * gridDim.x + a.missing, a.spin)) break;
  }
  cp_wait<0>();
  // every CTA, on every path, counts itself out; the last one puts the
  // barrier counter (and the exit counter) back to zero for the next launch
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned* done = a.bar + 2;
    __threadfence();
    if (atomicAdd(done, 1u) == gridDim.x - 1) {
      atomicExch(a.bar, 0u);
      atomicExch(done, 0u);
    }
  }
}

// Launch plan: R rows per CTA (1, 2, 4 or 8), the fewest that keep one CTA
// per SM; P = 8/R warps per row; shared memory for two stages of every
// warp's longest part. No plan (ps_grid = 0) if the stages do not fit or
// the grid cannot be co-resident.
static void ps_plan(tp_ctx* c) {
  Coarse& C = c->coarse;
  C.ps_grid = 0;
  if (!C.bar || C.nblk < 1) return;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int R = 1;
  while (R < kPsWarps && (C.nbs + R - 1) / R > nsm) R *= 2;
  const int P = kPsWarps / R;
  const int grid = (C.nbs + R - 1) / R;
  if (grid > nsm) return;
  const long seg = std::max((C.bw + P - 1) / P, (long)(C.nbs + P - 1) / P);
  const size_t smem = (size_t)(2 * kPsWarps * seg + kPsWarps * 8) * sizeof(double);
  if (smem > 200 * 1024) return;
  auto fits = [&](const void* f) {
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return false;
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, kPsWarps * 32, smem) != cudaSuccess) return false;
    return per >= 1;
  };
  const bool ok = fits((const void*)ps_solve_kernel<1>) && fits((const void*)ps_solve_kernel<2>) &&
                  fits((const void*)ps_solve_kernel<4>) && fits((const void*)ps_solve_kernel<8>);
  cudaGetLastError();
  if (!ok) return;
  C.ps_R = R;
  C.ps_P = P;
  C.ps_seg = (int)seg;
  C.ps_smem = smem;
  C.ps_grid = grid;
}

template <int NR>
static void ps_launch(tp_ctx* c, const double* rhs, double* sol, double* y, double* t) {
  Coarse& C = c->coarse;
  PsArgs a{C.lrow, C.band, C.dinv, C.dinvT, C.bw, C.n, C.nbs, C.nblk, C.ps_R, C.ps_P, C.ps_seg,
           rhs, y, t, sol, C.bar, C.serr, C.ps_spin > 0 ? C.ps_spin : kBarrierSpin, (unsigned)C.ps_missing};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)C.ps_grid);
  cfg.blockDim = dim3(kPsWarps * 32);
  cfg.dynamicSmemBytes = C.ps_smem;
  cfg.stream = c->s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, ps_solve_kernel<NR>, a);
}

tp_status coarse_status(tp_ctx* c) {
  Coarse& C = c->coarse;
  if (!C.serr) return TP_OK;
  int e = 0;
  cudaMemcpyAsync(&e, C.serr, sizeof(int), cudaMemcpyDeviceToHost, c->s);
  if (cudaStreamSynchronize(c->s) != cudaSuccess) return TP_OK;  // the caller's own check reports it
  if (e != 0) {
    cudaMemsetAsync(C.serr, 0, sizeof(int), c->s);  // the context stays usable
    cudaStreamSynchronize(c->s);
    c->note = "coarse solve: a grid barrier wait gave up";
    return TP_ERR_TIMEOUT;
  }
  return TP_OK;
}

// the launch sequence of one solve of NR columns from rhs into sol (y and t
// are work columns of the same count)
template <int NR>
static void coarse_solve_launches(tp_ctx* c, const double* rhs, double* sol, double* y, double* t) {
  Coarse& C = c->coarse;
  if (C.solve_variant == 0 && C.ps_grid > 0) {
    ps_launch<NR>(c, rhs, sol, y, t);
    return;
  }
  const unsigned g = (unsigned)((C.nbs + 7) / 8);  // 8 warps per CTA, one row per warp
  for (int b = 0; b < C.nblk; b++) {
    const double* tin = rhs;
    if (b > 0) {
      fwd_rows_kernel<NR><<<g, 256, 0, c->s>>>(C.lrow, C.bw, C.n, C.nbs, b, rhs, y, t);
      tin = t;
    }
    fwd_diag_kernel<NR><<<g, 256, 0, c->s>>>(C.dinv, C.n, C.nbs, b, tin, y);
  }
  for (int b = C.nblk - 1; b >= 0; b--) {
    const double* tin = y;
    if (b < C.nblk - 1) {
      bwd_rows_kernel<NR><<<g, 256, 0, c->s>>>(C.band, C.bw, C.n, C.nbs, b, y, sol, t);
      tin = t;
    }
    bwd_diag_kernel<NR><<<g, 256, 0, c->s>>>(C.dinvT, C.n, C.nbs, b, tin, sol);
  }
}

// x = K_c^{-1} rhs for nr columns (n apart). Single solves replay a graph of
// the block launches captured once on the context's stream; inside a stream
// capture of a larger sequence (c->capturing) the launches are recorded
// directly, in chunks of kSolveCols columns working in the caller's buffers
// with the internal work columns.
void coarse_solve(tp_ctx* c, const double* rhs, double* x, int nr) {
  ProfScope ps(c, P_COARSE_SOLVE);
  Coarse& C = c->coarse;
  if (nr > 1 || c->capturing) {
    double *y = C.vec, *t = C.vec + (long)kSolveCols * C.n;
    for (int r0 = 0; r0 < nr;) {
      const double* b = rhs + (long)r0 * C.n;
      double* xx = x + (long)r0 * C.n;
      const int left = nr - r0;
      if (left >= 8) {
        coarse_solve_launches<8>(c, b, xx, y, t);
        r0 += 8;
      } else if (left >= 4) {
        coarse_solve_launches<4>(c, b, xx, y, t);
        r0 += 4;
      } else if (left >= 2) {
        coarse_solve_launches<2>(c, b, xx, y, t);
        r0 += 2;
      } else {
        coarse_solve_launches<1>(c, b, xx, y, t);
        r0 += 1;
      }
    }
    TP_CHECK_LAUNCH(c, "coarse_solve");
    return;
  }
  cudaMemcpyAsync(C.rhs, rhs, sizeof(double) * C.n, cudaMemcpyDeviceToDevice, c->s);
  if (!C.graph_exec) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      coarse_solve_launches<1>(c, C.rhs, C.sol, C.vec, C.vec + C.n);
      if (cudaStreamEndCapture(c->s, &g) == cudaSuccess && g) {
        if (cudaGraphInstantiate(&C.graph_exec, g, 0) != cudaSuccess) C.graph_exec = nullptr;
        cudaGraphDestroy(g);
      }
    }
    cudaGetLastError();
  }
  if (C.graph_exec)
    cudaGraphLaunch(C.graph_exec, c->s);
  else
    coarse_solve_launches<1>(c, C.rhs, C.sol, C.vec, C.vec + C.n);
  cudaMemcpyAsync(x, C.sol, sizeof(double) * C.n, cudaMemcpyDeviceToDevice, c->s);
  TP_CHECK_LAUNCH(c, "coarse_solve");
}

}  // namespace tp
