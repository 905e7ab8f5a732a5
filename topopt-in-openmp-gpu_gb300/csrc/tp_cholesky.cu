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
// The mixed form runs the single-launch factor and the block inverses in
// double-single arithmetic (tp_dsf.cuh) on the same FP64 storage: its V-cycle
// is FP32, so the last bits of FP64 buy its coarse correction nothing, while
// FP64 instructions hold the FP64 unit ~67 cycles each. Its factor kernel
// (pf_chain_ds / pf_bulk_ds) is laid out for FP32 latency rather than FP64
// throughput: at 256x128x128 the natural band takes 15.6 ms per
// factorisation against 28 ms for the same double-single operations in the
// FP64 layout (and 33 ms in FP64), with the same result bit for bit. The
// sweeps stay FP64: their phases wait on grid barriers and L2 reads, not on
// their few multiply-adds.
// By default the operator is eliminated in a one-level nested-dissection
// order (the nd_* code at the end of this file): the middle x node plane
// separates two halves whose partial band factors run in one launch, and
// whose solve sweeps share the phases of one launch, which halves the solve's
// chain of grid barriers (0.92 -> 0.63 ms per solve at 256x128x128); the
// factor, bound by its tile items rather than its chain once the chains are
// halved, runs two or three CTAs per SM (15.6 + 1.9 ms -> 11 + 0.8 ms for
// the partial factors and the block inverses).
#include <algorithm>
#include <type_traits>

#include "tp_dsf.cuh"
#include "tp_internal.h"

namespace tp {

constexpr int NB = 32;    // factor panel width
constexpr int NBS = 512;      // solve block size: at least this, or 4 rows per SM (608 on 152 SMs)
constexpr int kNbsMax = 768;  // the block inverses' staged rows fit the shared memory
constexpr long kBarrierSpin = 1L << 22;  // polls of a flag or barrier counter in global memory (about a second)

__host__ __device__ __forceinline__ long lmax(long a, long b) { return a > b ? a : b; }
__host__ __device__ __forceinline__ long lmin(long a, long b) { return a < b ? a : b; }

__device__ __forceinline__ double bget(const double* B, long bw, long r, long c) {
  const long d = r - c;
  return (d >= 0 && d <= bw) ? B[c * bw + r] : 0.0;
}

static void ps_plan(tp_ctx* c);
static void pf_plan(tp_ctx* c);
static void nd_layout(tp_ctx* c);
static void nd_plan(tp_ctx* c);

// the operations the factor and solve kernels need on either value type
__device__ __forceinline__ double vshfl(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ Dsf vshfl(Dsf v, int src) { return ds_shfl(v, src); }
__device__ __forceinline__ double vrsqrt(double d) { return rsqrt(d); }
__device__ __forceinline__ Dsf vrsqrt(Dsf d) { return ds_rsqrt(d); }
__device__ __forceinline__ bool vpos(double d) { return d > 0.0; }
__device__ __forceinline__ bool vpos(Dsf d) { return ds_val(d) > 0.0f; }
__device__ __forceinline__ double vrcp(double d) { return d != 0.0 ? 1.0 / d : 0.0; }
__device__ __forceinline__ Dsf vrcp(Dsf d) { return ds_val(d) != 0.0f ? ds_rcp(d) : Dsf(0.0f); }

// 8-byte asynchronous copies global -> shared (cp.async); the z form writes
// zero instead when the source is outside the band
__device__ __forceinline__ void cp_async8(double* dst, const double* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8z(double* dst, const double* src, bool in) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(src), "r"(in ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// sum over the warp (valid in lane 0), in a fixed tree
__device__ __forceinline__ double wsum(double s) {
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  return s;
}

// ----------------------------------------------------------------------------
// band assembly from the coarsest FP64 stencil (half stored, no boundary
// conditions) with the conditions of that level: fixed rows identity, and
// with masked the columns of fixed DOFs zeroed. Only neighbours m <= 13 (of
// smaller or equal node index) reach the lower band.
__global__ void band_scatter_kernel(int nx, int ny, int nz, int lim, long nnodes, long bw, int masked,
                                    const double* __restrict__ st, double* __restrict__ B) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= nnodes * 14) return;
  const long n = t % nnodes;
  const int m = (int)(t / nnodes);  // 0..13
  const int j = n % ny;
  const int k = (n / ny) % nz;
  const int i = n / ((long)ny * nz);
  const int mx = m / 9 - 1, mz = (m / 3) % 3 - 1, my = m % 3 - 1;
  const int mi = i + mx, mk = k + mz, mj = j + my;
  if (mi < 0 || mi >= nx || mk < 0 || mk >= nz || mj < 0 || mj >= ny) return;
  const long nm = ((long)mi * nz + mk) * ny + mj;
  const bool nfix = i == 0 && (j < lim || j >= ny - lim);
  const bool mfix = mi == 0 && (mj < lim || mj >= ny - lim);
  for (int c = 0; c < 3; c++)
    for (int d = 0; d < 3; d++) {
      const long r = 3 * n + c, col = 3 * nm + d;
      if (col > r || r - col > bw) continue;
      double v;
      if (nfix)
        v = (r == col) ? 1.0 : 0.0;
      else if (masked && m != 13 && mfix)
        v = 0.0;
      else
        v = (m == 13) ? st[(long)(3 * c + d) * nnodes + n] : st[((long)(13 - m) * 9 + 3 * d + c) * nnodes + nm];
      B[col * bw + r] = v;
    }
}

void coarse_alloc(tp_ctx* c) {
  Coarse& C = c->coarse;
  const Level& L = c->L[c->nl - 1];
  C.n = L.ndof;
  C.bw = 3L * ((long)L.nz * L.ny + L.ny + 1) + 2;
  if (C.bw > C.n - 1) C.bw = std::max(1L, C.n - 1);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&C.nsm, cudaDevAttrMultiProcessorCount, dev);
  // Solve blocks of 4 rows per SM: the single-launch solve's plan then gives
  // every SM a CTA of 4 rows in each phase (512-row blocks left 24 of 152 SMs
  // idle), and fewer blocks mean fewer phases (186 instead of 222 at
  // 256x128x128), for 19% more block-inverse work in the factorisation.
  const long nbs_sm = std::min((long)kNbsMax, std::max((long)NBS, (4L * C.nsm) / 32 * 32));
  C.nbs = (int)std::min(nbs_sm, ((C.n + 31) / 32) * 32);
  C.nblk = (int)((C.n + C.nbs - 1) / C.nbs);
  // the dissected factor shares the band, block inverse and block row arrays
  nd_layout(c);
  const long rows = C.nd_ok ? std::max(C.n, C.nd_ntot) : C.n;
  const long blks = C.nd_ok ? std::max((long)C.nblk, (long)C.nd_blk0[2] + C.nd_nblk[2]) : (long)C.nblk;
  C.band_elems = (size_t)rows * (C.bw + 1) + 1;
  dev_malloc(&C.band, C.band_elems * sizeof(double));
  const size_t dsz = (size_t)blks * C.nbs * C.nbs;
  const size_t lsz = (size_t)blks * C.nbs * C.bw;
  dev_malloc(&C.dinv, dsz * sizeof(double));
  dev_malloc(&C.dinvT, dsz * sizeof(double));
  dev_malloc(&C.lrow, lsz * sizeof(double));
  // work columns: y and t, kSolveCols each, then rhs and sol of a single solve
  dev_malloc(&C.vec, (size_t)C.n * (2 * 8 + 2) * sizeof(double));
  C.rhs = C.vec + 16 * C.n;
  C.sol = C.vec + 17 * C.n;
  dev_malloc(&C.info, sizeof(int));
  dev_malloc(&C.linv, (NB * NB + NB) * sizeof(double));  // current diagonal block of L and 1/L(j,j)
  cudaStreamCreateWithFlags(&C.s2, cudaStreamNonBlocking);
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  C.prio_high = hi;
  cudaEventCreateWithFlags(&C.ev_panel, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&C.ev_rest, cudaEventDisableTiming);
  c->mem_bytes += (long)(C.band_elems + 2 * dsz + lsz + C.n * 18) * 8;
  int* flags = nullptr;  // barrier counter, status word, exit counter
  if (dev_malloc(&flags, 3 * sizeof(int)) == cudaSuccess) {
    cudaMemsetAsync(flags, 0, 3 * sizeof(int), c->s);
    C.bar = reinterpret_cast<unsigned*>(flags);
    C.serr = flags + 1;
  } else {
    C.alloc_failed = true;
  }
  ps_plan(c);
  pf_plan(c);
  nd_plan(c);
}

void coarse_free(tp_ctx* c) {
  Coarse& C = c->coarse;
  dev_free(C.band);
  dev_free(C.dinv);
  dev_free(C.dinvT);
  dev_free(C.lrow);
  dev_free(C.vec);
  if (C.graph_exec) cudaGraphExecDestroy(C.graph_exec);
  if (C.factor_exec) cudaGraphExecDestroy(C.factor_exec);
  dev_free(C.info);
  dev_free(C.linv);
  if (C.s2) cudaStreamDestroy(C.s2);
  if (C.ev_panel) cudaEventDestroy(C.ev_panel);
  if (C.ev_rest) cudaEventDestroy(C.ev_rest);
  dev_free(C.bar);  // C.serr shares its allocation
  dev_free(C.pf_flags);
  dev_free(C.pf_rpk);
  dev_free(C.pf_off);
  if (C.nd_graph_exec) cudaGraphExecDestroy(C.nd_graph_exec);
  if (C.nd_factor_exec) cudaGraphExecDestroy(C.nd_factor_exec);
  dev_free(C.nd_map);
  dev_free(C.nd_vec);
  dev_free(C.nd_tail);
  dev_free(C.nd_flags);
  dev_free(C.nd_rpk);
  dev_free(C.nd_off);
  C = Coarse();
}

__global__ void nd_scatter_kernel(int nx, int ny, int nz, int lim, long nnodes, long bw, int masked,
                                  const double* __restrict__ st, double* __restrict__ B, int xs, long pad_a,
                                  long pad_b, long org_b);

void coarse_assemble(tp_ctx* c) {
  ProfScope ps(c, P_COARSE_FACTOR);
  Coarse& C = c->coarse;
  const int l = c->nl - 1;
  const Level& L = c->L[l];
  const bool nd = C.nd_ok && C.order >= 1 && C.solve_variant == 0;
  if (nd != C.nd_use) {  // captured loops hold the other form's solve launches
    C.nd_use = nd;
    graph_free(c);
  }
  cudaMemsetAsync(C.band, 0, C.band_elems * sizeof(double), c->s);
  const long work = L.nnodes * 14;
  if (nd)
    nd_scatter_kernel<<<grid_for(std::max(work, 32L), 256), 256, 0, c->s>>>(
        L.nx, L.ny, L.nz, L.lim, L.nnodes, C.bw, l >= 2 ? 1 : 0, c->st[l], C.band, C.nd_xs, C.nd_pad[0], C.nd_pad[1],
        C.nd_org[1]);
  else
    band_scatter_kernel<<<grid_for(work, 256), 256, 0, c->s>>>(L.nx, L.ny, L.nz, L.lim, L.nnodes, C.bw,
                                                               l >= 2 ? 1 : 0, c->st[l], C.band);
  TP_CHECK_LAUNCH(c, "band_scatter");
}

// The coarse factor came from a caller's matrix in the natural order
// (tp_coarse_factor_csr): the solves use the natural band until the next
// assembly from the grid.
void coarse_use_natural(tp_ctx* c) {
  Coarse& C = c->coarse;
  if (C.nd_use) {
    C.nd_use = false;
    graph_free(c);
  }
}

void coarse_graphs_free(tp_ctx* c) {
  Coarse& C = c->coarse;
  for (cudaGraphExec_t* g : {&C.graph_exec, &C.factor_exec, &C.nd_graph_exec, &C.nd_factor_exec})
    if (*g) {
      cudaGraphExecDestroy(*g);
      *g = nullptr;
    }
}

// ----------------------------------------------------------------------------
// Factor the nb x nb diagonal block held (updated, lower part, zero above the
// diagonal) in S with the 256 threads of the CTA: L into S and into the band,
// and into lblk_out (row-major 32x32, zero above the diagonal, followed by
// the 32 reciprocals 1/L(j,j)). A non-positive pivot sets *info (first
// column + 1) and is replaced by 1 so that the factor completes.
//
// This block lies on the factorisation's critical path (one per 32 columns).
// On this part an FP64 warp instruction holds its SM sub-partition's FP64
// unit for about 67 cycles whatever its active lanes, so the factor runs on
// four warps, one per sub-partition, each instruction with a full column of
// rows: warp w keeps columns w, w+4, ..., w+28 in registers (lane = row).
// The owner of column j forms its pivot (reciprocal square root, one
// multiply), writes L(:,j) to S and raises ready[j]; the others wait for the
// flag and update their columns. The owner of column j+1 updates that column
// first and defers its other updates until it has published pivot j+1, so
// the chain from pivot to pivot is one multiply-add, the reciprocal square
// root and one multiply. (No inverse is formed: the panel solve substitutes
// with L directly.) Waits on the flags are bounded; one that gives up sets
// kCoarseWaitGaveUp in *info.
constexpr int kFlagSpin = 1 << 20;

// A producer writes its column, fences, syncs its warp, then lane 0 raises
// the flag; a consumer polls the flag and fences before reading the column.
__device__ __forceinline__ void flag_wait(volatile int* flag, int* info) {
  int it = 0;
  while (!*flag && ++it < kFlagSpin) {
  }
  if (it >= kFlagSpin) atomicOr(info, kCoarseWaitGaveUp);
  __threadfence_block();
}

// The warp's columns are template parameters (W: the warp, FULL: nb == 32),
// so after unrolling every column test is resolved at compile time and no
// FP64 instruction is issued with all its lanes switched off (such an
// instruction still holds the FP64 unit).
template <typename V, int W, bool FULL>
__device__ __forceinline__ void diag_columns(V (*S)[NB + 1], V* rp, volatile int* ready, int nb, long k, int* info,
                                             int t) {
  V v[8];  // v[q] = A(t, W + 4q), lower part
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int c = W + 4 * q;
    v[q] = ((FULL || c < nb) && t >= c && (FULL || t < nb)) ? S[t][c] : V(0.0);
  }
#pragma unroll
  for (int j = 0; j < NB; j++) {
    if (!FULL && j >= nb) break;
    if ((j & 3) == W) {  // pivot j: column j (v[j >> 2]) has all its updates
      V d = vshfl(v[j >> 2], j);
      if (!vpos(d)) {
        if (t == 0) atomicCAS(info, 0, (int)(k + j + 1));
        d = V(1.0);
      }
      const V r = vrsqrt(d);
      const V l = (t >= j) ? v[j >> 2] * r : V(0.0);  // L(j,j) = d r
      v[j >> 2] = l;
      S[t][j] = l;
      if (t == 0) rp[j] = r;
      __threadfence_block();
      __syncwarp();
      if (t == 0) ready[j] = 1;
      if (j >= 1) {  // the updates from pivot j-1 deferred in the last step
        const V lt = S[t][j - 1];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int c = W + 4 * q;
          if (c > j && (FULL || c < nb)) v[q] -= lt * S[c][j - 1];
        }
      }
    } else {
      flag_wait(&ready[j], info);
    }
    const V lt = S[t][j];
    if (((j + 1) & 3) == W) {  // the next pivot's column first, the rest after it
      if (j + 1 < NB && (FULL || j + 1 < nb)) v[((j + 1) >> 2) & 7] -= lt * S[(j + 1) & (NB - 1)][j];
    } else {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int c = W + 4 * q;
        if (c > j && (FULL || c < nb)) v[q] -= lt * S[c][j];
      }
    }
  }
}

// named barrier 1 over warps 0-3 (orders their shared-memory accesses)
__device__ __forceinline__ void bar_warps0to3() { asm volatile("bar.sync 1, 128;\n" ::: "memory"); }

template <typename V, bool FULL>
__device__ __forceinline__ void diag_columns_of(int w, V (*S)[NB + 1], V* rp, volatile int* ready, int nb, long k,
                                                int* info, int t) {
  switch (w) {
    case 0: diag_columns<V, 0, FULL>(S, rp, ready, nb, k, info, t); break;
    case 1: diag_columns<V, 1, FULL>(S, rp, ready, nb, k, info, t); break;
    case 2: diag_columns<V, 2, FULL>(S, rp, ready, nb, k, info, t); break;
    default: diag_columns<V, 3, FULL>(S, rp, ready, nb, k, info, t); break;
  }
}

__device__ void factor_diag_block(double* __restrict__ B, long bw, long k, int nb, double (*S)[NB + 1],
                                  double* __restrict__ lblk_out, int* info) {
  __shared__ double rp[NB];       // 1/L(j,j)
  __shared__ volatile int ready[NB];
  const int tid = threadIdx.x, w = tid >> 5, t = tid & 31;
  if (tid < NB) ready[tid] = 0;
  __syncthreads();
  if (w < 4) {
    if (nb == NB)
      diag_columns_of<double, true>(w, S, rp, ready, nb, k, info, t);
    else
      diag_columns_of<double, false>(w, S, rp, ready, nb, k, info, t);
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int r = idx % NB, cc = idx / NB;
    const bool in = r < nb && cc < nb && r >= cc;
    if (in && r - cc <= bw) B[(k + cc) * bw + (k + r)] = S[r][cc];
    lblk_out[r * NB + cc] = in ? S[r][cc] : 0.0;
  }
  if (threadIdx.x < NB) lblk_out[NB * NB + threadIdx.x] = threadIdx.x < nb ? rp[threadIdx.x] : 0.0;
}

// the first diagonal block (later ones are factored inside syrk_panel_kernel)
__global__ void potrf_kernel(double* __restrict__ B, long bw, long k, int nb, double* __restrict__ linv, int* info) {
  __shared__ double S[NB][NB + 1];
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int r = idx % NB, cc = idx / NB;
    S[r][cc] = (r < nb && cc < nb && r >= cc) ? bget(B, bw, k + r, k + cc) : 0.0;
  }
  __syncthreads();
  factor_diag_block(B, bw, k, nb, S, linv, info);
}

// Panel rows R0..R1 of columns k..k+nb-1: solve X L_kk^T = A. One CTA of four
// warps per 32-row tile, laid out as the diagonal factor (lane = row, warp w
// holding columns w, w+4, ...): the owner of column p finishes
// X(:,p) = acc(:,p) / L(p,p) with one multiply and raises ready[p]; the
// others subtract X(:,p) L(c,p) from their columns c > p; the owner of p+1
// updates that column first and defers the rest.
constexpr int kTrsmThreads = 128;

// warp W's columns W, W+4, ... of the tile (compile-time, as in diag_columns)
// The tile A (row t, column c; 32 x 32 in shared memory) is solved in place;
// a finished column is published in A itself (its other entries live in the
// owner's registers until the end).
template <typename V, int W, bool FULL>
__device__ __forceinline__ void trsm_columns(V (*A)[NB + 1], int nb, const V (*Lb)[NB + 1], const V* rp,
                                             volatile int* ready, int* info, int t) {
  V (*X)[NB + 1] = A;
  V v[8];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int c = W + 4 * q;
    v[q] = (FULL || c < nb) ? A[t][c] : V(0.0);
  }
#pragma unroll
  for (int p = 0; p < NB; p++) {
    if (!FULL && p >= nb) break;
    if ((p & 3) == W) {
      const V x = v[p >> 2] * rp[p];
      v[p >> 2] = x;
      X[t][p] = x;
      __threadfence_block();
      __syncwarp();
      if (t == 0) ready[p] = 1;
      if (p >= 1) {  // the updates from column p-1 deferred in the last step
        const V xt = X[t][p - 1];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int c = W + 4 * q;
          if (c > p && (FULL || c < nb)) v[q] -= xt * Lb[c][p - 1];
        }
      }
    } else {
      flag_wait(&ready[p], info);
    }
    const V xt = X[t][p];
    if (((p + 1) & 3) == W) {
      if (p + 1 < NB && (FULL || p + 1 < nb)) v[((p + 1) >> 2) & 7] -= xt * Lb[(p + 1) & (NB - 1)][p];
    } else {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int c = W + 4 * q;
        if (c > p && (FULL || c < nb)) v[q] -= xt * Lb[c][p];
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int c = W + 4 * q;
    if (FULL || c < nb) A[t][c] = v[q];
  }
}

// solve the tile A in place with warps 0-3 (the caller syncs before and after)
template <typename V>
__device__ __forceinline__ void trsm_tile(V (*A)[NB + 1], int nb, const V (*Lb)[NB + 1], const V* rp,
                                          volatile int* ready, int* info) {
  const int w = threadIdx.x >> 5, t = threadIdx.x & 31;
  if (w >= 4) return;
  if (nb == NB) {
    switch (w) {
      case 0: trsm_columns<V, 0, true>(A, nb, Lb, rp, ready, info, t); break;
      case 1: trsm_columns<V, 1, true>(A, nb, Lb, rp, ready, info, t); break;
      case 2: trsm_columns<V, 2, true>(A, nb, Lb, rp, ready, info, t); break;
      default: trsm_columns<V, 3, true>(A, nb, Lb, rp, ready, info, t); break;
    }
  } else {
    switch (w) {
      case 0: trsm_columns<V, 0, false>(A, nb, Lb, rp, ready, info, t); break;
      case 1: trsm_columns<V, 1, false>(A, nb, Lb, rp, ready, info, t); break;
      case 2: trsm_columns<V, 2, false>(A, nb, Lb, rp, ready, info, t); break;
      default: trsm_columns<V, 3, false>(A, nb, Lb, rp, ready, info, t); break;
    }
  }
}

__global__ void __launch_bounds__(kTrsmThreads) trsm_kernel(double* __restrict__ B, long bw, long k, int nb, long R0,
                                                            long R1, const double* __restrict__ lblk, int* info) {
  __shared__ double Lb[NB][NB + 1], rp[NB], A[NB][NB + 1];
  __shared__ volatile int ready[NB];
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) Lb[idx / NB][idx % NB] = lblk[idx];
  const long r0 = R0 + (long)blockIdx.x * 32;
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int t = idx & 31, c = idx >> 5;  // consecutive threads: consecutive rows of one column
    const long r = r0 + t;
    A[t][c] = (r <= R1 && c < nb) ? bget(B, bw, r, k + c) : 0.0;
  }
  if (threadIdx.x < NB) {
    rp[threadIdx.x] = lblk[NB * NB + threadIdx.x];
    ready[threadIdx.x] = 0;
  }
  __syncthreads();
  trsm_tile(A, nb, Lb, rp, ready, info);
  __syncthreads();
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int t = idx & 31, c = idx >> 5;
    const long r = r0 + t;
    if (r <= R1 && c < nb && r - (k + c) <= bw) B[(k + c) * bw + r] = A[t][c];
  }
}

// A(r,c) -= sum_t L(r,k+t) L(c,k+t), R0 <= c <= r <= R1, over 32x32 tiles
// (tr, tc) of the trailing triangle. syrk_panel_kernel: the first tile column
// (tc = 0, the next panel), one tile per CTA; CTA 0 then factors tile (0,0),
// the next diagonal block, for the next step. syrk_rest_kernel: the tiles
// with tc >= 1, as quarter tiles (32 rows x 8 columns) dealt round-robin to
// two CTAs per SM, so every SM gets nearly the same FP64 work.
__global__ void syrk_panel_kernel(double* __restrict__ B, long bw, long n, long k, int nb, long R0, long R1,
                                  double* __restrict__ linv, int* info) {
  __shared__ double Lr[NB][33], Lc[NB][33];
  __shared__ double S[NB][NB + 1];
  const long tr = blockIdx.x;
  const long rb = R0 + tr * 32, cb = R0;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 256 threads
  for (int t = ty; t < NB; t += 8) {
    const long r = rb + tx, cc = cb + tx;
    Lr[t][tx] = (t < nb && r <= R1) ? bget(B, bw, r, k + t) : 0.0;
    Lc[t][tx] = (t < nb && cc <= R1) ? bget(B, bw, cc, k + t) : 0.0;
  }
  __syncthreads();
  const bool diag_next = tr == 0;
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

// lower-triangular tile b among those with tc >= 1 -> (tr, tc)
__device__ __forceinline__ void rest_tile(long b, long& tr, long& tc) {
  long q = (long)((sqrt(8.0 * (double)b + 1.0) - 1.0) / 2.0);
  while ((q + 1) * (q + 2) / 2 <= b) q++;
  while (q * (q + 1) / 2 > b) q--;
  tr = q + 1;
  tc = b - q * (q + 1) / 2 + 1;
}

constexpr int kRestStage = 2 * NB * 33;  // doubles per stage: the row and the column panel blocks
constexpr size_t kRestSmem = 2 * kRestStage * sizeof(double);

// stage the panel blocks of tile b (rows rb.., columns cb.. of columns k..k+nb-1)
__device__ __forceinline__ void rest_stage(const double* __restrict__ B, long bw, long k, int nb, long R0, long R1,
                                           long b, double* st) {
  long tr, tc;
  rest_tile(b, tr, tc);
  const long rb = R0 + tr * 32, cb = R0 + tc * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int t = ty; t < NB; t += 8) {
    const long r = rb + tx, cc = cb + tx;
    const bool ir = t < nb && r <= R1 && r - (k + t) <= bw, ic = t < nb && cc <= R1 && cc - (k + t) <= bw;
    cp_async8z(st + t * 33 + tx, ir ? B + (k + t) * bw + r : B, ir);
    cp_async8z(st + NB * 33 + t * 33 + tx, ic ? B + (k + t) * bw + cc : B, ic);
  }
}

__global__ void __launch_bounds__(256) syrk_rest_kernel(double* __restrict__ B, long bw, long k, int nb, long R0,
                                                        long R1, long ntiles) {
  extern __shared__ double sm[];  // two stages
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  long b = blockIdx.x;
  int s = 0;
  if (b < ntiles) rest_stage(B, bw, k, nb, R0, R1, b, sm);
  cp_commit();
  for (; b < ntiles; b += gridDim.x, s ^= 1) {
    if (b + gridDim.x < ntiles) rest_stage(B, bw, k, nb, R0, R1, b + gridDim.x, sm + (s ^ 1) * kRestStage);
    cp_commit();
    cp_wait<1>();
    __syncthreads();
    const double* Lr = sm + s * kRestStage;
    const double* Lc = Lr + NB * 33;
    long tr, tc;
    rest_tile(b, tr, tc);
    const long r = R0 + tr * 32 + tx;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int cy = ty + 8 * q;
      const long cc = R0 + tc * 32 + cy;
      double acc = 0.0;
#pragma unroll
      for (int t = 0; t < NB; t++) acc += Lr[t * 33 + tx] * Lc[t * 33 + cy];
      if (r <= R1 && cc <= R1 && cc <= r && r - cc <= bw) B[cc * bw + r] -= acc;
    }
    __syncthreads();  // every read of stage s is done before it is refilled
  }
  cp_wait<0>();
}

// ----------------------------------------------------------------------------
// The whole factorisation as ONE cooperative launch (one CTA per SM; two for
// the dissected order's launches, kPfSmem2). Tiles
// are the 32 x 32 blocks (I, J), I >= J, of the band; step k factors diagonal
// tile k. The first CTA runs the chain every step waits on: factor tile (k,k), solve
// the panel tile (k+1,k), apply step k's update to tile (k+1,k+1) -- which it
// keeps in shared memory and factors as step k+1. The other CTAs take, in
// step order and round-robin, the rest of each step: the panel tiles (I,k),
// I >= k+2, then the updates of the trailing band, column k+1 first (the
// next step's panel) and tile (k+2,k+2) right after it (the chain's next
// input). Each item waits, bounded, on flags for what it reads:
//   fdone[k]        diagonal tile k factored (and its 1/L(j,j) in rpk[k])
//   sdone[k][I-k]   panel tile (I,k) solved
//   tver[J][I-J]    tile (I,J) holds the updates of steps < tver
// A producer stores, syncs, fences and releases the flag; a consumer's
// thread 0 acquires it, and the band is read through L2 (ld.global.cg).
// Items only wait on items of earlier steps or on earlier items of their
// own step, and every CTA takes its items in order, so the waits end.
// A partial factor runs NT steps of a longer band: its last step's updates
// complete the trailing block (rows 32 NT ..), which is stored unfactored.
// Two factors can share one launch on disjoint CTAs (the dissected order).
struct PfArgs {
  double* B;
  long bw, n;
  int NT, TS;        // steps (diagonal tiles factored); row stride of sdone and tver
  double* rpk;       // [NT][NB]
  int* fdone;        // [NT]
  int* sdone;        // [NT][TS]
  int* tver;         // [tiles][TS], tiles = ceil(n / 32)
  const long* off;   // [NT+1]: bulk items before step k
  int* info;
  int* abort_flag;
  long spin;
  int cta0, ncta;    // the CTAs of this factor: cta0 (the chain) .. cta0 + ncta - 1
  int partial;       // 1: NT steps leave a trailing block (rows 32 NT ..) with all their
                     //    updates, unfactored; tile (NT, NT) is stored by the chain
};
// Shared memory of a factor CTA. The natural band's launch reserves more
// than half an SM's, so that each SM runs one CTA and its one chain has an SM
// to itself. The dissected order's two partial factors have chains of half
// the length and are bound by the other CTAs' tile items instead: their
// launch reserves what the double-single chain's buffers need, so two CTAs
// share an SM (the registers, 128 x 256 each, allow two) and one CTA's item
// overlaps the other's loads and waits (at 256x128x128: 20.5 -> 17.1 ms per
// assembly; the natural band with two CTAs per SM: 21.0 ms).
constexpr size_t kPfSmem = 120 * 1024;
constexpr size_t kPfSmem2 = 68 * 1024;
constexpr int kPfPerSm2 = 3;
// CTAs per SM the factor kernel's registers are sized for (pf_kernel's MB):
// 2 gives 128 per thread; 3 gives 80 (a few spilled bytes), so that three
// CTAs of the dissected double-single factor share an SM (16.4 -> 16.0 ms per
// assembly at 256x128x128; the natural band's chain slows down with the cap,
// 20.5 -> 23.2 ms, so its launch keeps 128)
template <typename V>
constexpr int kPfMinBlocksNd = std::is_same<V, Dsf>::value ? 3 : 2;

// last tile row of step k's panel (k itself: no panel)
__host__ __device__ __forceinline__ long pf_imax(long n, long bw, long k) {
  if (32 * (k + 1) >= n) return k;
  return lmin(n - 1, 32 * k + 31 + bw) / 32;
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// every thread of the CTA: wait until *flag >= target; false if the
// factorisation is being abandoned (this or another wait gave up)
__device__ bool pf_wait(const PfArgs& a, const int* flag, int target) {
  int ok = 1;
  if (threadIdx.x == 0) {
    for (long it = 0; ld_acquire(flag) < target; it++) {
      if (*(volatile int*)a.abort_flag) {
        ok = 0;
        break;
      }
      if (it >= a.spin) {
        atomicOr(a.info, kCoarseWaitGaveUp);
        atomicExch(a.abort_flag, 1);
        ok = 0;
        break;
      }
    }
  }
  return __syncthreads_and(ok) != 0;
}

// the CTA's stores happen before the barrier, the barrier before thread 0's
// release store at GPU scope, which is cumulative: a CTA that acquires the
// flag sees them all (no separate fence needed)
__device__ __forceinline__ void pf_release(int* flag, int v) {
  __syncthreads();
  if (threadIdx.x == 0) asm volatile("st.release.gpu.global.s32 [%0], %1;\n" ::"l"(flag), "r"(v) : "memory");
}

// tile (I, J) into A[r][c] (TR: A[c][r]); zero outside the matrix, above the
// diagonal and outside the band
template <bool TR, typename V>
__device__ void pf_load(const PfArgs& a, long I, long J, V (*A)[NB + 1]) {
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int r = idx & 31, c = idx >> 5;
    const long gr = 32 * I + r, gc = 32 * J + c;
    const bool in = gr < a.n && gr >= gc && gr - gc <= a.bw;
    const V v = ds_in<V>(in ? __ldcg(a.B + gc * a.bw + gr) : 0.0);
    if (TR)
      A[c][r] = v;
    else
      A[r][c] = v;
  }
}

template <typename V>
__device__ void pf_store(const PfArgs& a, long I, long J, const V (*A)[NB + 1]) {
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int r = idx & 31, c = idx >> 5;
    const long gr = 32 * I + r, gc = 32 * J + c;
    if (gr < a.n && gr >= gc && gr - gc <= a.bw) a.B[gc * a.bw + gr] = ds_out(A[r][c]);
  }
}

template <typename V>
__device__ void pf_chain(const PfArgs& a, double* smem) {
  V(*D)[NB + 1] = reinterpret_cast<V(*)[NB + 1]>(smem);                // diagonal tile, then L_kk
  V(*X)[NB + 1] = reinterpret_cast<V(*)[NB + 1]>(smem + NB * (NB + 1));  // panel tile (k+1,k)
  V* rp = reinterpret_cast<V*>(smem + 2 * NB * (NB + 1));
  volatile int* ready = reinterpret_cast<volatile int*>(rp + NB);
  const int w = threadIdx.x >> 5, t = threadIdx.x & 31;
  pf_load<false>(a, 0, 0, D);
  for (long k = 0; k < a.NT; k++) {
    const int nb = (int)lmin(NB, a.n - 32 * k);
    if (threadIdx.x < NB) ready[threadIdx.x] = 0;
    __syncthreads();
    if (w < 4) {
      if (nb == NB)
        diag_columns_of<V, true>(w, D, rp, ready, nb, 32 * k, a.info, t);
      else
        diag_columns_of<V, false>(w, D, rp, ready, nb, 32 * k, a.info, t);
    }
    __syncthreads();
    pf_store(a, k, k, D);
    if (threadIdx.x < NB) a.rpk[k * NB + threadIdx.x] = threadIdx.x < nb ? ds_out(rp[threadIdx.x]) : 0.0;
    pf_release(a.fdone + k, 1);
    if (pf_imax(a.n, a.bw, k) < k + 1) break;
    const bool prev = k >= 1 && k + 1 <= pf_imax(a.n, a.bw, k - 1);  // tiles (k+1, *) hold a step k-1 update
    // panel tile (k+1, k)
    if (prev && !pf_wait(a, a.tver + k * a.TS + 1, (int)k)) return;
    pf_load<false>(a, k + 1, k, X);
    if (threadIdx.x < NB) ready[threadIdx.x] = 0;
    __syncthreads();
    trsm_tile(X, NB, D, rp, ready, a.info);
    __syncthreads();
    pf_store(a, k + 1, k, X);
    pf_release(a.sdone + k * a.TS + 1, 1);
    // tile (k+1, k+1): step k-1's update (from the other CTAs), then step k's
    if (prev && !pf_wait(a, a.tver + (k + 1) * a.TS, (int)k)) return;
    pf_load<false>(a, k + 1, k + 1, D);
    __syncthreads();
    for (int e = threadIdx.x; e < NB * (NB + 1) / 2; e += blockDim.x) {  // the lower triangle, packed
      int r = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
      while ((r + 1) * (r + 2) / 2 <= e) r++;
      while (r * (r + 1) / 2 > e) r--;
      const int c = e - r * (r + 1) / 2;
      V s = V(0.0);
#pragma unroll
      for (int q = 0; q < NB; q++) s += X[r][q] * X[c][q];
      D[r][c] -= s;
    }
    __syncthreads();
  }
  if (a.partial && pf_imax(a.n, a.bw, a.NT - 1) >= a.NT) pf_store(a, a.NT, a.NT, D);  // D: tile (NT, NT)
}

// One work item of the non-chain CTAs: a panel tile (S: solve tile (I,k)
// with L_kk) or a tile update (U: tile (I,J) -= L(I,k) L(J,k)^T), with the
// flags it waits on.
struct PfItem {
  bool solve;
  long k, I, J;
  const int *f0, *f1, *f2;  // the first nf are used
  int t0, t1, t2;
  int nf;
  __device__ void add(const int* f, int tg) {
    if (nf == 0) f0 = f, t0 = tg;
    else if (nf == 1) f1 = f, t1 = tg;
    else f2 = f, t2 = tg;
    nf++;
  }
  __device__ const int* flag(int i) const { return i == 0 ? f0 : (i == 1 ? f1 : f2); }
  __device__ int target(int i) const { return i == 0 ? t0 : (i == 1 ? t1 : t2); }
};

// item g; k is the step of an earlier item and is advanced to g's step
__device__ void pf_item(const PfArgs& a, long g, long& k, PfItem& it) {
  while (a.off[k + 1] <= g) k++;
  const long idx = g - a.off[k];
  const long T = pf_imax(a.n, a.bw, k) - k;
  const long prev = k >= 1 ? pf_imax(a.n, a.bw, k - 1) : -1;  // tiles with I <= prev hold a step k-1 update
  it.k = k;
  it.nf = 0;
  if (idx < T - 1) {
    it.solve = true;
    it.I = k + 2 + idx;
    it.J = k;
    it.add(a.fdone + k, 1);
    if (it.I <= prev) it.add(a.tver + k * a.TS + (it.I - k), (int)k);
    return;
  }
  long u = idx - (T - 1);
  it.solve = false;
  if (u < T - 1) {
    it.I = k + 2 + u;
    it.J = k + 1;
  } else {
    u -= T - 1;
    // FP32 estimate (u < T (T + 1) / 2, a few hundred), corrected below: the
    // FP64 square root is a long sequence on this part's FP64 pipe
    long q = (long)((sqrtf(8.0f * (float)u + 1.0f) - 1.0f) * 0.5f);
    while ((q + 1) * (q + 2) / 2 <= u) q++;
    while (q * (q + 1) / 2 > u) q--;
    it.I = k + 2 + q;
    it.J = k + 2 + (u - q * (q + 1) / 2);
  }
  it.add(a.sdone + k * a.TS + (it.I - k), 1);
  if (it.J != it.I) it.add(a.sdone + k * a.TS + (it.J - k), 1);
  if (it.I <= prev) it.add(a.tver + it.J * a.TS + (it.I - it.J), (int)k);
}

// threads 0..nf-1 each watch one flag (bounded); false if the factorisation
// is being abandoned
__device__ bool pf_wait_item(const PfArgs& a, const PfItem& it) {
  int ok = 1;
  if (threadIdx.x < it.nf) {
    const int* f = it.flag(threadIdx.x);
    const int tg = it.target(threadIdx.x);
    for (long n = 0; ld_acquire(f) < tg; n++) {
      if (*(volatile int*)a.abort_flag) {
        ok = 0;
        break;
      }
      if (n >= a.spin) {
        atomicOr(a.info, kCoarseWaitGaveUp);
        atomicExch(a.abort_flag, 1);
        ok = 0;
        break;
      }
    }
  }
  return __syncthreads_and(ok) != 0;
}

// are the item's inputs ready now? (one look, no wait)
__device__ bool pf_ready(const PfItem& it) {
  int ok = 1;
  if (threadIdx.x < it.nf) ok = ld_acquire(it.flag(threadIdx.x)) >= it.target(threadIdx.x);
  return __syncthreads_and(ok) != 0;
}

__device__ __forceinline__ double pf_elem(const PfArgs& a, long I, long J, int r, int c) {
  const long gr = 32 * I + r, gc = 32 * J + c;
  return (gr < a.n && gr >= gc && gr - gc <= a.bw) ? __ldcg(a.B + gc * a.bw + gr) : 0.0;
}

// the item's inputs into registers: element idx = threadIdx.x + 256 m of the
// two tiles (S: tile (I,k) and L_kk; U: tiles (I,k) and (J,k)), and for S
// the reciprocal pivots
struct PfRegs {
  double p[4], q[4], r;
};

__device__ __forceinline__ void pf_fetch(const PfArgs& a, const PfItem& it, PfRegs& R) {
  const long qI = it.solve ? it.k : it.J;
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const int idx = threadIdx.x + 256 * m, r = idx & 31, c = idx >> 5;
    R.p[m] = pf_elem(a, it.I, it.k, r, c);
    R.q[m] = pf_elem(a, qI, it.k, r, c);
  }
  R.r = (it.solve && threadIdx.x < NB) ? __ldcg(a.rpk + it.k * NB + threadIdx.x) : 0.0;
}

// S: P, Q row-major (P solved in place); U: transposed, P[t][r] = L(32I + r, 32k + t)
template <typename V>
__device__ __forceinline__ void pf_put(const PfItem& it, const PfRegs& R, V (*P)[NB + 1], V (*Q)[NB + 1], V* rp,
                                       volatile int* ready) {
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const int idx = threadIdx.x + 256 * m, r = idx & 31, c = idx >> 5;
    const V p = ds_in<V>(R.p[m]), q = ds_in<V>(R.q[m]);
    if (it.solve) {
      P[r][c] = p;
      Q[r][c] = q;
    } else {
      P[c][r] = p;
      Q[c][r] = q;
    }
  }
  if (it.solve && threadIdx.x < NB) {
    rp[threadIdx.x] = ds_in<V>(R.r);
    ready[threadIdx.x] = 0;
  }
}

// The non-chain CTAs of the factor take items g = b - 1 + m (ncta - 1), b the
// CTA's place among the factor's ncta. While
// one item is computed, the next item's inputs are loaded into registers if
// its flags are already set (otherwise it waits for them when its turn comes).
template <typename V>
__device__ void pf_bulk(const PfArgs& a, double* smem) {
  V(*P)[NB + 1] = reinterpret_cast<V(*)[NB + 1]>(smem);
  V(*Q)[NB + 1] = reinterpret_cast<V(*)[NB + 1]>(smem + NB * (NB + 1));
  V* rp = reinterpret_cast<V*>(smem + 2 * NB * (NB + 1));
  volatile int* ready = reinterpret_cast<volatile int*>(rp + NB);
  const long nbulk = a.ncta - 1, total = a.off[a.NT];
  long g = (long)blockIdx.x - a.cta0 - 1, kk = 0;
  if (g >= total) return;
  PfItem cur, nxt;
  PfRegs R;
  pf_item(a, g, kk, cur);
  bool have = false;
  for (; g < total; g += nbulk) {
    if (!have) {
      if (!pf_wait_item(a, cur)) return;
      pf_fetch(a, cur, R);
    }
    pf_put(cur, R, P, Q, rp, ready);
    __syncthreads();
    have = false;
    if (g + nbulk < total) {
      pf_item(a, g + nbulk, kk, nxt);
      if (pf_ready(nxt)) {
        pf_fetch(a, nxt, R);  // in flight while this item is computed
        have = true;
      }
    }
    if (cur.solve) {
      trsm_tile(P, NB, Q, rp, ready, a.info);
      __syncthreads();
      pf_store(a, cur.I, cur.k, P);
      pf_release(a.sdone + cur.k * a.TS + (cur.I - cur.k), 1);
    } else {
      const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
      const long gr = 32 * cur.I + tx;
      double old[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {  // the tile's current values, loaded before the products
        const long gc = 32 * cur.J + ty + 8 * q;
        old[q] = (gr < a.n && gc <= gr && gr - gc <= a.bw) ? __ldcg(a.B + gc * a.bw + gr) : 0.0;
      }
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int cy = ty + 8 * q;
        const long gc = 32 * cur.J + cy;
        V s = V(0.0);
#pragma unroll
        for (int t = 0; t < NB; t++) s += P[t][tx] * Q[t][cy];
        if (gr < a.n && gc <= gr && gr - gc <= a.bw) a.B[gc * a.bw + gr] = ds_out(ds_in<V>(old[q]) - s);
      }
      pf_release(a.tver + cur.J * a.TS + (cur.I - cur.J), (int)cur.k + 1);
    }
    cur = nxt;
  }
}

// ----------------------------------------------------------------------------
// Double-single form of the single-launch factor. The schedule, the items and
// the flags are those of pf_chain / pf_bulk, and every entry goes through the
// same double-single operations in the same order, so the factor is the same
// bit for bit (up to the sign of exact zeros); the work is arranged for the
// latency of FP32 arithmetic instead of FP64 throughput. Measured on one CTA
// (cycles per 32 x 32 tile): a pivot hand-off through a shared-memory flag
// takes ~220 cycles, through a named barrier ~36; a double-single multiply,
// shuffle and multiply-add chain ~40; and code that runs once per tile and
// does not fit the instruction cache runs at a fraction of its warm speed
// (the unrolled column factor: 19k warm, 31k cold). Hence:
//  - the diagonal tile is factored by warps 0-3 with named-barrier hand-offs
//    and a loop over pivots whose slot indices are compile-time (13k);
//  - a panel tile is solved by four warps, each lane one row and every fourth
//    column, a column's solved entry reaching the row's other lanes by
//    shuffle (6.4k, no barrier per column); the chain's panel solve runs on
//    warps 4-7 one column behind the factor;
//  - fdone is released as soon as the factor is stored, ahead of the chain's
//    own panel solve, which waits on the other CTAs;
//  - tile products carry two outputs per f32x2 instruction (Dsf2);
//  - conversions to FP64 storage use integer operations plus one add (ds_to).

// wait of one warp (lane 0 polls, bounded); false if the factorisation is
// being abandoned. __syncwarp orders the warp's later loads after the acquire.
__device__ bool pf_wait_warp(const PfArgs& a, const int* flag, int target) {
  int ok = 1;
  if ((threadIdx.x & 31) == 0) {
    for (long it = 0; ld_acquire(flag) < target; it++) {
      if (*(volatile int*)a.abort_flag) {
        ok = 0;
        break;
      }
      if (it >= a.spin) {
        atomicOr(a.info, kCoarseWaitGaveUp);
        atomicExch(a.abort_flag, 1);
        ok = 0;
        break;
      }
    }
  }
  __syncwarp();
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// tile (I, J) into A[r][c] as pairs (zero outside the matrix, above the
// diagonal and outside the band) by nthr threads, thread i of them
__device__ __forceinline__ void pf_load_ds(const PfArgs& a, long I, long J, Dsf (*A)[NB + 1], int i, int nthr) {
  for (int idx = i; idx < NB * NB; idx += nthr) {
    const int r = idx & 31, c = idx >> 5;
    const long gr = 32 * I + r, gc = 32 * J + c;
    const bool in = gr < a.n && gr >= gc && gr - gc <= a.bw;
    A[r][c] = ds_from(in ? __ldcg(a.B + gc * a.bw + gr) : 0.0);
  }
}

// Operand layouts of the tile product s(r, c) = sum_t a(r, t) b(c, t), one
// CTA of 256 threads, thread (r = lane, warp ty) computing c = ty + 8q:
//   PA[t][r] = (h, h, -h, -h), PL[t][r] = (-l, -l)      a(r, t)
//   QB[t][c & 7][c >> 4] = (h(c0), h(c0 + 8), l(c0), l(c0 + 8)),
//                          c0 = (c & 7) + 16 (c >> 4)    b(c, t)
__device__ __forceinline__ void put_a(float4* PA, float2* PL, int t, int r, Dsf x) {
  PA[t * 32 + r] = make_float4(x.h, x.h, -x.h, -x.h);
  PL[t * 32 + r] = make_float2(-x.l, -x.l);
}
__device__ __forceinline__ void put_b(float4* QB, int t, int c, Dsf x) {
  float* q = reinterpret_cast<float*>(QB + (t * 8 + (c & 7)) * 2 + (c >> 4));
  const int half = (c >> 3) & 1;
  q[half] = x.h;
  q[2 + half] = x.l;
}

// s[q] = sum over t = 0..31, in order, of a(r, t) * b(ty + 8q, t), each as
// Dsf's  s += a * b  from s = 0
__device__ __forceinline__ void pf_products_ds(const float4* PA, const float2* PL, const float4* QB, Dsf s[4]) {
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  Dsf2 s01 = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)}, s23 = s01;
#pragma unroll 8
  for (int t = 0; t < NB; t++) {
    const float4 pa = PA[t * 32 + tx];
    const float2 pl = PL[t * 32 + tx];
    const float4 q0 = QB[(t * 8 + ty) * 2], q1 = QB[(t * 8 + ty) * 2 + 1];
    const float2 ah = make_float2(pa.x, pa.y), nah = make_float2(pa.z, pa.w);
    ds2_add_prod(s01, ah, nah, pl, make_float2(q0.x, q0.y), make_float2(q0.z, q0.w));
    ds2_add_prod(s23, ah, nah, pl, make_float2(q1.x, q1.y), make_float2(q1.z, q1.w));
  }
  s[0] = Dsf(s01.h.x, s01.l.x);
  s[1] = Dsf(s01.h.y, s01.l.y);
  s[2] = Dsf(s23.h.x, s23.l.x);
  s[3] = Dsf(s23.h.y, s23.l.y);
}

// ready[j] == epoch (the step's number + 1, so nothing needs resetting
// between steps), polled at most kFlagSpin times; a wait that gives up sets
// kCoarseWaitGaveUp in *info.
__device__ __forceinline__ void flag_wait_epoch(volatile int* flag, int epoch, int* info) {
  int it = 0;
  while (*flag != epoch && ++it < kFlagSpin) {
  }
  if (it >= kFlagSpin) atomicOr(info, kCoarseWaitGaveUp);
  __threadfence_block();
}

// Factor of the diagonal tile by warps 0-3: warp W owns columns W + 4q
// (v[q], lane t = row t). The owner of pivot j forms d = A(j, j) (a
// non-positive one sets *info and is replaced by 1), r = 1/sqrt(d),
// L(t, j) = A(t, j) r, writes Lcol[j][t] = L(t, j) and rp[j] = r, and
// arrives on named barrier 3 + (j & 3), on which the other three warps
// wait; then every warp
// takes L(t, j) L(c, j) off its columns c > j. The loop over the four
// pivots of a slot group is not unrolled and the group's slot is a
// compile-time index, so the code is small and each step's updates form one
// block the compiler can interleave. (Barrier 3 + (j & 3) is reused at pivot
// j + 4 only after all four warps have passed pivots j + 1 .. j + 3, each of
// which they reach through barrier j's phase.)
__device__ __forceinline__ void diag_cols_ds(const Dsf (*Dt)[NB + 1], Dsf (*Lcol)[NB + 1], Dsf* rp, int nb, long k0,
                                             int* info) {
  const int W = threadIdx.x >> 5, t = threadIdx.x & 31;
  Dsf v[8];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int c = W + 4 * q;
    v[q] = (t >= c && c < nb && t < nb) ? Dt[t][c] : Dsf(0.f);
  }
#pragma unroll
  for (int qj = 0; qj < 8; qj++) {
#pragma unroll 1
    for (int jj = 0; jj < 4; jj++) {
      const int j = 4 * qj + jj;
      if (j >= nb) break;
      if (jj == W) {
        Dsf d = ds_shfl(v[qj], j);
        if (!vpos(d)) {
          if (t == 0) atomicCAS(info, 0, (int)(k0 + j + 1));
          d = Dsf(1.f);
        }
        const Dsf r = ds_rsqrt(d);
        const Dsf l = (t >= j) ? v[qj] * r : Dsf(0.f);
        Lcol[j][t] = l;
        if (t == 0) rp[j] = r;
        asm volatile("bar.arrive %0, 128;\n" ::"r"(3 + jj) : "memory");
      } else {
        asm volatile("bar.sync %0, 128;\n" ::"r"(3 + jj) : "memory");
      }
      const Dsf lt = Lcol[j][t];
      const Dsf y = v[qj] - lt * Lcol[j][W + 4 * qj];
      v[qj] = ds_sel(W > jj, y, v[qj]);
#pragma unroll
      for (int q = qj + 1; q < 8; q++) v[q] -= lt * Lcol[j][W + 4 * q];
    }
  }
}

// Panel tile solve X L_kk^T = A by the CTA's eight warps: lane (row
// r = 4w + (lane & 3), g = lane >> 2) holds v[q] = entry (r, g + 8q). Column p
// is finished by the lane of group p & 7 (x = v / L(p, p), as v * rp[p]) and
// reaches the row's other lanes (lane & 3) + 4g by shuffle; each lane then
// takes x L(c, p) off its columns c > p. L(c, p) = LT ? Lm[p][c] : Lm[c][p].
// Unrolled: every slot index and column test is resolved at compile time
// (about 2.5k instructions, run once per panel tile); with two warps per
// scheduler the column chain (multiply, shuffle, multiply-add) overlaps the
// other columns' updates.
template <bool LT>
__device__ __forceinline__ void trsm_rows_ds(const Dsf (*Lm)[NB + 1], const Dsf* rp, Dsf v[4]) {
  const int lane = threadIdx.x & 31, rl = lane & 3, g = lane >> 2;
#pragma unroll
  for (int p = 0; p < NB; p++) {
    const int qp = p >> 3;
    const Dsf x = v[qp] * rp[p];
    v[qp] = ds_sel(g == (p & 7), x, v[qp]);
    const Dsf xt = ds_shfl(x, rl + 4 * (p & 7));
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (8 * q + 7 <= p) continue;  // columns all finished
      const int c = g + 8 * q;
      const Dsf y = v[q] - xt * (LT ? Lm[p][c] : Lm[c][p]);
      v[q] = 8 * q > p ? y : ds_sel(c > p, y, v[q]);
    }
  }
}

// smem offsets (in doubles) of the chain's and the other CTAs' buffers
constexpr int kTile = NB * (NB + 1);  // a 32 x 33 tile of pairs
constexpr int kPA = 2 * NB * NB, kPL = NB * NB;  // PA, PL; then QB (NB * NB doubles)
static_assert((4 * kTile + NB + kPA + kPL + NB * NB) * sizeof(double) <= kPfSmem2, "chain buffers");

// The chain CTA, step k: warps 0-3 factor tile (k,k), store it and release
// fdone[k]; meanwhile warps 4-7 wait for and load the panel tile (k+1,k) and
// start loading tile (k+1,k+1). Then all eight warps solve the panel tile,
// store it, release sdone and lay it out as the product's operands, and
// apply (k+1,k+1) -= X X^T, which the next step factors.
__device__ void pf_chain_ds(const PfArgs& a, double* smem) {
  Dsf(*Lcol)[NB + 1] = reinterpret_cast<Dsf(*)[NB + 1]>(smem + 2 * kTile);
  Dsf(*Xa)[NB + 1] = reinterpret_cast<Dsf(*)[NB + 1]>(smem + 3 * kTile);
  Dsf* rp = reinterpret_cast<Dsf*>(smem + 4 * kTile);
  float4* PA = reinterpret_cast<float4*>(smem + 4 * kTile + NB);
  float2* PL = reinterpret_cast<float2*>(smem + 4 * kTile + NB + kPA);
  float4* QB = reinterpret_cast<float4*>(smem + 4 * kTile + NB + kPA + kPL);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  pf_load_ds(a, 0, 0, reinterpret_cast<Dsf(*)[NB + 1]>(smem), threadIdx.x, blockDim.x);
  __syncthreads();
  for (long k = 0; k < a.NT; k++) {
    Dsf(*D)[NB + 1] = reinterpret_cast<Dsf(*)[NB + 1]>(smem + (k & 1) * kTile);  // tiles (k,k), (k+1,k+1)
    Dsf(*Dn)[NB + 1] = reinterpret_cast<Dsf(*)[NB + 1]>(smem + ((k + 1) & 1) * kTile);
    const int nb = (int)lmin(NB, a.n - 32 * k);
    const bool more = pf_imax(a.n, a.bw, k) >= k + 1;
    const bool prev = k >= 1 && k + 1 <= pf_imax(a.n, a.bw, k - 1);  // tiles (k+1, *) hold a step k-1 update
    int ok = 1;
    double dn[8];  // entries i4 + 128 m of tile (k+1, k+1), in flight during the panel solve
    if (w < 4) {
      diag_cols_ds(D, Lcol, rp, nb, 32 * k, a.info);
      bar_warps0to3();
      for (int idx = threadIdx.x; idx < NB * NB; idx += 128) {  // L_kk, lower part
        const int r = idx & 31, c = idx >> 5;
        const long gr = 32 * k + r, gc = 32 * k + c;
        if (gr < a.n && gr >= gc && gr - gc <= a.bw) a.B[gc * a.bw + gr] = ds_to(Lcol[c][r]);
      }
      if (threadIdx.x < NB) a.rpk[k * NB + threadIdx.x] = threadIdx.x < nb ? ds_to(rp[threadIdx.x]) : 0.0;
      // the four warps' stores happen before the barrier, the barrier before
      // thread 0's release (cumulative): the other CTAs' panel solves of step k
      // start now, not after this CTA's own panel solve
      bar_warps0to3();
      if (threadIdx.x == 0) asm volatile("st.release.gpu.global.s32 [%0], %1;\n" ::"l"(a.fdone + k), "r"(1) : "memory");
    } else if (more) {
      const int i4 = threadIdx.x - 128;
      if (prev) ok = pf_wait_warp(a, a.tver + k * a.TS + 1, (int)k);
      if (ok) pf_load_ds(a, k + 1, k, Xa, i4, 128);
      if (ok && prev) ok = pf_wait_warp(a, a.tver + (k + 1) * a.TS, (int)k);
#pragma unroll
      for (int m = 0; m < 8; m++) {
        const int idx = i4 + 128 * m, r = idx & 31, c = idx >> 5;
        const long gr = 32 * (k + 1) + r, gc = 32 * (k + 1) + c;
        dn[m] = (ok && gr < a.n && gr >= gc && gr - gc <= a.bw) ? __ldcg(a.B + gc * a.bw + gr) : 0.0;
      }
    }
    if (!__syncthreads_and(ok)) return;
    if (!more) break;
    {  // panel tile (k+1, k): into the band and into the product's operands
      const int r = 4 * w + (lane & 3), g = lane >> 2;
      Dsf v[4];
#pragma unroll
      for (int q = 0; q < 4; q++) v[q] = Xa[r][g + 8 * q];
      trsm_rows_ds<true>(Lcol, rp, v);
      const long gr = 32 * (k + 1) + r;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int c = g + 8 * q;
        const long gc = 32 * k + c;
        if (gr < a.n && gr - gc <= a.bw) a.B[gc * a.bw + gr] = ds_to(v[q]);
        put_a(PA, PL, c, r, v[q]);
        put_b(QB, c, r, v[q]);
      }
    }
    if (w >= 4) {
#pragma unroll
      for (int m = 0; m < 8; m++) {
        const int idx = threadIdx.x - 128 + 128 * m;
        Dn[idx & 31][idx >> 5] = ds_from(dn[m]);
      }
    }
    // the stores of the panel tile happen before the barrier, the barrier
    // before thread 0's release (cumulative)
    __syncthreads();
    if (threadIdx.x == 0) asm volatile("st.release.gpu.global.s32 [%0], %1;\n" ::"l"(a.sdone + k * a.TS + 1), "r"(1) : "memory");
    // tile (k+1, k+1) -= X X^T, lower part
    Dsf s[4];
    pf_products_ds(PA, PL, QB, s);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int c = w + 8 * q;
      if (lane >= c) Dn[lane][c] -= s[q];
    }
    __syncthreads();
  }
  if (a.partial && pf_imax(a.n, a.bw, a.NT - 1) >= a.NT) {  // tile (NT, NT), updated by the last step
    const Dsf(*Dl)[NB + 1] = reinterpret_cast<const Dsf(*)[NB + 1]>(smem + (a.NT & 1) * kTile);
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
      const int r = idx & 31, c = idx >> 5;
      const long gr = 32L * a.NT + r, gc = 32L * a.NT + c;
      if (gr < a.n && gr >= gc) a.B[gc * a.bw + gr] = ds_to(Dl[r][c]);
    }
  }
}

__device__ void pf_bulk_ds(const PfArgs& a, double* smem) {
  Dsf(*P)[NB + 1] = reinterpret_cast<Dsf(*)[NB + 1]>(smem);
  Dsf(*Q)[NB + 1] = reinterpret_cast<Dsf(*)[NB + 1]>(smem + kTile);
  Dsf* rp = reinterpret_cast<Dsf*>(smem + 2 * kTile);
  float4* PA = reinterpret_cast<float4*>(smem + 2 * kTile + NB);
  float2* PL = reinterpret_cast<float2*>(smem + 2 * kTile + NB + kPA);
  float4* QB = reinterpret_cast<float4*>(smem + 2 * kTile + NB + kPA + kPL);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long nbulk = a.ncta - 1, total = a.off[a.NT];
  long g = (long)blockIdx.x - a.cta0 - 1, kk = 0;
  if (g >= total) return;
  PfItem cur, nxt;
  PfRegs R;
  pf_item(a, g, kk, cur);
  bool have = false;
  for (; g < total; g += nbulk) {
    if (!have) {
      if (!pf_wait_item(a, cur)) return;
      pf_fetch(a, cur, R);
    }
    // the next item's flags, probed now (one look, no wait) so that the
    // acquire's round trip overlaps the layout of this item's operands
    const bool more = g + nbulk < total;
    int okn = 0;
    if (more) {
      pf_item(a, g + nbulk, kk, nxt);
      okn = threadIdx.x < nxt.nf ? ld_acquire(nxt.flag(threadIdx.x)) >= nxt.target(threadIdx.x) : 1;
    }
#pragma unroll
    for (int m = 0; m < 4; m++) {  // S: tile (I,k) and L_kk row-major; U: the product's operands
      const int idx = threadIdx.x + 256 * m, r = idx & 31, c = idx >> 5;
      const Dsf p = ds_from(R.p[m]), q = ds_from(R.q[m]);
      if (cur.solve) {
        P[r][c] = p;
        Q[r][c] = q;
      } else {
        put_a(PA, PL, c, r, p);
        put_b(QB, c, r, q);
      }
    }
    if (cur.solve && threadIdx.x < NB) rp[threadIdx.x] = ds_from(R.r);
    have = __syncthreads_and(okn) != 0;  // false when there is no next item
    if (have) pf_fetch(a, nxt, R);       // in flight while this item is computed
    if (cur.solve) {
      {
        const int r = 4 * w + (lane & 3), gq = lane >> 2;
        Dsf v[4];
#pragma unroll
        for (int q = 0; q < 4; q++) v[q] = P[r][gq + 8 * q];
        trsm_rows_ds<false>(Q, rp, v);
        const long gr = 32 * cur.I + r;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const long gc = 32 * cur.k + gq + 8 * q;
          if (gr < a.n && gr - gc <= a.bw) a.B[gc * a.bw + gr] = ds_to(v[q]);
        }
      }
      pf_release(a.sdone + cur.k * a.TS + (cur.I - cur.k), 1);
    } else {
      const long gr = 32 * cur.I + lane;
      double old[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {  // the tile's current values, loaded before the products
        const long gc = 32 * cur.J + w + 8 * q;
        old[q] = (gr < a.n && gc <= gr && gr - gc <= a.bw) ? __ldcg(a.B + gc * a.bw + gr) : 0.0;
      }
      Dsf s[4];
      pf_products_ds(PA, PL, QB, s);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const long gc = 32 * cur.J + w + 8 * q;
        if (gr < a.n && gc <= gr && gr - gc <= a.bw) a.B[gc * a.bw + gr] = ds_to(ds_from(old[q]) - s[q]);
      }
      pf_release(a.tver + cur.J * a.TS + (cur.I - cur.J), (int)cur.k + 1);
    }
    cur = nxt;
  }
}

template <typename V>
__device__ __forceinline__ void pf_run(const PfArgs& a, double* sm) {
  if constexpr (std::is_same<V, Dsf>::value) {
    if ((int)blockIdx.x == a.cta0)
      pf_chain_ds(a, sm);
    else
      pf_bulk_ds(a, sm);
  } else {
    if ((int)blockIdx.x == a.cta0)
      pf_chain<V>(a, sm);
    else
      pf_bulk<V>(a, sm);
  }
}

// one factor (a1.cta0 >= gridDim.x) or two independent ones, the CTAs below
// a1.cta0 on a0 and the others on a1
template <typename V, int MB>
__global__ void __launch_bounds__(256, MB) pf_kernel(PfArgs a0, PfArgs a1) {
  extern __shared__ double sm[];
  if ((int)blockIdx.x < a1.cta0)
    pf_run<V>(a0, sm);
  else
    pf_run<V>(a1, sm);
}

// Inverse of each diagonal nbs x nbs block of L, one CTA per (block, 32-column
// chunk): the chunk's columns X of L_bb^{-1} are found by blocked forward
// substitution over 32-row chunks R,
//   acc = E_R - sum_{S<R} L_RS X_S,    X_R = L_RR^{-1} acc (substitution),
// with X kept in shared memory. Writes D (row-major) and D^T (row-major).
// The tiles L_RS of a row chunk are loaded into registers one tile ahead, so
// a tile's product does not wait on its load. blockIdx.x is the block and
// blockIdx.y the chunk: CTAs go out chunk by chunk, the heaviest (chunk 0,
// nR(nR-1)/2 tile products) first, so the last wave holds the lightest. The
// blocks of up to three bands (the dissected order's views) go in one launch:
// a launch takes as long as its heaviest CTAs, whatever its block count.
constexpr int kDinvThreads = 256;

struct DinvBands {
  const double* B[3];  // the bands (origin at their first row)
  long n[3];           // rows in blocks
  int blk0[3];         // first block of each band; blocks are numbered across the bands
};

template <typename V>
__global__ void __launch_bounds__(kDinvThreads)
    dinv_kernel(DinvBands bands, long bw, int nbs, double* __restrict__ D, double* __restrict__ DT) {
  extern __shared__ double smem_d[];
  V* X = reinterpret_cast<V*>(smem_d);  // nbs x 33
  V* Lt = X + (long)nbs * 33;           // 32 x 33
  V* Acc = Lt + 32 * 33;                // the chunk's 32 reciprocal pivots
  const int blk = blockIdx.x, cc = blockIdx.y, tid = threadIdx.x;
  const int v = blk >= bands.blk0[2] ? 2 : (blk >= bands.blk0[1] ? 1 : 0);
  const double* B = v == 2 ? bands.B[2] : (v == 1 ? bands.B[1] : bands.B[0]);
  const long n = v == 2 ? bands.n[2] : (v == 1 ? bands.n[1] : bands.n[0]);
  const long b0 = (long)(blk - (v == 2 ? bands.blk0[2] : (v == 1 ? bands.blk0[1] : 0))) * nbs;
  const int s = (int)lmin((long)nbs, n - b0);
  const int j0 = cc * 32;
  double* Db = D + (long)blk * nbs * nbs;
  double* DTb = DT + (long)blk * nbs * nbs;
  const int a = tid >> 3, q0 = (tid & 7) * 4;
  const int nR = (s + 31) / 32;
  for (int R = cc; R < nR; R++) {
    V acc[4];
#pragma unroll
    for (int q = 0; q < 4; q++) acc[q] = V((R == cc && a == q0 + q) ? 1.0f : 0.0f);
    // tile L_RS, element idx = tid + 256 m at (ra, cs) = (idx & 31, idx >> 5)
    auto load_tile = [&](int S, double* v) {
#pragma unroll
      for (int m = 0; m < 4; m++) {
        const int idx = tid + kDinvThreads * m, ra = idx & 31, cs = idx >> 5;
        const long r = b0 + R * 32 + ra, col = b0 + S * 32 + cs;
        v[m] = (R * 32 + ra < s) ? bget(B, bw, r, col) : 0.0;
      }
    };
    double nxt[4];
    if (cc < R) load_tile(cc, nxt);
    for (int S = cc; S < R; S++) {
#pragma unroll
      for (int m = 0; m < 4; m++) {
        const int idx = tid + kDinvThreads * m;
        Lt[(idx & 31) * 33 + (idx >> 5)] = ds_in<V>(nxt[m]);
      }
      __syncthreads();
      if (S + 1 < R) load_tile(S + 1, nxt);  // in flight during this tile's product
#pragma unroll 4
      for (int t = 0; t < 32; t++) {
        const V l = Lt[a * 33 + t];
        const V* xr = X + (long)(S * 32 + t) * 33 + q0;
#pragma unroll
        for (int q = 0; q < 4; q++) acc[q] -= l * xr[q];
      }
      __syncthreads();
    }
    for (int idx = tid; idx < 1024; idx += kDinvThreads) {
      const int ra = idx & 31, cs = idx >> 5;
      const long r = b0 + R * 32 + ra, col = b0 + R * 32 + cs;
      Lt[ra * 33 + cs] = ds_in<V>((R * 32 + ra < s && R * 32 + cs < s && ra >= cs) ? bget(B, bw, r, col) : 0.0);
    }
    __syncthreads();
    if (tid < 32) {  // reciprocal pivots of the chunk (rows past s give zero rows of X)
      Acc[tid] = R * 32 + tid < s ? vrcp(Lt[tid * 33 + tid]) : V(0.0f);
    }
    __syncthreads();
    // X_R = L_RR^{-1} acc, right-looking over all warps: row t is finished
    // by its 8 threads, then every row below subtracts L(a,t) X(t,:)
    for (int t = 0; t < 32; t++) {
      if (a == t) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
          acc[q] *= Acc[t];
          X[(long)(R * 32 + t) * 33 + q0 + q] = acc[q];
        }
      }
      __syncthreads();
      if (a > t) {
        const V l = Lt[a * 33 + t];
        const V* xr = X + (long)(R * 32 + t) * 33 + q0;
#pragma unroll
        for (int q = 0; q < 4; q++) acc[q] -= l * xr[q];
      }
    }
    __syncthreads();
  }
  // D[r][j0+col] for r in [0, nbs): zero above the diagonal chunk and past s
  for (int idx = tid; idx < nbs * 32; idx += kDinvThreads) {
    const int r = idx >> 5, col = idx & 31;
    const double v = (r >= j0 && r < s && j0 + col < s) ? ds_out(X[(long)r * 33 + col]) : 0.0;
    Db[(long)r * nbs + j0 + col] = v;
  }
  for (int idx = tid; idx < nbs * 32; idx += kDinvThreads) {
    const int col = idx / nbs, r = idx % nbs;
    const double v = (r >= j0 && r < s && j0 + col < s) ? ds_out(X[(long)r * 33 + col]) : 0.0;
    DTb[(long)(j0 + col) * nbs + r] = v;
  }
}

// row-major copy of the band rows of each block left of the block:
// Lrow[blk][i][t] = L(b0 + i, b0 - bw + t), b0 = base + blk nbs, zero
// outside the band or the matrix
__global__ void lrow_kernel(const double* __restrict__ B, long bw, long n, int nbs, double* __restrict__ Lrow,
                            long base = 0) {
  __shared__ double tile[32][33];
  const int blk = blockIdx.z;
  const long b0 = base + (long)blk * nbs;
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

// ----------------------------------------------------------------------------
// Nested dissection of the coarsest grid, one level (Coarse::nd_*). The node
// plane xs separates part A (planes < xs) from part B (planes > xs); no
// entry of the operator couples A and B. In the composite order
//   view A: pad_a identity rows, A in natural order, then S (natural order)
//   view B: pad_b identity rows, B in mirrored plane order (plane nx-1 first,
//           so that the plane next to S comes last), then S
//   view S: S
// each of A and B is a band of the natural half bandwidth with S as a
// trailing block. Eliminating A's and B's own rows (the partial factors)
// leaves in the trailing blocks  S_A = K_SS - L_SA L_SA^T  and
// -L_SB L_SB^T, whose sum is the Schur complement K_SS - K_SA K_AA^-1 K_AS
// - K_SB K_BB^-1 K_BS that view S then factors. The two partial factors are
// independent, so they run at the same time on halves of the grid, each
// with its own 32-column chain (half the natural chain's length).
//   solve: y_A = L_A^-1 b_A, y_B = L_B^-1 b_B; y_S = L_S^-1 (b_S - L_SA y_A
//   - L_SB y_B); x_S = L_S^-T y_S; x_A = L_A^-T (y_A - L_SA^T x_S), x_B alike.

// position of DOF (node (p, k, j), component c), p >= xs, in view B
__host__ __device__ __forceinline__ long nd_pos_b(int p, int k, int j, int c, int nx, int ny, int nz, long pad_b) {
  return pad_b + 3L * (((long)(nx - 1 - p) * nz + k) * ny + j) + c;
}

// the entries band_scatter_kernel writes, placed in the views: a pair of
// nodes in planes <= xs goes to view A (natural order, after pad_a rows; the
// S x S block only there), any other pair to view B (mirrored order, its
// S x S block left zero); then the pads' unit diagonals
__global__ void nd_scatter_kernel(int nx, int ny, int nz, int lim, long nnodes, long bw, int masked,
                                  const double* __restrict__ st, double* __restrict__ B, int xs, long pad_a,
                                  long pad_b, long org_b) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t < pad_a) B[t * bw + t] = 1.0;
  if (t < pad_b) B[(org_b + t) * bw + org_b + t] = 1.0;
  if (t >= nnodes * 14) return;
  const long n = t % nnodes;
  const int m = (int)(t / nnodes);  // 0..13
  const int j = n % ny;
  const int k = (n / ny) % nz;
  const int i = n / ((long)ny * nz);
  const int mx = m / 9 - 1, mz = (m / 3) % 3 - 1, my = m % 3 - 1;
  const int mi = i + mx, mk = k + mz, mj = j + my;
  if (mi < 0 || mi >= nx || mk < 0 || mk >= nz || mj < 0 || mj >= ny) return;
  const long nm = ((long)mi * nz + mk) * ny + mj;
  const bool nfix = i == 0 && (j < lim || j >= ny - lim);
  const bool mfix = mi == 0 && (mj < lim || mj >= ny - lim);
  for (int c = 0; c < 3; c++)
    for (int d = 0; d < 3; d++) {
      const long r = 3 * n + c, col = 3 * nm + d;
      if (col > r || r - col > bw) continue;
      double v;
      if (nfix)
        v = (r == col) ? 1.0 : 0.0;
      else if (masked && m != 13 && mfix)
        v = 0.0;
      else
        v = (m == 13) ? st[(long)(3 * c + d) * nnodes + n] : st[((long)(13 - m) * 9 + 3 * d + c) * nnodes + nm];
      if (i <= xs) {  // mi <= i: both nodes in A or S
        B[(col + pad_a) * bw + r + pad_a] = v;
      } else {        // i > xs, mi >= i - 1 >= xs: both in B or S
        const long pr = nd_pos_b(i, k, j, c, nx, ny, nz, pad_b), pc = nd_pos_b(mi, mk, mj, d, nx, ny, nz, pad_b);
        const long hi = lmax(pr, pc), lo = lmin(pr, pc);
        if (hi - lo <= bw) B[(org_b + lo) * bw + org_b + hi] = v;
      }
    }
}

// view S (lower part) = the trailing blocks of views A and B, summed
__global__ void nd_schur_kernel(double* __restrict__ B, long bw, long ns, long own_a, long org_b, long own_b,
                                long org_s) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= ns * ns) return;
  const long i = t % ns, j = t / ns;
  if (i < j) return;
  const double a = B[(own_a + j) * bw + own_a + i];
  const double b = B[(org_b + own_b + j) * bw + org_b + own_b + i];
  B[(org_s + j) * bw + org_s + i] = a + b;
}

// composite <- natural (pads and tails zero), per column
__global__ void nd_gather_kernel(const int* __restrict__ map, long ntot, const double* __restrict__ src, long n,
                                 double* __restrict__ dst, int nr) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= ntot * nr) return;
  const long v = t / ntot, i = t % ntot;
  const int m = map[i];
  dst[t] = m >= 0 ? src[v * n + m] : 0.0;
}

// natural <- composite, per column
__global__ void nd_scatter_out_kernel(const int* __restrict__ map, long ntot, const double* __restrict__ src,
                                      long n, double* __restrict__ dst, int nr) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= ntot * nr) return;
  const long v = t / ntot, i = t % ntot;
  const int m = map[i];
  if (m >= 0) dst[v * n + m] = src[t];
}

// b_S -= L_SA y_A + L_SB y_B, one CTA of kCoupleThreads per row of S; the
// tails' rows are row-major (tail[s][e] = L(own + s, own - bw + e)). Thread
// t sums positions t, t + 128, ... of each tail in order, each warp in a
// fixed tree, then the four warps in order.
constexpr int kCoupleThreads = 128;
template <int NR>
__global__ void __launch_bounds__(kCoupleThreads)
    nd_couple_kernel(const double* __restrict__ tail_a, const double* __restrict__ tail_b, long bw, long ns,
                     long own_a, long org_a, long own_b, long org_b, long org_s, long vn,
                     const double* __restrict__ y, double* __restrict__ rhs) {
  __shared__ double red[kCoupleThreads / 32][NR];
  const long s = blockIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double acc[NR];
#pragma unroll
  for (int v = 0; v < NR; v++) acc[v] = 0.0;
  for (int part = 0; part < 2; part++) {
    const double* L = (part == 0 ? tail_a : tail_b) + s * bw;
    const long own = part == 0 ? own_a : own_b, org = part == 0 ? org_a : org_b;
    const double* yy = y + org + own - bw;  // column own - bw + e of the view
    for (long e = lmax(s, bw - own) + threadIdx.x; e < bw; e += kCoupleThreads) {
      const double l = L[e];
#pragma unroll
      for (int v = 0; v < NR; v++) acc[v] += l * yy[v * vn + e];
    }
  }
#pragma unroll
  for (int v = 0; v < NR; v++) {
    const double sv = wsum(acc[v]);
    if (lane == 0) red[w][v] = sv;
  }
  __syncthreads();
  if (threadIdx.x < NR) {
    double t = 0.0;
    for (int q = 0; q < kCoupleThreads / 32; q++) t += red[q][threadIdx.x];
    rhs[threadIdx.x * vn + org_s + s] -= t;
  }
}

// x_S into the tails of views A and B, per column
__global__ void nd_tails_kernel(double* __restrict__ x, long ns, long vn, long tail_a, long tail_b, long org_s,
                                int nr) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= ns * nr) return;
  const long v = t / ns, s = t % ns;
  const double xs = x[v * vn + org_s + s];
  x[v * vn + tail_a + s] = xs;
  x[v * vn + tail_b + s] = xs;
}

// The factorisation as launches per 32-column step (where the single launch
// does not apply, and as its cross-check), with lookahead over two streams.
// Per step k: the panel solve T_k, then on the main stream the update of the
// next panel's tile column with the factorisation of the next diagonal block
// (the chain every step waits on), and on the second stream the rest of the
// trailing update, which overlaps that chain and the next step's panel
// solve. The next step's first-column update waits for this step's rest,
// which writes the same tiles.
static void step_launches(tp_ctx* c) {
  Coarse& C = c->coarse;
  cudaStream_t s = c->s, s2 = C.s2;
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
      const long T = (m + 31) / 32;  // 32-row tiles of the panel
      cudaLaunchConfig_t cfg = {};
      cfg.blockDim = dim3(kTrsmThreads);
      cfg.stream = s;
      cfg.attrs = pri;
      cfg.numAttrs = 1;
      cfg.gridDim = dim3((unsigned)T);
      double* band = C.band;
      const long bw = C.bw, n = C.n;
      const double* lc = C.linv;
      int* info = C.info;
      cudaLaunchKernelEx(&cfg, trsm_kernel, band, bw, k, nb, R0, R1, lc, info);
      if (T > 1) {
        cudaEventRecord(C.ev_panel, s);
        cudaStreamWaitEvent(s2, C.ev_panel, 0);
      }
      if (rest_pending) cudaStreamWaitEvent(s, C.ev_rest, 0);
      cfg.blockDim = dim3(256);
      cudaLaunchKernelEx(&cfg, syrk_panel_kernel, band, bw, n, k, nb, R0, R1, C.linv, info);
      rest_pending = false;
      if (T > 1) {
        const long tiles = T * (T - 1) / 2;
        const unsigned g = (unsigned)std::min(tiles, (long)std::max(1, C.nsm));
        syrk_rest_kernel<<<g, 256, kRestSmem, s2>>>(C.band, C.bw, k, nb, R0, R1, tiles);
        cudaEventRecord(C.ev_rest, s2);
        rest_pending = true;
      }
    }
  }
  if (rest_pending) cudaStreamWaitEvent(s, C.ev_rest, 0);
}

// Plan of the single-launch factorisation: the flag arrays and the count of
// the other CTAs' work items per step (T-1 panel tiles and T(T+1)/2 - 1 tile
// updates for a panel of T tile rows).
// the other CTAs' work items before each of NT steps of a band of n rows
static long pf_items(long n, long bw, long NT, std::vector<long>& off) {
  long TS = 2;
  off.assign(NT + 1, 0);
  for (long k = 0; k < NT; k++) {
    const long T = pf_imax(n, bw, k) - k;
    TS = std::max(TS, T + 2);
    off[k + 1] = off[k] + (T >= 1 ? (T - 1) + T * (T + 1) / 2 - 1 : 0);
  }
  return TS;
}

// whether the factor launch fits with kPfSmem (one CTA per SM), and how
// many CTAs per SM (up to two) it holds with kPfSmem2
static bool pf_fits(int per2[2]) {
  for (auto kern : {pf_kernel<double, 2>, pf_kernel<Dsf, 2>}) {
    int per = 0;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPfSmem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, 256, kPfSmem) != cudaSuccess || per < 1) {
      cudaGetLastError();
      return false;
    }
  }
  int q = 0;
  for (auto kern : {pf_kernel<double, kPfMinBlocksNd<double>>, pf_kernel<Dsf, kPfMinBlocksNd<Dsf>>}) {
    int p2 = 0;
    // (the attribute is the larger size: the FP64 kernel serves both launches)
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPfSmem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p2, kern, 256, kPfSmem2) != cudaSuccess || p2 < 1) {
      cudaGetLastError();
      return false;
    }
    per2[q++] = std::min(kPfPerSm2, p2);
  }
  return true;
}

static void pf_plan(tp_ctx* c) {
  Coarse& C = c->coarse;
  C.pf_ok = false;
  const long NT = (C.n + 31) / 32;
  if (NT < 2 || C.nsm < 2) return;
  std::vector<long> off;
  const long TS = pf_items(C.n, C.bw, NT, off);
  int per2[2] = {0, 0};
  if (!pf_fits(per2)) return;
  C.pf_grid = C.nsm;
  C.nd_grid[0] = per2[0] * C.nsm;
  C.nd_grid[1] = per2[1] * C.nsm;
  C.pf_NT = (int)NT;
  C.pf_TS = (int)TS;
  C.pf_flag_bytes = sizeof(int) * (size_t)(NT + 2 * NT * TS + 1);
  if (dev_malloc(&C.pf_flags, C.pf_flag_bytes) != cudaSuccess ||
      dev_malloc(&C.pf_rpk, sizeof(double) * NT * NB) != cudaSuccess ||
      dev_malloc(&C.pf_off, sizeof(long) * (NT + 1)) != cudaSuccess) {
    cudaGetLastError();
    C.alloc_failed = true;
    return;
  }
  cudaMemcpy(C.pf_off, off.data(), sizeof(long) * (NT + 1), cudaMemcpyHostToDevice);
  c->mem_bytes += (long)C.pf_flag_bytes + 8L * NT * NB + 8L * (NT + 1);
  C.pf_ok = true;
}

static void pf_launch(tp_ctx* c) {
  Coarse& C = c->coarse;
  const long NT = C.pf_NT, TS = C.pf_TS;
  int* f = C.pf_flags;
  PfArgs a{C.band, C.bw, C.n, (int)NT, (int)TS, C.pf_rpk, f, f + NT, f + NT + NT * TS, C.pf_off, C.info,
           f + NT + 2 * NT * TS, C.ps_spin > 0 ? C.ps_spin : kBarrierSpin, 0, C.pf_grid, 0};
  PfArgs none = a;
  none.cta0 = C.pf_grid;
  cudaMemsetAsync(C.pf_flags, 0, C.pf_flag_bytes, c->s);
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)C.pf_grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = kPfSmem;
  cfg.stream = c->s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, C.ds ? pf_kernel<Dsf, 2> : pf_kernel<double, 2>, a, none);
}

static void coarse_factor_launches(tp_ctx* c, size_t dinv_smem) {
  Coarse& C = c->coarse;
  cudaMemsetAsync(C.info, 0, sizeof(int), c->s);
  if (C.solve_variant == 0 && C.pf_ok)
    pf_launch(c);
  else
    step_launches(c);
  const DinvBands one{{C.band, C.band, C.band}, {C.n, C.n, C.n}, {0, C.nblk, C.nblk}};
  (C.ds ? dinv_kernel<Dsf> : dinv_kernel<double>)<<<dim3(C.nblk, C.nbs / 32), kDinvThreads, dinv_smem, c->s>>>(
      one, C.bw, C.nbs, C.dinv, C.dinvT);
  lrow_kernel<<<dim3((unsigned)((C.bw + 31) / 32), C.nbs / 32, C.nblk), dim3(32, 8), 0, c->s>>>(C.band, C.bw, C.n,
                                                                                               C.nbs, C.lrow);
}

// The launch sequence (about 2 per 32 columns) is captured once into a CUDA
// graph on the context's stream and replayed at every design iteration.
static void nd_factor_launches(tp_ctx* c, size_t dinv_smem);

void coarse_factor(tp_ctx* c) {
  ProfScope ps(c, P_COARSE_FACTOR);
  Coarse& C = c->coarse;
  const size_t smem = ((size_t)C.nbs * 33 + 2 * 32 * 33) * sizeof(double);
  const bool nd = C.nd_use;
  cudaGraphExec_t& ex = nd ? C.nd_factor_exec : C.factor_exec;
  auto launches = [&]() {
    if (nd)
      nd_factor_launches(c, smem);
    else
      coarse_factor_launches(c, smem);
  };
  if (!ex) {
    static size_t smem_max = 0;  // the attribute only grows (contexts of other sizes)
    smem_max = std::max(smem_max, smem);
    cudaFuncSetAttribute(dinv_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
    cudaFuncSetAttribute(dinv_kernel<Dsf>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      launches();
      if (cudaStreamEndCapture(c->s, &g) == cudaSuccess && g) {
        if (cudaGraphInstantiate(&ex, g, cudaGraphInstantiateFlagUseNodePriority) != cudaSuccess) ex = nullptr;
        cudaGraphDestroy(g);
      }
    }
    cudaGetLastError();
  }
  if (ex)
    cudaGraphLaunch(ex, c->s);
  else
    launches();
  TP_CHECK_LAUNCH(c, "coarse_factor");
}

// ----------------------------------------------------------------------------
// Block triangular solves, NBS rows per block, warp per row, coalesced:
//   forward   t = b_k - Lrow_k y,   y_k = D_k t
//   backward  t = y_k - L_{.,k}^T x (band columns are contiguous), x_k = D_k^T t
// Up to kSolveCols right-hand sides (columns n apart) share each load of L.
constexpr int kSolveCols = 8;


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
// between phases instead of at a kernel boundary. CTA b owns R rows of every
// block, from mirrored positions (ps_row_of), because a block row's length
// grows or shrinks linearly with its position in every phase: each CTA then
// has the same work. Each row is split into P = 8/R fixed parts, one warp
// each, so every sum is formed in the same order on every call.
// While a CTA works on phase h (and waits at the barrier after it), the
// matrix rows of phase h+1 -- constant during the solve -- arrive in shared
// memory by cp.async; the vectors written by other CTAs are read through L2
// (ld.global.cg). Each barrier wait is bounded: a CTA that gives up sets the
// status word and every CTA leaves at its next barrier; the host reads (and
// clears) the word after the solve and reports TP_ERR_TIMEOUT.
constexpr int kPsWarps = 8;

// Row rl (0 .. R-1) of CTA b among G: rl*G + b for even rl, rl*G + G-1-b for
// odd rl, so the R rows of a CTA pair short with long; a bijection onto
// 0 .. R*G-1.
__device__ __forceinline__ int ps_row_of(int b, int rl, int G) { return rl * G + ((rl & 1) ? G - 1 - b : b); }

// Warp w's row rl and part p. Warps w and w+4 share a sub-partition's FP64
// unit; with R = 4 (P = 2) they take rows 0 and 3 (or 1 and 2), whose
// lengths add up to the same total, so the four units carry equal work.
__device__ __forceinline__ void ps_warp_row(int w, int R, int P, int& rl, int& p) {
  if (R == 4) {
    p = w & 1;
    rl = (w < 4) ? (w >> 1) : 3 - ((w - 4) >> 1);
  } else {
    rl = w / P;
    p = w % P;
  }
}
__device__ __forceinline__ int ps_part_warp(int rl, int q, int R, int P) {
  if (R == 4) return (rl < 2) ? rl * 2 + q : 4 + (3 - rl) * 2 + q;
  return rl * P + q;
}

// A view: a band matrix solved by blocks of nbs rows. Its own rows (nown,
// in blocks) may be followed by a tail (rows nown .. nview-1, solved
// elsewhere): the backward sweep then reads the tail's solution, which the
// caller has put behind the own rows in x. Vector entries of the view sit at
// voff + row of every column.
struct PsView {
  const double* lrow;  // row-major band rows left of each block, nbs x bw per block
  const double* band;  // the view's band (its first row at the origin)
  const double* D;     // block inverses, row-major
  const double* DT;
  long nown, nview, voff;
  int nblk;
};

struct PsArgs {
  PsView v0, v1;  // rows i < nbs of a phase belong to v0, nbs <= i < 2 nbs to v1 (nv = 2)
  int nv;
  long bw, vn;    // half bandwidth; distance between the vectors' columns
  int nbs, m, R, P, seg;  // m: blocks of the longest view
  int tail;       // the views have tails: every block, the last included, has a BA phase
  int h0, h1;     // phases of this launch
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

// phases of the forward sweep, and of both
__host__ __device__ __forceinline__ int ps_nfwd(int m) { return 2 * m - 1; }
__host__ __device__ __forceinline__ int ps_nall(int m, int tail) { return 4 * m - (tail ? 1 : 2); }

// phase h -> (kind, block): forward FB_0, FA_1, FB_1, ..., FB_{m-1}, then
// backward BB_{m-1}, BA_{m-2}, BB_{m-2}, ..., BB_0; with tails the backward
// sweep is BA_{m-1}, BB_{m-1}, BA_{m-2}, ..., BB_0
__device__ __forceinline__ void ps_phase(const PsArgs& a, int h, int& kind, int& k) {
  const int nf = ps_nfwd(a.m);
  if (h < nf) {
    k = (h + 1) / 2;
    kind = (h & 1) ? PH_FA : PH_FB;
  } else if (a.tail) {
    const int q = h - nf;
    k = a.m - 1 - q / 2;
    kind = (q & 1) ? PH_BB : PH_BA;
  } else {
    const int q = h - nf;
    k = a.m - 1 - (q + 1) / 2;
    kind = (q & 1) ? PH_BA : PH_BB;
  }
}

// the view of phase row i (a copy, selected field by field so that it stays
// in registers), and i within it
__device__ __forceinline__ PsView ps_view(const PsArgs& a, int& i) {
  const bool q = a.nv == 2 && i >= a.nbs;
  if (q) i -= a.nbs;
  PsView V;
  V.lrow = q ? a.v1.lrow : a.v0.lrow;
  V.band = q ? a.v1.band : a.v0.band;
  V.D = q ? a.v1.D : a.v0.D;
  V.DT = q ? a.v1.DT : a.v0.DT;
  V.nown = q ? a.v1.nown : a.v0.nown;
  V.nview = q ? a.v1.nview : a.v0.nview;
  V.voff = q ? a.v1.voff : a.v0.voff;
  V.nblk = q ? a.v1.nblk : a.v0.nblk;
  return V;
}

// Row i of block k in phase kind: the matrix entry at position e is m[e], the
// vector entry of column v at vb[v*n + voff + e], for lo <= e < hi. This
// warp's part of the row is [a0, a1).
struct PsRow {
  const double* m;
  const double* vb;
  long voff, a0, a1;
};

// row i of the view V (i within the view's block)
__device__ __forceinline__ bool ps_row(const PsArgs& a, const PsView& V, int kind, int k, int i, int p, PsRow& r) {
  if (k >= V.nblk) return false;
  const long b0 = (long)k * a.nbs;
  const int s = (int)lmin((long)a.nbs, V.nown - b0);
  if (i >= s) return false;
  long lo, hi;
  if (kind == PH_FA) {  // t = b - Lrow_k y over columns b0-bw+e, e in [max(0, bw-b0, i), bw)
    r.m = V.lrow + ((long)k * a.nbs + i) * a.bw;
    r.vb = a.y + V.voff;
    r.voff = b0 - a.bw;
    lo = lmax(lmax(0L, a.bw - b0), (long)i);
    hi = a.bw;
  } else if (kind == PH_FB) {  // y_k = D_k t_k, lower triangle
    r.m = V.D + ((long)k * a.nbs + i) * a.nbs;
    r.vb = (k == 0 ? a.rhs : a.t) + V.voff;
    r.voff = b0;
    lo = 0;
    hi = i + 1;
  } else if (kind == PH_BA) {  // t = y - L(b1.., r)^T x: band column r is contiguous
    const long rr = b0 + i, b1 = lmin(V.nown, b0 + a.nbs);
    r.m = V.band + rr * a.bw;
    r.vb = a.x + V.voff;
    r.voff = 0;
    lo = b1;
    hi = lmin(V.nview - 1, rr + a.bw) + 1;
  } else {  // x_k = D_k^T t_k, upper triangle
    r.m = V.DT + ((long)k * a.nbs + i) * a.nbs;
    r.vb = (a.tail || k != V.nblk - 1 ? a.t : a.y) + V.voff;
    r.voff = b0;
    lo = i;
    hi = s;
  }
  const long len = lmax(0L, hi - lo), cs = (len + a.P - 1) / a.P;  // cs <= seg
  r.a0 = lo + p * cs;
  r.a1 = lmin(hi, r.a0 + cs);
  return true;
}

// stage this warp's part of phase h's matrix row; lane l copies (and later
// reads) positions a0 + l, a0 + l + 32, ...
__device__ __forceinline__ void ps_stage(const PsArgs& a, const PsView& V, int h, double* wbuf, int i, int p,
                                         int lane) {
  int kind, k;
  ps_phase(a, h, kind, k);
  PsRow r;
  if (!ps_row(a, V, kind, k, i, p, r)) return;
  for (long e = r.a0 + lane; e < r.a1; e += 32) cp_async8(wbuf + (e - r.a0), r.m + e);
}

// Grid barrier number h (targets h * gridDim.x arrivals), at most spin polls;
// false if this or another CTA gave up.
__device__ __forceinline__ bool ps_barrier(unsigned* bar, int* err, unsigned target, long spin) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    // arrive with a release (cumulative over the CTA's stores, which the
    // barrier above ordered before it)
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;\n" ::"l"(bar) : "memory");
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

// WIDE: 32 positions per lane per round instead of 16 (one warp per whole
// row, P = 1: a 923-long row in one L2 round trip instead of two; 0.627 ->
// 0.611 ms per solve of both halves at 256x128x128, the same bits; with two
// warps per row the narrow rounds are faster, 0.92 against 1.10 ms)
template <int NR, bool WIDE>
__device__ __forceinline__ void ps_solve_body(const PsArgs& a) {
  extern __shared__ double sm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int rl, p;
  ps_warp_row(w, a.R, a.P, rl, p);
  int i = ps_row_of(blockIdx.x, rl, gridDim.x);
  const PsView V = ps_view(a, i);  // this warp's view and row, the same in every phase
  auto buf = [&](int b) { return sm + (long)(b * kPsWarps + w) * a.seg; };  // stage b of this warp
  double* part = sm + 2L * kPsWarps * a.seg;  // [warp][NR]
  ps_stage(a, V, a.h0, buf(0), i, p, lane);
  cp_commit();
  for (int h = a.h0; h < a.h1; h++) {
    if (h + 1 < a.h1) {
      ps_stage(a, V, h + 1, buf((h + 1 - a.h0) & 1), i, p, lane);
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
    if (ps_row(a, V, kind, k, i, p, r)) {
      // U positions per lane per round: all their L2 loads are issued before
      // the first multiply-add, so a round costs one L2 latency; the sum
      // still runs over the positions in order
      constexpr int U = (NR == 1 ? 16 : (NR == 2 ? 8 : (NR == 4 ? 4 : 2))) * (WIDE ? 2 : 1);
      const double* mb = buf((h - a.h0) & 1);
      for (long e0 = r.a0 + lane; e0 < r.a1; e0 += 32L * U) {
        double mv[U], vv[U][NR];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const long e = e0 + 32L * u;
          const bool in = e < r.a1;
          mv[u] = in ? mb[e - r.a0] : 0.0;
#pragma unroll
          for (int v = 0; v < NR; v++) vv[u][v] = in ? __ldcg(r.vb + (v * a.vn + r.voff + e)) : 0.0;
        }
        // (the compiler keeps the round's loads ahead of its multiply-adds)
        asm volatile("" ::: "memory");
#pragma unroll
        for (int u = 0; u < U; u++)
#pragma unroll
          for (int v = 0; v < NR; v++) acc[v] += mv[u] * vv[u][v];
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
      int row = ps_row_of(blockIdx.x, rr, gridDim.x);
      const PsView W = ps_view(a, row);
      if (k < W.nblk && row < lmin((long)a.nbs, W.nown - b0)) {
        double sum = 0.0;
        for (int q = 0; q < a.P; q++) sum += part[ps_part_warp(rr, q, a.R, a.P) * NR + v];
        const long o = v * a.vn + W.voff + b0 + row;
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
    if (h + 1 < a.h1 && !ps_barrier(a.bar, a.err, (unsigned)(h + 1 - a.h0) * gridDim.x + a.missing, a.spin)) break;
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

// the narrow form keeps the compiler's register choice for 256 threads; the
// wide one may take more (its 32 positions' loads in flight)
template <int NR>
__global__ void __launch_bounds__(kPsWarps * 32) ps_solve_kernel(PsArgs a) {
  ps_solve_body<NR, false>(a);
}
template <int NR>
__global__ void __launch_bounds__(kPsWarps * 32, 1) ps_solve_wide_kernel(PsArgs a) {
  ps_solve_body<NR, true>(a);
}

// Launch plan for phases of `rows` rows: R rows per CTA (1, 2, 4 or 8), the
// fewest that keep at most per_sm CTAs per SM; P = 8/R warps per row; shared
// memory for two stages of every warp's longest part. false if the stages do
// not fit or the grid cannot be co-resident.
struct PsPlan {
  int R = 0, P = 0, grid = 0, seg = 0;
  size_t smem = 0;
};
static bool ps_plan_rows(long rows, long bw, int nbs, int nsm, int per_sm, PsPlan& pl) {
  int R = 1;
  while (R < kPsWarps && (rows + R - 1) / R > (long)per_sm * nsm) R *= 2;
  const int P = kPsWarps / R;
  const long grid = (rows + R - 1) / R;
  if (grid > (long)per_sm * nsm) return false;
  const int need = (int)((grid + nsm - 1) / nsm);  // CTAs per SM
  const long seg = std::max((bw + P - 1) / P, (long)(nbs + P - 1) / P);
  const size_t smem = (size_t)(2 * kPsWarps * seg + kPsWarps * 8) * sizeof(double);
  if (smem > 200 * 1024) return false;
  // the attribute only grows: contexts of other sizes keep their larger plans
  static size_t smem_max = 0;
  const size_t attr = std::max(smem, smem_max);
  auto fits = [&](const void* f) {
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)attr) != cudaSuccess) return false;
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, kPsWarps * 32, smem) != cudaSuccess) return false;
    return per >= need;
  };
  const bool ok = fits((const void*)ps_solve_kernel<1>) && fits((const void*)ps_solve_kernel<2>) &&
                  fits((const void*)ps_solve_kernel<4>) && fits((const void*)ps_solve_kernel<8>) &&
                  fits((const void*)ps_solve_wide_kernel<1>) && fits((const void*)ps_solve_wide_kernel<2>) &&
                  fits((const void*)ps_solve_wide_kernel<4>) && fits((const void*)ps_solve_wide_kernel<8>);
  cudaGetLastError();
  if (!ok) return false;
  smem_max = attr;
  pl.R = R;
  pl.P = P;
  pl.grid = (int)grid;
  pl.seg = (int)seg;
  pl.smem = smem;
  return true;
}

static void ps_plan(tp_ctx* c) {
  Coarse& C = c->coarse;
  C.ps_grid = 0;
  if (!C.bar || C.nblk < 1) return;
  PsPlan pl;
  if (!ps_plan_rows(C.nbs, C.bw, C.nbs, C.nsm, 1, pl)) return;
  C.ps_R = pl.R;
  C.ps_P = pl.P;
  C.ps_seg = pl.seg;
  C.ps_smem = pl.smem;
  C.ps_grid = pl.grid;
}

static PsView ps_view_natural(const Coarse& C) {
  return PsView{C.lrow, C.band, C.dinv, C.dinvT, C.n, C.n, 0, C.nblk};
}

// one cooperative launch of phases [h0, h1) over nv views
template <int NR>
static void ps_launch_views(tp_ctx* c, const PsView& v0, const PsView& v1, int nv, long vn, int m, int tail, int h0,
                            int h1, int R, int P, int seg, int grid, size_t smem, const double* rhs, double* y,
                            double* t, double* x) {
  Coarse& C = c->coarse;
  PsArgs a{v0, v1, nv, C.bw, vn, C.nbs, m, R, P, seg, tail, h0, h1, rhs, y, t, x,
           C.bar, C.serr, C.ps_spin > 0 ? C.ps_spin : kBarrierSpin, (unsigned)C.ps_missing};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kPsWarps * 32);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = c->s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (P == 1)
    cudaLaunchKernelEx(&cfg, ps_solve_wide_kernel<NR>, a);
  else
    cudaLaunchKernelEx(&cfg, ps_solve_kernel<NR>, a);
}

template <int NR>
static void ps_launch(tp_ctx* c, const double* rhs, double* sol, double* y, double* t) {
  Coarse& C = c->coarse;
  const PsView v = ps_view_natural(C);
  ps_launch_views<NR>(c, v, v, 1, C.n, C.nblk, 0, 0, ps_nall(C.nblk, 0), C.ps_R, C.ps_P, C.ps_seg, C.ps_grid,
                      C.ps_smem, rhs, y, t, sol);
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
static void nd_solve(tp_ctx* c, const double* rhs, double* x, int nr);

void coarse_solve(tp_ctx* c, const double* rhs, double* x, int nr) {
  ProfScope ps(c, P_COARSE_SOLVE);
  Coarse& C = c->coarse;
  if (C.nd_use) {
    nd_solve(c, rhs, x, nr);
    return;
  }
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


// ----------------------------------------------------------------------------
// The dissected factor and solve: layout, plans and launch sequences.

static void nd_layout(tp_ctx* c) {
  Coarse& C = c->coarse;
  C.nd_ok = false;
  const Level& L = c->L[c->nl - 1];
  const int xs = (L.nx - 1) / 2;
  if (xs < 1 || L.nx - 1 - xs < 1) return;
  const long plane = 3L * L.ny * L.nz;
  const long na = plane * xs, nb = plane * (L.nx - 1 - xs);
  C.nd_xs = xs;
  C.nd_ns = plane;
  C.nd_pad[0] = (32 - na % 32) % 32;
  C.nd_pad[1] = (32 - nb % 32) % 32;
  C.nd_own[0] = C.nd_pad[0] + na;
  C.nd_own[1] = C.nd_pad[1] + nb;
  C.nd_own[2] = plane;
  C.nd_org[0] = 0;
  C.nd_org[1] = C.nd_own[0] + plane;
  C.nd_org[2] = C.nd_org[1] + C.nd_own[1] + plane;
  C.nd_ntot = C.nd_org[2] + plane;
  int b0 = 0;
  for (int v = 0; v < 3; v++) {
    C.nd_blk0[v] = b0;
    C.nd_nblk[v] = (int)((C.nd_own[v] + C.nbs - 1) / C.nbs);
    b0 += C.nd_nblk[v];
  }
  // two steps per partial factor and two tiles of S at least; the natural
  // half bandwidth (it holds the mirrored couplings and S x S); both halves
  // of the grid with several CTAs
  const long bw_nat = 3L * ((long)L.nz * L.ny + L.ny + 1) + 2;
  if (C.nd_own[0] / 32 < 2 || C.nd_own[1] / 32 < 2 || plane < 64 || C.bw != bw_nat || plane - 1 > C.bw ||
      C.nsm < 8 || C.nd_ntot >= (1L << 31))
    return;
  C.nd_ok = true;
}

static void nd_plan(tp_ctx* c) {
  Coarse& C = c->coarse;
  if (!C.nd_ok) return;
  C.nd_ok = false;
  if (!C.pf_ok || C.ps_grid <= 0) return;
  PsPlan p2;
  // two views per phase: eight rows per CTA, one warp per row (two CTAs per
  // SM of four rows each measured slower: 0.65 against 0.63 ms per solve).
  // Where a warp's staged row does not fit (wide bands: 1,955 at the
  // coarsest level of 384x192x192), the halves are swept one after the
  // other with the single-view plan (ps2_grid = 0).
  if (!ps_plan_rows(2L * C.nbs, C.bw, C.nbs, C.nsm, 1, p2)) p2 = PsPlan();
  const Level& L = c->L[c->nl - 1];
  const long ns = C.nd_ns;
  std::vector<long> offs[3];
  long nflags = 0, nrpk = 0, noff = 0;
  for (int v = 0; v < 3; v++) {
    const long nview = v < 2 ? C.nd_own[v] + ns : ns;
    const long NT = v < 2 ? C.nd_own[v] / 32 : (ns + 31) / 32;
    const long TS = pf_items(nview, C.bw, NT, offs[v]);
    C.nd_NT[v] = (int)NT;
    C.nd_TS[v] = (int)TS;
    C.nd_fo[v] = nflags;
    // tver has a row per tile of the view: the partial factors update the
    // tiles of the trailing block too (rows NT .. tiles-1)
    const long tiles = (nview + 31) / 32;
    nflags += NT + NT * TS + tiles * TS;
    C.nd_ro[v] = nrpk;
    nrpk += NT;
    C.nd_io[v] = noff;
    noff += NT + 1;
  }
  nflags += 1;  // the abort flag of all three factors
  C.nd_flag_bytes = sizeof(int) * (size_t)nflags;
  // the CTAs of the concurrent partial factors, in proportion to their rows
  const double fa = (double)C.nd_own[0] / (double)(C.nd_own[0] + C.nd_own[1]);
  for (int q = 0; q < 2; q++)
    C.nd_split[q] = (int)std::min((long)C.nd_grid[q] - 2, std::max(2L, std::lround(fa * C.nd_grid[q])));
  // composite row -> natural row
  std::vector<int> map(C.nd_ntot, -1);
  for (long r = C.nd_pad[0]; r < C.nd_own[0]; r++) map[r] = (int)(r - C.nd_pad[0]);
  for (int p = C.nd_xs + 1; p < L.nx; p++)
    for (int k = 0; k < L.nz; k++)
      for (int j = 0; j < L.ny; j++)
        for (int q = 0; q < 3; q++)
          map[C.nd_org[1] + nd_pos_b(p, k, j, q, L.nx, L.ny, L.nz, C.nd_pad[1])] =
              (int)(3L * (((long)p * L.nz + k) * L.ny + j) + q);
  for (long r = 0; r < ns; r++) map[C.nd_org[2] + r] = (int)(C.nd_xs * ns + r);
  std::vector<long> off_all;
  for (int v = 0; v < 3; v++) off_all.insert(off_all.end(), offs[v].begin(), offs[v].end());
  if (dev_malloc(&C.nd_map, sizeof(int) * C.nd_ntot) != cudaSuccess ||
      dev_malloc(&C.nd_vec, sizeof(double) * 32 * C.nd_ntot) != cudaSuccess ||
      dev_malloc(&C.nd_tail, sizeof(double) * 2 * ns * C.bw) != cudaSuccess ||
      dev_malloc(&C.nd_flags, C.nd_flag_bytes) != cudaSuccess ||
      dev_malloc(&C.nd_rpk, sizeof(double) * nrpk * NB) != cudaSuccess ||
      dev_malloc(&C.nd_off, sizeof(long) * noff) != cudaSuccess) {
    cudaGetLastError();
    C.alloc_failed = true;
    return;
  }
  cudaMemcpy(C.nd_map, map.data(), sizeof(int) * C.nd_ntot, cudaMemcpyHostToDevice);
  cudaMemcpy(C.nd_off, off_all.data(), sizeof(long) * noff, cudaMemcpyHostToDevice);
  c->mem_bytes += (long)(4 * C.nd_ntot + 8 * 32 * C.nd_ntot + 16 * ns * C.bw + (long)C.nd_flag_bytes +
                         8 * nrpk * NB + 8 * noff);
  C.ps2_R = p2.R;
  C.ps2_P = p2.P;
  C.ps2_seg = p2.seg;
  C.ps2_grid = p2.grid;
  C.ps2_smem = p2.smem;
  C.nd_ok = true;
}

static PfArgs nd_args(const Coarse& C, int v, int cta0, int ncta) {
  int* f = C.nd_flags + C.nd_fo[v];
  const long NT = C.nd_NT[v], TS = C.nd_TS[v];
  return PfArgs{C.band + C.nd_org[v] * (C.bw + 1),
                C.bw,
                v < 2 ? C.nd_own[v] + C.nd_ns : C.nd_ns,
                (int)NT,
                (int)TS,
                C.nd_rpk + C.nd_ro[v] * NB,
                f,
                f + NT,
                f + NT + NT * TS,
                C.nd_off + C.nd_io[v],
                C.info,
                C.nd_flags + C.nd_flag_bytes / sizeof(int) - 1,
                C.ps_spin > 0 ? C.ps_spin : kBarrierSpin,
                cta0,
                ncta,
                v < 2 ? 1 : 0};
}

static void nd_pf_launch(tp_ctx* c, const PfArgs& a0, const PfArgs& a1) {
  Coarse& C = c->coarse;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)C.nd_grid[C.ds ? 1 : 0]);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = kPfSmem2;
  cfg.stream = c->s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, C.ds ? pf_kernel<Dsf, kPfMinBlocksNd<Dsf>> : pf_kernel<double, kPfMinBlocksNd<double>>, a0,
                     a1);
}

// partial factors of A and B (one launch), S = the sum of their trailing
// blocks, S's factor, then the block inverses and block rows of each view
// and the tails' rows
static void nd_factor_launches(tp_ctx* c, size_t dinv_smem) {
  Coarse& C = c->coarse;
  const long ns = C.nd_ns, bw = C.bw;
  cudaMemsetAsync(C.info, 0, sizeof(int), c->s);
  cudaMemsetAsync(C.nd_flags, 0, C.nd_flag_bytes, c->s);
  const int grid = C.nd_grid[C.ds ? 1 : 0], split = C.nd_split[C.ds ? 1 : 0];
  nd_pf_launch(c, nd_args(C, 0, 0, split), nd_args(C, 1, split, grid - split));
  nd_schur_kernel<<<grid_for(ns * ns, 256), 256, 0, c->s>>>(C.band, bw, ns, C.nd_own[0], C.nd_org[1], C.nd_own[1],
                                                           C.nd_org[2]);
  PfArgs s = nd_args(C, 2, 0, grid), none = s;
  none.cta0 = grid;
  nd_pf_launch(c, s, none);
  DinvBands views;
  for (int v = 0; v < 3; v++) {
    views.B[v] = C.band + C.nd_org[v] * (bw + 1);
    views.n[v] = C.nd_own[v];
    views.blk0[v] = C.nd_blk0[v];
  }
  (C.ds ? dinv_kernel<Dsf> : dinv_kernel<double>)<<<dim3(C.nd_blk0[2] + C.nd_nblk[2], C.nbs / 32), kDinvThreads,
                                                    dinv_smem, c->s>>>(views, bw, C.nbs, C.dinv, C.dinvT);
  for (int v = 0; v < 3; v++)
    lrow_kernel<<<dim3((unsigned)((bw + 31) / 32), C.nbs / 32, C.nd_nblk[v]), dim3(32, 8), 0, c->s>>>(
        views.B[v], bw, C.nd_own[v], C.nbs, C.lrow + (size_t)C.nd_blk0[v] * C.nbs * bw);
  for (int v = 0; v < 2; v++)
    lrow_kernel<<<dim3((unsigned)((bw + 31) / 32), (unsigned)((ns + 31) / 32), 1), dim3(32, 8), 0, c->s>>>(
        C.band + C.nd_org[v] * (bw + 1), bw, C.nd_own[v] + ns, (int)ns, C.nd_tail + v * ns * bw, C.nd_own[v]);
}

static PsView nd_view(const Coarse& C, int v) {
  const size_t b0 = (size_t)C.nd_blk0[v];
  return PsView{C.lrow + b0 * C.nbs * C.bw,
                C.band + C.nd_org[v] * (C.bw + 1),
                C.dinv + b0 * C.nbs * C.nbs,
                C.dinvT + b0 * C.nbs * C.nbs,
                C.nd_own[v],
                v < 2 ? C.nd_own[v] + C.nd_ns : C.nd_ns,
                C.nd_org[v],
                C.nd_nblk[v]};
}

// one solve of NR columns (n apart) from rhs into x: forward sweeps of A
// and B (one launch, both views in every phase), b_S -= L_SA y_A + L_SB y_B,
// S forward and backward, x_S into the tails, backward sweeps of A and B
template <int NR>
static void nd_solve_launches(tp_ctx* c, const double* rhs, double* x) {
  Coarse& C = c->coarse;
  const long vn = C.nd_ntot, ns = C.nd_ns;
  double *rb = C.nd_vec, *y = rb + 8 * vn, *t = y + 8 * vn, *xc = t + 8 * vn;
  nd_gather_kernel<<<grid_for(vn * NR, 256), 256, 0, c->s>>>(C.nd_map, vn, rhs, C.n, rb, NR);
  const PsView va = nd_view(C, 0), vb = nd_view(C, 1), vs = nd_view(C, 2);
  const int m = std::max(C.nd_nblk[0], C.nd_nblk[1]);
  // both halves in every phase, or one half after the other
  const bool two = C.ps2_grid > 0 && C.order != 2;
  auto sweep = [&](bool fwd) {
    if (two) {
      ps_launch_views<NR>(c, va, vb, 2, vn, m, 1, fwd ? 0 : ps_nfwd(m), fwd ? ps_nfwd(m) : ps_nall(m, 1), C.ps2_R,
                          C.ps2_P, C.ps2_seg, C.ps2_grid, C.ps2_smem, rb, y, t, xc);
      return;
    }
    for (const PsView& v : {va, vb})
      ps_launch_views<NR>(c, v, v, 1, vn, v.nblk, 1, fwd ? 0 : ps_nfwd(v.nblk), fwd ? ps_nfwd(v.nblk) : ps_nall(v.nblk, 1),
                          C.ps_R, C.ps_P, C.ps_seg, C.ps_grid, C.ps_smem, rb, y, t, xc);
  };
  sweep(true);
  nd_couple_kernel<NR><<<(unsigned)ns, kCoupleThreads, 0, c->s>>>(C.nd_tail, C.nd_tail + ns * C.bw, C.bw, ns,
                                                                 C.nd_own[0], C.nd_org[0], C.nd_own[1], C.nd_org[1],
                                                                 C.nd_org[2], vn, y, rb);
  ps_launch_views<NR>(c, vs, vs, 1, vn, C.nd_nblk[2], 0, 0, ps_nall(C.nd_nblk[2], 0), C.ps_R, C.ps_P, C.ps_seg,
                      C.ps_grid, C.ps_smem, rb, y, t, xc);
  nd_tails_kernel<<<grid_for(ns * NR, 256), 256, 0, c->s>>>(xc, ns, vn, C.nd_org[0] + C.nd_own[0],
                                                           C.nd_org[1] + C.nd_own[1], C.nd_org[2], NR);
  sweep(false);
  nd_scatter_out_kernel<<<grid_for(vn * NR, 256), 256, 0, c->s>>>(C.nd_map, vn, xc, C.n, x, NR);
}

static void nd_solve(tp_ctx* c, const double* rhs, double* x, int nr) {
  Coarse& C = c->coarse;
  if (nr > 1 || c->capturing) {
    for (int r0 = 0; r0 < nr;) {
      const double* b = rhs + (long)r0 * C.n;
      double* xx = x + (long)r0 * C.n;
      const int left = nr - r0;
      if (left >= 8) {
        nd_solve_launches<8>(c, b, xx);
        r0 += 8;
      } else if (left >= 4) {
        nd_solve_launches<4>(c, b, xx);
        r0 += 4;
      } else if (left >= 2) {
        nd_solve_launches<2>(c, b, xx);
        r0 += 2;
      } else {
        nd_solve_launches<1>(c, b, xx);
        r0 += 1;
      }
    }
    TP_CHECK_LAUNCH(c, "coarse_solve");
    return;
  }
  cudaMemcpyAsync(C.rhs, rhs, sizeof(double) * C.n, cudaMemcpyDeviceToDevice, c->s);
  if (!C.nd_graph_exec) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      nd_solve_launches<1>(c, C.rhs, C.sol);
      if (cudaStreamEndCapture(c->s, &g) == cudaSuccess && g) {
        if (cudaGraphInstantiate(&C.nd_graph_exec, g, 0) != cudaSuccess) C.nd_graph_exec = nullptr;
        cudaGraphDestroy(g);
      }
    }
    cudaGetLastError();
  }
  if (C.nd_graph_exec)
    cudaGraphLaunch(C.nd_graph_exec, c->s);
  else
    nd_solve_launches<1>(c, C.rhs, C.sol);
  cudaMemcpyAsync(x, C.sol, sizeof(double) * C.n, cudaMemcpyDeviceToDevice, c->s);
  TP_CHECK_LAUNCH(c, "coarse_solve");
}

}  // namespace tp
