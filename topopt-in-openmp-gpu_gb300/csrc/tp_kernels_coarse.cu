// Levels >= 1: assembled 27-point block stencils, and the grid transfers.
//
// The reference applies level 1 matrix-free, summing for every coarse
// element the E(rho)-weighted stiffness of its ncell^3 fine sub-cells
// (stencil_methods.c:436-519), and assembles levels >= 2 into CSR on the
// host (stencil_assembly.c:126-260). Here every level >= 1 is assembled once
// per design iteration on the GPU into a block stencil of the symmetric
// operator without boundary conditions, stored in half: for each node the
// 3x3 blocks to itself and to its 13 neighbours of larger index (the other
// 13 are the transposes of blocks the neighbours store). The operator
// semantics of the reference are applied when the stencil is applied:
//   level 1      : free rows couple to every neighbour, fixed rows = identity
//                  (the matrix-free subspace operator);
//   level >= 2   : additionally the columns of fixed DOFs are zeroed (the CSR
//                  with BC rows/columns zeroed and a unit diagonal).
// The Jacobi diagonal comes from the unmodified sum, 1 at fixed DOFs, as
// assembleInvertedMatrixDiagonalSubspace_halo does for every level.
#include "tp_internal.h"

namespace tp {

__host__ __device__ constexpr int cloc(int dx, int dy, int dz) {
  return dz * 4 + (dy ? (dx ? 1 : 0) : (dx ? 2 : 3));
}

struct CGeom {
  int nx, ny, nz, ex, ey, ez, lim;
  int ncell, lg2;  // fine sub-cells per coarse element edge
  int fex, fey, fez;  // fine elements
  long nnodes;
};

static CGeom cgeom(const tp_ctx* c, int l) {
  const Level& L = c->L[l];
  const Level& F = c->L[0];
  return CGeom{L.nx, L.ny, L.nz, L.ex, L.ey, L.ez, L.lim, 1 << l, l, F.ex, F.ey, F.ez, L.nnodes};
}

__device__ __forceinline__ bool is_fixed(const CGeom& g, int i, int j) {
  return i == 0 && (j < g.lim || j >= g.ny - g.lim);
}

// G lanes cooperate on one node; each lane sums a strided share of the
// ncell^3 sub-cells, then the lanes reduce by shuffles.
template <typename T, int G>
__global__ void assemble_kernel(CGeom g, const T* __restrict__ E, const T* __restrict__ ke,
                                T* __restrict__ st, double* __restrict__ invD) {
  const long tid = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long n = tid / G;
  const int lane = threadIdx.x % G;
  if (n >= g.nnodes) return;  // G divides the block size: whole groups leave together
  const int j = n % g.ny;
  const int k = (n / g.ny) % g.nz;
  const int i = n / ((long)g.ny * g.nz);
  const int nc = g.ncell, nsub = nc * nc * nc;
  const bool nfix = is_fixed(g, i, j);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) / G * G));

  for (int m = 13; m < 27; m++) {  // the stored half: the node and its 13 higher neighbours
    const int mx = m / 9 - 1, mz = (m / 3) % 3 - 1, my = m % 3 - 1;
    T acc[9];
#pragma unroll
    for (int q = 0; q < 9; q++) acc[q] = T(0);
    const int mi = i + mx, mk = k + mz, mj = j + my;
    const bool minside = mi >= 0 && mi < g.nx && mk >= 0 && mk < g.nz && mj >= 0 && mj < g.ny;
    if (minside) {
#pragma unroll
      for (int e = 0; e < 8; e++) {
        const int ex = -(e & 1), ez = -((e >> 1) & 1), ey = -((e >> 2) & 1);
        const int rx = mx - ex, ry = my - ey, rz = mz - ez;
        if (rx < 0 || rx > 1 || ry < 0 || ry > 1 || rz < 0 || rz > 1) continue;
        const int ci = i + ex, ck = k + ez, cj = j + ey;
        if (ci < 0 || ci >= g.ex || ck < 0 || ck >= g.ez || cj < 0 || cj >= g.ey) continue;
        const int qn = cloc(-ex, -ey, -ez), qm = cloc(rx, ry, rz);
        for (int s = lane; s < nsub; s += G) {
          const int ii = s >> (2 * g.lg2), kk = (s >> g.lg2) & (nc - 1), jj = s & (nc - 1);
          const long fe = ((long)(ci * nc + ii) * g.fez + (ck * nc + kk)) * g.fey + (cj * nc + jj);
          const T Es = E[fe];
          const T* K = ke + (long)s * 576 + (3 * qn) * 24 + 3 * qm;
#pragma unroll
          for (int c = 0; c < 3; c++)
#pragma unroll
            for (int d = 0; d < 3; d++) acc[3 * c + d] += Es * K[24 * c + d];
        }
      }
    }
    if (G > 1) {
#pragma unroll
      for (int q = 0; q < 9; q++)
        for (int o = G / 2; o > 0; o >>= 1) acc[q] += __shfl_down_sync(gmask, acc[q], o, G);
    }
    if (lane == 0) {
      if (m == 13) {  // the node itself: Jacobi diagonal before BCs
        for (int c = 0; c < 3; c++) invD[3 * n + c] = nfix ? 1.0 : 1.0 / (double)acc[4 * c];
      }
#pragma unroll
      for (int q = 0; q < 9; q++) st[(long)((m - 13) * 9 + q) * g.nnodes + n] = acc[q];
    }
  }
}

// Levels >= 2 (tables from moment_tables, tp_setup.cpp): first the 27
// moments M[px*9 + py*3 + pz] = sum_s E_s mx^px my^py mz^pz of each coarse
// element's sub-cell densities (one thread per element, factorised along
// y, z, x), then per node the same 27 x 8 blocks as assemble_kernel, each
// entry a short sparse combination of one element's moments (about 11
// coefficients, staged in shared memory) instead of a sum over ncell^3
// sub-cells. FP64 throughout; the stencil is stored in T.
__global__ void moments_kernel(CGeom g, const double* __restrict__ E, double* __restrict__ M, long ncoarse) {
  const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (e >= ncoarse) return;
  const int cj = e % g.ey, ck = (e / g.ey) % g.ez, ci = e / ((long)g.ey * g.ez);
  const int nc = g.ncell;
  const double h = 1.0 / nc;
  double mom[27];
#pragma unroll
  for (int p = 0; p < 27; p++) mom[p] = 0.0;
  for (int ii = 0; ii < nc; ii++) {
    const double mx = (ii + 0.5) * h - 0.5;
    double yz[9];
#pragma unroll
    for (int q = 0; q < 9; q++) yz[q] = 0.0;
    for (int kk = 0; kk < nc; kk++) {
      const double mz = (kk + 0.5) * h - 0.5;
      const double* row = E + ((long)(ci * nc + ii) * g.fez + (ck * nc + kk)) * g.fey + (long)cj * nc;
      double s0 = 0.0, s1 = 0.0, s2 = 0.0;
      for (int jj = 0; jj < nc; jj++) {
        const double my = (jj + 0.5) * h - 0.5, ev = row[jj], t = my * ev;
        s0 += ev;
        s1 += t;
        s2 += my * t;
      }
      const double s[3] = {s0, s1, s2}, pz[3] = {1.0, mz, mz * mz};
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) yz[a * 3 + b] += s[a] * pz[b];
    }
    const double px[3] = {1.0, mx, mx * mx};
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int q = 0; q < 9; q++) mom[a * 9 + q] += yz[q] * px[a];
  }
#pragma unroll
  for (int p = 0; p < 27; p++) M[(long)p * ncoarse + e] = mom[p];
}

template <typename T>
__global__ void __launch_bounds__(256, 1) moment_stencil_kernel(CGeom g, const double* __restrict__ M, long ncoarse,
                                                             const double* __restrict__ gcoef,
                                                             const int* __restrict__ gint, int nnz,
                                                             T* __restrict__ st, double* __restrict__ invD) {
  extern __shared__ double smg[];
  double* sc = smg;                                   // coefficients
  int* sp = reinterpret_cast<int*>(smg + nnz);        // moment indices
  int* so = sp + nnz;                                 // offsets, 64 blocks x 9 entries + 1
  for (int q = threadIdx.x; q < nnz; q += blockDim.x) {
    sc[q] = gcoef[q];
    sp[q] = gint[q];
  }
  for (int q = threadIdx.x; q <= 576; q += blockDim.x) so[q] = gint[nnz + q];
  __syncthreads();
  const long n = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (n >= g.nnodes) return;
  const int j = n % g.ny;
  const int k = (n / g.ny) % g.nz;
  const int i = n / ((long)g.ny * g.nz);
  const bool nfix = is_fixed(g, i, j);
  for (int m = 13; m < 27; m++) {  // the stored half: the node and its 13 higher neighbours
    const int mx = m / 9 - 1, mz = (m / 3) % 3 - 1, my = m % 3 - 1;
    double acc[9];
#pragma unroll
    for (int q = 0; q < 9; q++) acc[q] = 0.0;
    const int mi = i + mx, mk = k + mz, mj = j + my;
    const bool minside = mi >= 0 && mi < g.nx && mk >= 0 && mk < g.nz && mj >= 0 && mj < g.ny;
    if (minside) {
#pragma unroll
      for (int e = 0; e < 8; e++) {
        const int ex = -(e & 1), ez = -((e >> 1) & 1), ey = -((e >> 2) & 1);
        const int rx = mx - ex, ry = my - ey, rz = mz - ez;
        if (rx < 0 || rx > 1 || ry < 0 || ry > 1 || rz < 0 || rz > 1) continue;
        const int ci = i + ex, ck = k + ez, cj = j + ey;
        if (ci < 0 || ci >= g.ex || ck < 0 || ck >= g.ez || cj < 0 || cj >= g.ey) continue;
        const int blk = (cloc(-ex, -ey, -ez) * 8 + cloc(rx, ry, rz)) * 9;
        const double* Me = M + ((long)ci * g.ez + ck) * g.ey + cj;
#pragma unroll
        for (int q = 0; q < 9; q++) {
          double a = 0.0;
          for (int t = so[blk + q]; t < so[blk + q + 1]; t++) a += sc[t] * Me[(long)sp[t] * ncoarse];
          acc[q] += a;
        }
      }
    }
    if (m == 13) {  // the node itself: Jacobi diagonal before BCs
      for (int c = 0; c < 3; c++) invD[3 * n + c] = nfix ? 1.0 : 1.0 / acc[4 * c];
    }
#pragma unroll
    for (int q = 0; q < 9; q++) st[(long)((m - 13) * 9 + q) * g.nnodes + n] = (T)acc[q];
  }
}

template <typename T>
void assemble_stencil(tp_ctx* c, int l, const T* E, const T* ke, T* st, double* invD) {
  ProfScope ps(c, P_ASSEMBLE);
  const CGeom g = cgeom(c, l);
  const int nsub = g.ncell * g.ncell * g.ncell;
  const int threads = 256;
  if (l >= 2 && c->mg_nnz[l] > 0 && c->d_mom) {
    const long nce = (long)c->L[l].ex * c->L[l].ey * c->L[l].ez;
    const int nnz = c->mg_nnz[l];
    const size_t smem = sizeof(double) * nnz + sizeof(int) * (nnz + 577);
    moments_kernel<<<grid_for(nce, 128), 128, 0, c->s>>>(g, c->d_E, c->d_mom, nce);
    cudaFuncSetAttribute(moment_stencil_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    moment_stencil_kernel<T><<<grid_for(g.nnodes, threads), threads, smem, c->s>>>(
        g, c->d_mom, nce, c->d_mgc[l], c->d_mgi[l], nnz, st, invD);
    TP_CHECK_LAUNCH(c, "assemble_stencil");
    return;
  }
  // 8 sub-cells per coarse element (level 1): one thread per node sums them
  // in order; the lanes' shuffle reductions of the 8-lane form cost more
  // instructions than the sums themselves
  if (nsub >= 32)
    assemble_kernel<T, 32><<<grid_for(g.nnodes * 32, threads), threads, 0, c->s>>>(g, E, ke, st, invD);
  else
    assemble_kernel<T, 1><<<grid_for(g.nnodes, threads), threads, 0, c->s>>>(g, E, ke, st, invD);
  TP_CHECK_LAUNCH(c, "assemble_stencil");
}
template void assemble_stencil<double>(tp_ctx*, int, const double*, const double*, double*, double*);
template void assemble_stencil<float>(tp_ctx*, int, const float*, const float*, float*, double*);

enum { S_APPLY = 0, S_JACOBI = 1, S_RESID = 2 };

// The stencil holds the symmetric operator without boundary conditions in
// half: for each node n its own block and the blocks to the 13 neighbours
// with a larger node index (m = 13..26, stored as m - 13); the block to a
// neighbour with a smaller index is the transpose of the block that
// neighbour stores (index 13 - m). The conditions are applied here: a
// fixed node's rows are the identity; with masked (levels >= 2) a free row
// drops the columns of fixed neighbours. NR right-hand sides (columns
// 3*nnodes apart) share each coefficient load.
template <typename T, int MODE, int NR>
__global__ void __launch_bounds__(128, (NR == 1 && sizeof(T) == 4) ? 4 : 1)
    stencil_kernel(CGeom g, const T* __restrict__ st, const T* __restrict__ in,
                               T* __restrict__ out, const T* __restrict__ b,
                               const T* __restrict__ invD, T omega, int masked) {
  const long n = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (n >= g.nnodes) return;
  const long vs = 3 * g.nnodes;
  const int j = n % g.ny;
  const int k = (n / g.ny) % g.nz;
  const int i = n / ((long)g.ny * g.nz);
  T y[NR][3];
  if (is_fixed(g, i, j)) {
#pragma unroll
    for (int r = 0; r < NR; r++)
#pragma unroll
      for (int c = 0; c < 3; c++) y[r][c] = in[r * vs + 3 * n + c];
  } else {
#pragma unroll
    for (int r = 0; r < NR; r++) y[r][0] = y[r][1] = y[r][2] = T(0);
    // BATCH neighbours at a time (a whole x plane for one column): all their
    // coefficient and vector loads are issued before the first multiply-add
    // (a neighbour outside the grid, or a masked fixed one, reads the node's
    // own entries and contributes zero), so that many loads are in flight
    constexpr int BATCH = NR == 1 ? 9 : 3;
#pragma unroll
    for (int m0 = 0; m0 < 27; m0 += BATCH) {
      T a[BATCH][9], u[BATCH][NR][3];
      bool ok[BATCH];
#pragma unroll
      for (int t = 0; t < BATCH; t++) {
        const int m = m0 + t;
        const int mx = m / 9 - 1, mz = (m / 3) % 3 - 1, my = m % 3 - 1;
        const int mi = i + mx, mk = k + mz, mj = j + my;
        ok[t] = mi >= 0 && mi < g.nx && mk >= 0 && mk < g.nz && mj >= 0 && mj < g.ny &&
                !(masked && m != 13 && is_fixed(g, mi, mj));
        const long nm = ok[t] ? ((long)mi * g.nz + mk) * g.ny + mj : n;
        if (m >= 13) {
          const T* A = st + (long)(m - 13) * 9 * g.nnodes + n;
#pragma unroll
          for (int q = 0; q < 9; q++) a[t][q] = A[q * g.nnodes];
        } else {
          const T* A = st + (long)(13 - m) * 9 * g.nnodes + nm;
#pragma unroll
          for (int c = 0; c < 3; c++)
#pragma unroll
            for (int d = 0; d < 3; d++) a[t][3 * c + d] = A[(3 * d + c) * g.nnodes];
        }
#pragma unroll
        for (int r = 0; r < NR; r++)
#pragma unroll
          for (int d = 0; d < 3; d++) u[t][r][d] = in[r * vs + 3 * nm + d];
      }
#pragma unroll
      for (int t = 0; t < BATCH; t++) {
        if (!ok[t]) continue;
#pragma unroll
        for (int r = 0; r < NR; r++)
#pragma unroll
          for (int c = 0; c < 3; c++)
            y[r][c] += a[t][3 * c] * u[t][r][0] + a[t][3 * c + 1] * u[t][r][1] + a[t][3 * c + 2] * u[t][r][2];
      }
    }
  }
#pragma unroll
  for (int r = 0; r < NR; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const long o = r * vs + 3 * n + c;
      if (MODE == S_APPLY) out[o] = y[r][c];
      if (MODE == S_JACOBI) out[o] = in[o] + omega * invD[3 * n + c] * (b[o] - y[r][c]);
      if (MODE == S_RESID) out[o] = b[o] - y[r][c];
    }
}

// nr columns in chunks of 8, 4, 2, 1 (each chunk reads the stencil once)
template <typename T, int MODE>
static void stencil_launch(tp_ctx* c, int l, const T* st, const T* in, T* out, const T* b, const T* invD, T omega,
                           int nr, int masked) {
  const CGeom g = cgeom(c, l);
  const long vs = 3 * g.nnodes;
  const unsigned grid = grid_for(g.nnodes, 128);
  if (masked < 0) masked = l >= 2;
  for (int r0 = 0; r0 < nr;) {
    const int left = nr - r0;
    const long o = r0 * vs;
    const T* bb = b ? b + o : nullptr;
    if (left >= 8) {
      stencil_kernel<T, MODE, 8><<<grid, 128, 0, c->s>>>(g, st, in + o, out + o, bb, invD, omega, masked);
      r0 += 8;
    } else if (left >= 4) {
      stencil_kernel<T, MODE, 4><<<grid, 128, 0, c->s>>>(g, st, in + o, out + o, bb, invD, omega, masked);
      r0 += 4;
    } else if (left >= 2) {
      stencil_kernel<T, MODE, 2><<<grid, 128, 0, c->s>>>(g, st, in + o, out + o, bb, invD, omega, masked);
      r0 += 2;
    } else {
      stencil_kernel<T, MODE, 1><<<grid, 128, 0, c->s>>>(g, st, in + o, out + o, bb, invD, omega, masked);
      r0 += 1;
    }
  }
}

template <typename T>
void stencil_apply(tp_ctx* c, int l, const T* st, const T* in, T* out, int nr, int masked) {
  ProfScope ps(c, P_STENCIL);
  stencil_launch<T, S_APPLY>(c, l, st, in, out, nullptr, nullptr, T(0), nr, masked);
  TP_CHECK_LAUNCH(c, "stencil_apply");
}
template <typename T>
void stencil_jacobi(tp_ctx* c, int l, const T* st, const T* invD, const T* b, const T* u, T* unew, T omega, int nr,
                    int masked) {
  ProfScope ps(c, P_STENCIL);
  stencil_launch<T, S_JACOBI>(c, l, st, u, unew, b, invD, omega, nr, masked);
  TP_CHECK_LAUNCH(c, "stencil_jacobi");
}
template <typename T>
void stencil_resid(tp_ctx* c, int l, const T* st, const T* b, const T* u, T* d, int nr, int masked) {
  ProfScope ps(c, P_STENCIL);
  stencil_launch<T, S_RESID>(c, l, st, u, d, b, nullptr, T(0), nr, masked);
  TP_CHECK_LAUNCH(c, "stencil_resid");
}
template void stencil_apply<double>(tp_ctx*, int, const double*, const double*, double*, int, int);
template void stencil_apply<float>(tp_ctx*, int, const float*, const float*, float*, int, int);
template void stencil_jacobi<double>(tp_ctx*, int, const double*, const double*, const double*, const double*, double*,
                                     double, int, int);
template void stencil_jacobi<float>(tp_ctx*, int, const float*, const float*, const float*, const float*, float*, float,
                                    int, int);
template void stencil_resid<double>(tp_ctx*, int, const double*, const double*, const double*, double*, int, int);
template void stencil_resid<float>(tp_ctx*, int, const float*, const float*, const float*, float*, int, int);

// The stencil of level l in the full 27-block form with the boundary
// conditions applied (masked: also the columns of fixed neighbours), as the
// reference-layout entry points hand it out: out[(m*9 + 3c + d)*nnodes + n].
__global__ void stencil_expand_kernel(CGeom g, const double* __restrict__ st, double* __restrict__ out, int masked) {
  const long n = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (n >= g.nnodes) return;
  const int j = n % g.ny;
  const int k = (n / g.ny) % g.nz;
  const int i = n / ((long)g.ny * g.nz);
  const bool nfix = is_fixed(g, i, j);
  for (int m = 0; m < 27; m++) {
    const int mx = m / 9 - 1, mz = (m / 3) % 3 - 1, my = m % 3 - 1;
    const int mi = i + mx, mk = k + mz, mj = j + my;
    const bool minside = mi >= 0 && mi < g.nx && mk >= 0 && mk < g.nz && mj >= 0 && mj < g.ny;
    const bool zero = !minside || nfix || (masked && m != 13 && is_fixed(g, mi, mj));
    const long nm = minside ? ((long)mi * g.nz + mk) * g.ny + mj : n;
    for (int c = 0; c < 3; c++)
      for (int d = 0; d < 3; d++) {
        double v = 0.0;
        if (!zero) v = m >= 13 ? st[((long)(m - 13) * 9 + 3 * c + d) * g.nnodes + n]
                               : st[((long)(13 - m) * 9 + 3 * d + c) * g.nnodes + nm];
        if (nfix && m == 13 && c == d) v = 1.0;
        out[((long)m * 9 + 3 * c + d) * g.nnodes + n] = v;
      }
  }
}

void stencil_expand(tp_ctx* c, int l, const double* st, double* out, int masked) {
  const CGeom g = cgeom(c, l);
  stencil_expand_kernel<<<grid_for(g.nnodes, 128), 128, 0, c->s>>>(g, st, out, masked);
  TP_CHECK_LAUNCH(c, "stencil_expand");
}

// ---------------------------------------------------------------------------
// Full-weighting restriction, level l+1 <- level l (stencil_methods.c:595-688):
// the coarse node at fine (2i, 2j, 2k) gathers its 27 fine neighbours with
// weights 1, 1/2, 1/4, 1/8 by squared distance, in the reference's x, z, y
// loop order.
template <typename T>
__global__ void restrict_kernel(CGeom f, CGeom cg, const T* __restrict__ fine, T* __restrict__ coarse) {
  const long n = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (n >= cg.nnodes) return;
  fine += blockIdx.y * 3 * f.nnodes;  // column of this right-hand side
  coarse += blockIdx.y * 3 * cg.nnodes;
  const int jc = n % cg.ny;
  const int kc = (n / cg.ny) % cg.nz;
  const int ic = n / ((long)cg.ny * cg.nz);
  const int i1 = 2 * ic, j1 = 2 * jc, k1 = 2 * kc;
  T acc[3] = {T(0), T(0), T(0)};
  for (int i = i1 - 1; i < i1 + 2; i++)
    for (int k = k1 - 1; k < k1 + 2; k++)
      for (int j = j1 - 1; j < j1 + 2; j++) {
        if (i < 0 || i >= f.nx || j < 0 || j >= f.ny || k < 0 || k >= f.nz) continue;
        const int d2 = (i1 - i) * (i1 - i) + (j1 - j) * (j1 - j) + (k1 - k) * (k1 - k);
        const T w = d2 == 0 ? T(1.0) : d2 == 1 ? T(0.5) : d2 == 2 ? T(0.25) : T(0.125);
        const long nf = ((long)i * f.nz + k) * f.ny + j;
        acc[0] += w * fine[3 * nf];
        acc[1] += w * fine[3 * nf + 1];
        acc[2] += w * fine[3 * nf + 2];
      }
  coarse[3 * n] = acc[0];
  coarse[3 * n + 1] = acc[1];
  coarse[3 * n + 2] = acc[2];
}

// Trilinear prolongation, level l <- level l+1 (stencil_methods.c:521-590):
// each fine node averages the (possibly repeated) 8 coarse nodes
// (i>>1 | (i+1)>>1) x (j>>1 | (j+1)>>1) x (k>>1 | (k+1)>>1) with weight 1/8,
// summed in the reference's order. ADD adds the result to the fine vector.
template <typename T, bool ADD>
__global__ void prolong_kernel(CGeom f, CGeom cg, const T* __restrict__ coarse, T* __restrict__ fine) {
  const long n = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (n >= f.nnodes) return;
  fine += blockIdx.y * 3 * f.nnodes;
  coarse += blockIdx.y * 3 * cg.nnodes;
  const int j = n % f.ny;
  const int k = (n / f.ny) % f.nz;
  const int i = n / ((long)f.ny * f.nz);
  const int i1 = i >> 1, i2 = (i + 1) >> 1, j1 = j >> 1, j2 = (j + 1) >> 1, k1 = k >> 1, k2 = (k + 1) >> 1;
  auto cn = [&](int a, int b, int d) { return ((long)a * cg.nz + b) * cg.ny + d; };
  const long c1 = cn(i1, k1, j2), c2 = cn(i2, k1, j2), c3 = cn(i2, k1, j1), c4 = cn(i1, k1, j1),
             c5 = cn(i1, k2, j2), c6 = cn(i2, k2, j2), c7 = cn(i2, k2, j1), c8 = cn(i1, k2, j1);
  const T h = T(0.125);
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const T v = h * coarse[3 * c1 + c] + h * coarse[3 * c2 + c] + h * coarse[3 * c3 + c] +
                h * coarse[3 * c4 + c] + h * coarse[3 * c5 + c] + h * coarse[3 * c6 + c] +
                h * coarse[3 * c7 + c] + h * coarse[3 * c8 + c];
    if (ADD)
      fine[3 * n + c] += v;
    else
      fine[3 * n + c] = v;
  }
}

template <typename T>
void restrict_fw(tp_ctx* c, int l, const T* fine, T* coarse, int nr) {
  ProfScope ps(c, P_TRANSFER);
  const CGeom f = cgeom(c, l), cg = cgeom(c, l + 1);
  restrict_kernel<T><<<dim3(grid_for(cg.nnodes, 128), nr), 128, 0, c->s>>>(f, cg, fine, coarse);
  TP_CHECK_LAUNCH(c, "restrict");
}
template <typename T>
void prolong_add(tp_ctx* c, int l, const T* coarse, T* fine, int nr) {
  ProfScope ps(c, P_TRANSFER);
  const CGeom f = cgeom(c, l), cg = cgeom(c, l + 1);
  prolong_kernel<T, true><<<dim3(grid_for(f.nnodes, 128), nr), 128, 0, c->s>>>(f, cg, coarse, fine);
  TP_CHECK_LAUNCH(c, "prolong_add");
}
template <typename T>
void prolong_set(tp_ctx* c, int l, const T* coarse, T* fine, int nr) {
  ProfScope ps(c, P_TRANSFER);
  const CGeom f = cgeom(c, l), cg = cgeom(c, l + 1);
  prolong_kernel<T, false><<<dim3(grid_for(f.nnodes, 128), nr), 128, 0, c->s>>>(f, cg, coarse, fine);
  TP_CHECK_LAUNCH(c, "prolong_set");
}
template void restrict_fw<double>(tp_ctx*, int, const double*, double*, int);
template void restrict_fw<float>(tp_ctx*, int, const float*, float*, int);
template void prolong_add<double>(tp_ctx*, int, const double*, double*, int);
template void prolong_add<float>(tp_ctx*, int, const float*, float*, int);
template void prolong_set<double>(tp_ctx*, int, const double*, double*, int);
template void prolong_set<float>(tp_ctx*, int, const float*, float*, int);

}  // namespace tp
