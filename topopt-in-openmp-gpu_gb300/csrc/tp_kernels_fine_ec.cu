// Level-0 operator, element-centric and sum-factorised: the same
// y = K(rho) u as the hex8 stencil of stencil_methods.c:7-428, with the same
// fused consumers (CG matvec + dot, Jacobi sweep, residual), at about a third
// of the arithmetic.
//
// Basis. Per axis, the two nodal values of an element edge are replaced by
// their sum and difference. For the 8 nodes of an element this is the
// transform T8[b][q] = prod_axes s(bit_b, offset_q) with s(0, .) = 1,
// s(1, 0) = -1, s(1, 1) = +1, b = bx*4 + by*2 + bz; T8 T8^T = 8 I, so
//   KE = T^T KZ T,   KZ = T KE T^T / 64   (T = T8 (x) I_3).
// For the isotropic trilinear hexahedron KZ has 45 non-zeros out of 576 (row
// and column b = 0 -- rigid translations -- vanish); the host checks that
// pattern numerically when it builds KZ from KE. Per element the operator is
// then: three butterfly stages forward (y, x, z), 45 multiply-adds, three
// butterfly stages back, with E(rho) folded into the last accumulation.
//
// Schedule. One thread per element column in y (thread t <-> elements
// ej = t); a thread owns node column t+1 (thread 0 also column 0), and a z
// group of at most RMAX consecutive node rows. The CTA streams along x over
// a chunk of node planes: element layer L (between planes L and L+1) is
// computed from the two planes, its contributions complete plane L (which
// already holds layer L-1's share, carried in registers) and start plane
// L+1. Node planes of the CTA's rows (plus one halo row each side) and, for
// the sweep, the b and invD rows are staged in shared memory by cp.async,
// two planes ahead of the compute; the moduli E of the CTA's element rows
// one layer ahead, so no thread waits on a global load in the compute. The y-neighbour exchange is a warp
// shuffle; the column shared by two warps goes through shared memory.
// Halo work: one element row per z group and one element layer per x chunk
// are computed twice.
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "tp_dsf.cuh"
#include "tp_internal.h"

namespace tp {

__constant__ double c_kz[45];
__constant__ float c_kzf[45];
__constant__ float c_kzd[45][2];  // c_kz as double-single pairs
__constant__ float2 c_kz2[45];     // c_kzf as (k, k) pairs for the packed FP32 kernel

// storage type T <-> arithmetic type A of the element-centric kernel
template <typename A, typename T>
struct EcCvt {
  static __device__ __forceinline__ A in(T v) { return v; }
  static __device__ __forceinline__ T out(A v) { return v; }
};
template <>
struct EcCvt<Dsf, double> {
  static __device__ __forceinline__ Dsf in(double v) { return ds_from(v); }
  static __device__ __forceinline__ double out(Dsf v) { return ds_to(v); }
};
template <typename A>
__device__ __forceinline__ A ec_shfl_down(A v, int d) {
  return __shfl_down_sync(0xffffffffu, v, d);
}
__device__ __forceinline__ Dsf ec_shfl_down(Dsf v, int d) {
  return Dsf(__shfl_down_sync(0xffffffffu, v.h, d), __shfl_down_sync(0xffffffffu, v.l, d));
}

template <typename T>
__device__ __forceinline__ T kz(int i);
template <>
__device__ __forceinline__ double kz<double>(int i) { return c_kz[i]; }
template <>
__device__ __forceinline__ float kz<float>(int i) { return c_kzf[i]; }
template <>
__device__ __forceinline__ Dsf kz<Dsf>(int i) { return Dsf(c_kzd[i][0], c_kzd[i][1]); }

// (row, column) of the 45 non-zeros of KZ, row = 3*b + c, in the order the
// kernel consumes them
#define TP_KZ_PAIR(i, r, s) {r, s},
static const unsigned char kKzPattern[45][2] = {TP_KZ_PATTERN(TP_KZ_PAIR)};
#undef TP_KZ_PAIR

static int loc_node(int dx, int dy, int dz) { return dz * 4 + (dy ? (dx ? 1 : 0) : (dx ? 2 : 3)); }

bool set_fine_kz(const double* ke0, double* kz_out) {
  double t8[8][8];
  for (int b = 0; b < 8; b++)
    for (int dx = 0; dx < 2; dx++)
      for (int dy = 0; dy < 2; dy++)
        for (int dz = 0; dz < 2; dz++) {
          const int bits[3] = {(b >> 2) & 1, (b >> 1) & 1, b & 1}, off[3] = {dx, dy, dz};
          double w = 1.0;
          for (int a = 0; a < 3; a++)
            if (bits[a]) w *= off[a] ? 1.0 : -1.0;
          t8[b][loc_node(dx, dy, dz)] = w;
        }
  static double KZ[24][24];
  double mx = 0.0;
  for (int b = 0; b < 8; b++)
    for (int c = 0; c < 3; c++)
      for (int b2 = 0; b2 < 8; b2++)
        for (int c2 = 0; c2 < 3; c2++) {
          double s = 0.0;
          for (int q = 0; q < 8; q++)
            for (int q2 = 0; q2 < 8; q2++) s += t8[b][q] * ke0[(3 * q + c) * 24 + 3 * q2 + c2] * t8[b2][q2];
          KZ[3 * b + c][3 * b2 + c2] = s / 64.0;
          mx = std::fmax(mx, std::fabs(s / 64.0));
        }
  bool in_pat[24][24] = {};
  double v[45];
  float vf[45], vd[45][2];
  for (int i = 0; i < 45; i++) {
    in_pat[kKzPattern[i][0]][kKzPattern[i][1]] = true;
    v[i] = KZ[kKzPattern[i][0]][kKzPattern[i][1]];
    vf[i] = (float)v[i];
    vd[i][0] = vf[i];
    vd[i][1] = (float)(v[i] - (double)vf[i]);
  }
  bool ok = mx > 0.0;
  for (int r = 0; r < 24; r++)
    for (int s = 0; s < 24; s++)
      if (!in_pat[r][s] && std::fabs(KZ[r][s]) > 1e-12 * mx) ok = false;
  if (kz_out)
    for (int i = 0; i < 45; i++) kz_out[i] = v[i];
  if (ok) {
    cudaMemcpyToSymbol(c_kz, v, sizeof(v));
    cudaMemcpyToSymbol(c_kzf, vf, sizeof(vf));
    float2 v2[45];
    for (int i = 0; i < 45; i++) v2[i] = make_float2(vf[i], vf[i]);
    cudaMemcpyToSymbol(c_kz2, v2, sizeof(v2));
    cudaMemcpyToSymbol(c_kzd, vd, sizeof(vd));
  }
  return ok;
}

// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void* dst, const void* src, int bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Stage the contiguous range [src, src + n) into buf (16-byte aligned) in
// 16-byte chunks from the 16-byte boundary at or below src; element 0 lands
// at buf + (src & 15). The last chunk copies only the bytes inside the range
// (zero fill), so nothing past src + n is read. The caller guarantees that
// the bytes between the boundary and src belong to the same allocation (its
// base is 16-byte aligned).
template <typename T>
__device__ __forceinline__ void ec_stage(unsigned char* buf, const T* src, long n, int tid, int nthr) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(src);
  const uintptr_t a0 = a & ~uintptr_t(15);
  const uintptr_t ae = a + (uintptr_t)n * sizeof(T);
  const int nch = (int)((ae - a0 + 15) >> 4);
  for (int q = tid; q < nch; q += nthr) {
    const uintptr_t s = a0 + ((uintptr_t)q << 4);
    const uintptr_t rem = ae - s;
    cp_async16(buf + ((size_t)q << 4), reinterpret_cast<const void*>(s), rem < 16 ? (int)rem : 16);
  }
}
template <typename T>
__device__ __forceinline__ const T* ec_view(const unsigned char* buf, const T* src) {
  return reinterpret_cast<const T*>(buf + (reinterpret_cast<uintptr_t>(src) & 15));
}

__device__ __forceinline__ void ec_rows(const EcGeom& g, int gi, int& k0, int& k1) {
  k0 = gi * g.zbase + min(gi, g.zextra);
  k1 = k0 + g.zbase + (gi < g.zextra ? 1 : 0);
}

constexpr int EC_APPLY = FM_APPLY, EC_APPLY_DOT = FM_APPLY_DOT, EC_JACOBI = FM_JACOBI, EC_RESID = FM_RESID;

// T: the type of the vectors in memory; A: the type the operator is evaluated
// in (T itself, or Dsf for double vectors)
// MINB: CTAs per SM the register allocation is sized for (1: up to 255
// registers, the double-vector forms; 2: at most 128, the FP32 default;
// 3: at most 80, with a few spills, for three 256-thread CTAs per SM)
template <typename T, typename A, int MODE, int RMAX, int MINB, bool ES, bool PT>
__global__ void __launch_bounds__(256, MINB) fine_ec_kernel(EcGeom g, const T* __restrict__ E, const T* __restrict__ in,
                                                      T* __restrict__ out, const T* __restrict__ bv,
                                                      const T* __restrict__ invD, T omega,
                                                      double* __restrict__ partials) {
  constexpr int NST = 3;  // slab stages: planes L, L+1 in use, L+2 in flight
  // the items of the columns shared by warps, (ey/32 + 1) * rows * 3, fit one
  // per thread of a group when 3 * RMAX <= 16
  static_assert(3 * RMAX <= 16, "one shared-column item per thread");
  static_assert(sizeof(A) == sizeof(T), "shared-memory exchange arrays are sized for T");
  using Cv = EcCvt<A, T>;
  constexpr bool HASB = (MODE == EC_JACOBI || MODE == EC_RESID);
  constexpr bool HASD = (MODE == EC_JACOBI);
  extern __shared__ __align__(16) unsigned char smem[];
  const int t = threadIdx.x, tz = threadIdx.y;
  const int nyt = blockDim.x, nzg = blockDim.y;
  const int nthr = nyt * nzg, tid = t + nyt * tz;
  const int lane = t & 31, wy = t >> 5, nwy = nyt >> 5;
  const int ny = g.ny, nz = g.nz, ey = g.ey, ez = g.ez;
  const long row3 = 3L * ny;
  {
    const long rs = (long)blockIdx.z * g.vstride;
    in += rs;
    out += rs;
    if (HASB) bv += rs;
  }
  const int gfirst = blockIdx.x * nzg;
  const int glast = min(gfirst + nzg, g.ngz) - 1;
  int K0, K1, k0 = 0, k1 = 0, dum;
  ec_rows(g, gfirst, K0, dum);
  ec_rows(g, glast, dum, K1);
  const int gi = gfirst + tz;
  const bool gact = gi <= glast;
  if (gact) ec_rows(g, gi, k0, k1);
  const int nrow = k1 - k0;
  const int kmin = max(K0 - 1, 0), kmax = min(K1, nz - 1);
  const long slab_n = (long)(kmax - kmin + 1) * row3;
  const long own_n = (long)(K1 - K0) * row3;
  const int ekmin = max(K0 - 1, 0), ekmax = min(K1 - 1, ez - 1);  // element rows of the CTA
  const long e_n = (long)(ekmax - ekmin + 1) * ey;
  const bool stage_own = g.own_bytes > 0;

  const int i0 = blockIdx.y * g.cx;
  const int i1 = min(i0 + g.cx, g.nx);
  const int Ls = max(i0 - 1, 0), Le = min(i1, g.ex);  // element layers [Ls, Le), planes Ls..Le

  unsigned char* sl = smem;
  unsigned char* sb = sl + NST * g.slab_bytes;
  unsigned char* sd = sb + 2 * g.own_bytes;
  unsigned char* se = sd + 2 * g.own_bytes;
  A* bnd_nb = reinterpret_cast<A*>(se + 2 * g.e_bytes);    // [nzg][nwy][RMAX][6]
  A* bnd_own = bnd_nb + nzg * nwy * RMAX * 6;              // [nzg][nwy][RMAX][6]
  A* carry_b = bnd_own + nzg * nwy * RMAX * 6;             // [nzg][nwy + 1][RMAX][3]
  // FP32 sweeps and residuals: b and invD of the thread's own nodes in this
  // layer, copied by the thread itself when the layer starts, slot i of
  // thread tid at [i * nthr + tid], i = (r * 2 + array) * 3 + c
  T* slot = reinterpret_cast<T*>(carry_b + nzg * (nwy + 1) * RMAX * 3);
  constexpr bool own_pt = PT && HASB && sizeof(T) == 4;  // PT: the per-thread copies (plan staging 2)

  auto slab_src = [&](int p) { return in + ((long)p * nz + kmin) * row3; };
  auto own_src = [&](const T* v, int p) { return v + ((long)p * nz + K0) * row3; };
  auto issue_slab = [&](int p) { ec_stage<T>(sl + (p % NST) * g.slab_bytes, slab_src(p), slab_n, tid, nthr); };
  auto issue_own = [&](int p) {
    if (HASB && stage_own) ec_stage<T>(sb + (p & 1) * g.own_bytes, own_src(bv, p), own_n, tid, nthr);
    if (HASD && stage_own) ec_stage<T>(sd + (p & 1) * g.own_bytes, own_src(invD, p), own_n, tid, nthr);
  };
  auto e_src = [&](int L) { return E + ((long)L * ez + ekmin) * ey; };
  // ES: the moduli staged in shared memory one layer ahead; otherwise each
  // thread loads its own into registers when the layer starts
  auto issue_e = [&](int L) {
    if (ES) ec_stage<T>(se + (L & 1) * g.e_bytes, e_src(L), e_n, tid, nthr);
  };
  // views: value of node row kr, column j, component c at [(kr - base row) * row3 + 3 j + c]
  auto slab_at = [&](int p) { return ec_view<T>(sl + (p % NST) * g.slab_bytes, slab_src(p)); };

  for (int q = tid; q < nzg * (nwy + 1) * RMAX * 3; q += nthr) carry_b[q] = A(0);

  double dot = 0.0;
  // output components [c0, c1) of plane P, node row kr, column j
  auto epi = [&](const T* uP, const T* bP, const T* dP, int P, int kr, int j, int c0, int c1, const A* y,
                 bool from_slot) {
    if (P < i0) return;
    const long li = (long)(kr - kmin) * row3 + 3 * j;
    const long n3 = ((long)P * nz + kr) * row3 + 3 * j;
    const long lo = (long)(kr - K0) * row3 + 3 * j;
    const bool fixed = P == 0 && (j < g.lim || j >= ny - g.lim);  // identity rows
#pragma unroll
    for (int c = 0; c < 3; c++) {
      if (c < c0 || c >= c1) continue;
      const T u = uP[li + c];
      const T yc = fixed ? u : Cv::out(y[c]);
      if (MODE == EC_APPLY || MODE == EC_APPLY_DOT) out[n3 + c] = yc;
      if (MODE == EC_APPLY_DOT) dot += (double)u * (double)yc;
      if (HASB) {
        const int r = kr - k0;
        const T b = from_slot ? slot[((r * 2 + 0) * 3 + c) * nthr + tid] : stage_own ? bP[lo + c] : bv[n3 + c];
        if (MODE == EC_RESID) out[n3 + c] = b - yc;
        if (MODE == EC_JACOBI) {
          const T d = from_slot ? slot[((r * 2 + 1) * 3 + c) * nthr + tid] : stage_own ? dP[lo + c] : invD[n3 + c];
          out[n3 + c] = u + omega * d * (b - yc);
        }
      }
    }
  };
  // the columns shared by two warps (0, 32, 64, ...): one (column, row,
  // component) item per thread of the group, fixed for the whole launch
  const int ncb = ey / 32 + 1;
  const bool tail = gact && t < ncb * nrow * 3;
  const int tc = tail ? t % 3 : 0, tr = tail ? (t / 3) % nrow : 0, tcb = tail ? t / (3 * nrow) : 0;
  auto own_at = [&](unsigned char* base, const T* v, int p) -> const T* {
    if (!stage_own) return nullptr;
    return ec_view<T>(base + (p & 1) * g.own_bytes, own_src(v, p));
  };

  issue_slab(Ls);
  issue_slab(Ls + 1);
  issue_own(Ls);
  issue_e(Ls);
  cp_async_commit();

  A carry[RMAX][3];
#pragma unroll
  for (int r = 0; r < RMAX; r++) carry[r][0] = carry[r][1] = carry[r][2] = A(0);
  const bool lact = gact && t < ey;
  const bool pt_thread = own_pt && lact && lane != 31;
  auto issue_pt = [&](int L) {
    if constexpr (own_pt) {
      if (!pt_thread || L < i0) return;
#pragma unroll
      for (int r = 0; r < RMAX; r++) {
        if (r >= nrow) break;
        const long n = (((long)L * nz + k0 + r) * ny + t + 1) * 3;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          cp_async4(&slot[((r * 2 + 0) * 3 + c) * nthr + tid], bv + n + c);
          if (HASD) cp_async4(&slot[((r * 2 + 1) * 3 + c) * nthr + tid], invD + n + c);
        }
      }
    }
  };

  for (int L = Ls; L < Le; ++L) {
    if constexpr (own_pt) {
      issue_pt(L);
      cp_async_commit();
    }
    if (L + 2 <= Le) issue_slab(L + 2);
    if (L + 1 <= Le) issue_own(L + 1);
    if (L + 1 < Le) issue_e(L + 1);
    cp_async_commit();
    // the next stages (and this layer's slot copies) may still be in flight
    cp_async_wait<own_pt ? 2 : 1>();
    __syncthreads();
    // E of element row ek of layer L at EL[(ek - ekmin) * ey + t]
    const T* EL = ES ? ec_view<T>(se + (L & 1) * g.e_bytes, e_src(L)) + t : e_src(L) + t;
    A Ev[RMAX + 1];
    if (!ES) {
#pragma unroll
      for (int q = 0; q <= RMAX; q++) {
        const int ek = k0 - 1 + q;
        Ev[q] = (lact && q <= nrow && ek >= 0 && ek < ez) ? Cv::in(EL[(long)(ek - ekmin) * ey]) : A(0);
      }
    }
    const T* u0 = slab_at(L);
    const T* u1 = slab_at(L + 1);
    const T* bL = HASB ? own_at(sb, bv, L) : nullptr;
    const T* dL = HASD ? own_at(sd, invD, L) : nullptr;

    if (gact) {
      // y and x butterflies of node row kr: X[(bx*2 + by)*3 + c]
      auto xrow = [&](int kr, A* X) {
        if (lact && kr >= 0 && kr < nz) {
          const long o = (long)(kr - kmin) * row3 + 3 * t;
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const A a0 = Cv::in(u0[o + c]), a1 = Cv::in(u0[o + 3 + c]);
            const A b0 = Cv::in(u1[o + c]), b1 = Cv::in(u1[o + 3 + c]);
            const A s0 = a0 + a1, d0 = a1 - a0, s1 = b0 + b1, d1 = b1 - b0;
            X[c] = s0 + s1;
            X[3 + c] = d0 + d1;
            X[6 + c] = s1 - s0;
            X[9 + c] = d1 - d0;
          }
        } else {
#pragma unroll
          for (int a = 0; a < 12; a++) X[a] = A(0);
        }
      };
      A Xp[12], Xn[12], accp[12], accn[12];
      xrow(k0 - 1, Xp);
#pragma unroll
      for (int a = 0; a < 12; a++) accp[a] = A(0);
      // Unrolled, the double-single body (each operation 4 to 8 FP32
      // instructions, ~2.4k per row) outgrows the instruction cache: it stays
      // a loop, and the carries and moduli it indexes by row live in local
      // memory.
      auto row_step = [&](int q) {
        const int ek = k0 - 1 + q;
        xrow(ek + 1, Xn);
        if (ek >= 0 && ek < ez) {
          const A Ee = ES ? (lact ? Cv::in(EL[(long)(ek - ekmin) * ey]) : A(0)) : Ev[q];
          A Z[24];
#pragma unroll
          for (int a = 0; a < 4; a++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
              // a = bx*2 + by  ->  b = bx*4 + by*2 + bz = 2a + bz
              Z[(2 * a) * 3 + c] = Xp[a * 3 + c] + Xn[a * 3 + c];
              Z[(2 * a + 1) * 3 + c] = Xn[a * 3 + c] - Xp[a * 3 + c];
            }
          // w = KZ Z, pairs (bz = 0, 1) of each (bx, by, c); node row ek takes
          // E (w0 - w1), node row ek + 1 takes E (w0 + w1)
          {
            const A w1 = kz<A>(0) * Z[3] + kz<A>(1) * Z[14];
            accp[0] -= Ee * w1;
            accn[0] = Ee * w1;
          }
          {
            const A w1 = kz<A>(2) * Z[4] + kz<A>(3) * Z[8];
            accp[1] -= Ee * w1;
            accn[1] = Ee * w1;
          }
          {
            const A w1 = kz<A>(4) * Z[5] + kz<A>(5) * Z[7] + kz<A>(6) * Z[12];
            accp[2] -= Ee * w1;
            accn[2] = Ee * w1;
          }
          {
            const A w0 = kz<A>(7) * Z[6] + kz<A>(8) * Z[13];
            const A w1 = kz<A>(9) * Z[9] + kz<A>(10) * Z[16] + kz<A>(11) * Z[20];
            accp[3] += Ee * (w0 - w1);
            accn[3] = Ee * (w0 + w1);
          }
          {
            const A w0 = kz<A>(12) * Z[5] + kz<A>(13) * Z[7] + kz<A>(14) * Z[12];
            const A w1 = kz<A>(15) * Z[10] + kz<A>(16) * Z[15];
            accp[4] += Ee * (w0 - w1);
            accn[4] = Ee * (w0 + w1);
          }
          {
            const A w0 = kz<A>(17) * Z[4] + kz<A>(18) * Z[8];
            const A w1 = kz<A>(19) * Z[11] + kz<A>(20) * Z[18];
            accp[5] += Ee * (w0 - w1);
            accn[5] = Ee * (w0 + w1);
          }
          {
            const A w0 = kz<A>(21) * Z[5] + kz<A>(22) * Z[7] + kz<A>(23) * Z[12];
            const A w1 = kz<A>(24) * Z[10] + kz<A>(25) * Z[15];
            accp[6] += Ee * (w0 - w1);
            accn[6] = Ee * (w0 + w1);
          }
          {
            const A w0 = kz<A>(26) * Z[6] + kz<A>(27) * Z[13];
            const A w1 = kz<A>(28) * Z[9] + kz<A>(29) * Z[16] + kz<A>(30) * Z[20];
            accp[7] += Ee * (w0 - w1);
            accn[7] = Ee * (w0 + w1);
          }
          {
            const A w0 = kz<A>(31) * Z[3] + kz<A>(32) * Z[14];
            const A w1 = kz<A>(33) * Z[17] + kz<A>(34) * Z[19];
            accp[8] += Ee * (w0 - w1);
            accn[8] = Ee * (w0 + w1);
          }
          {
            const A w0 = kz<A>(35) * Z[11] + kz<A>(36) * Z[18];
            const A w1 = kz<A>(37) * Z[21];
            accp[9] += Ee * (w0 - w1);
            accn[9] = Ee * (w0 + w1);
          }
          {
            const A w0 = kz<A>(38) * Z[17] + kz<A>(39) * Z[19];
            const A w1 = kz<A>(40) * Z[22];
            accp[10] += Ee * (w0 - w1);
            accn[10] = Ee * (w0 + w1);
          }
          {
            const A w0 = kz<A>(41) * Z[9] + kz<A>(42) * Z[16] + kz<A>(43) * Z[20];
            const A w1 = kz<A>(44) * Z[23];
            accp[11] += Ee * (w0 - w1);
            accn[11] = Ee * (w0 + w1);
          }
        } else {
#pragma unroll
          for (int a = 0; a < 12; a++) accn[a] = A(0);
        }
        if (q >= 1) {
          // node row ek = k0 + r is complete: x and y butterflies back
          const int r = q - 1;
          if constexpr (own_pt)
            if (q == 1) cp_async_wait<1>();  // the thread's slot copies of this layer
          A own0[3], own1[3], nb0[3], nb1[3];
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const A p0s = accp[c] - accp[6 + c], p0d = accp[3 + c] - accp[9 + c];
            const A p1s = accp[c] + accp[6 + c], p1d = accp[3 + c] + accp[9 + c];
            own0[c] = p0s + p0d;  // plane L,   column t + 1
            own1[c] = p1s + p1d;  // plane L+1, column t + 1
            nb0[c] = p0s - p0d;   // plane L,   column t
            nb1[c] = p1s - p1d;   // plane L+1, column t
          }
          A rv0[3], rv1[3];
#pragma unroll
          for (int c = 0; c < 3; c++) {
            rv0[c] = ec_shfl_down(nb0[c], 1);
            rv1[c] = ec_shfl_down(nb1[c], 1);
          }
          const int bo = ((tz * nwy + wy) * RMAX + r) * 6;
          if (lane == 0) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
              bnd_nb[bo + c] = nb0[c];
              bnd_nb[bo + 3 + c] = nb1[c];
            }
          }
          if (lane == 31) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
              bnd_own[bo + c] = own0[c];
              bnd_own[bo + 3 + c] = own1[c];
            }
          } else if (lact) {
            A y[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
              y[c] = carry[r][c] + own0[c] + rv0[c];
              carry[r][c] = own1[c] + rv1[c];
            }
            epi(u0, bL, dL, L, k0 + r, t + 1, 0, 3, y, own_pt);
          }
        }
#pragma unroll
        for (int a = 0; a < 12; a++) {
          Xp[a] = Xn[a];
          accp[a] = accn[a];
        }
      };
      if constexpr (std::is_same<A, Dsf>::value) {
#pragma unroll 1
        for (int q = 0; q <= RMAX; q++) {
          if (q > nrow) break;
          row_step(q);
        }
      } else {
#pragma unroll
        for (int q = 0; q <= RMAX; q++) {
          if (q > nrow) break;
          row_step(q);
        }
      }
    }
    __syncthreads();
    // columns 0, 32, 64, ...: the own share of lane 31 of the warp on the
    // left plus the share of lane 0 of the warp on the right
    if (tail) {
      const int j = 32 * tcb;
      A o0 = A(0), o1 = A(0), n0 = A(0), n1 = A(0);
      if (tcb >= 1) {
        const int bo = ((tz * nwy + tcb - 1) * RMAX + tr) * 6;
        o0 = bnd_own[bo + tc];
        o1 = bnd_own[bo + 3 + tc];
      }
      if (j < ey) {
        const int bo = ((tz * nwy + tcb) * RMAX + tr) * 6;
        n0 = bnd_nb[bo + tc];
        n1 = bnd_nb[bo + 3 + tc];
      }
      A& cr = carry_b[((tz * (nwy + 1) + tcb) * RMAX + tr) * 3 + tc];
      const A v = cr + o0 + n0;
      cr = o1 + n1;
      const A y[3] = {v, v, v};  // only component tc is stored
      epi(u0, bL, dL, L, k0 + tr, j, tc, tc + 1, y, false);
    }
    __syncthreads();
  }
  cp_async_wait<0>();
  __syncthreads();
  if (i1 == g.nx && gact) {
    // last plane (x = nelx): only layer nelx-1 touches it, its share is the carry
    const int P = g.ex;
    const T* uP = slab_at(P);
    const T* bP = HASB ? own_at(sb, bv, P) : nullptr;
    const T* dP = HASD ? own_at(sd, invD, P) : nullptr;
    if (lact && lane != 31) {
#pragma unroll
      for (int r = 0; r < RMAX; r++)
        if (r < nrow) epi(uP, bP, dP, P, k0 + r, t + 1, 0, 3, carry[r], false);
    }
    if (tail) {
      const A v = carry_b[((tz * (nwy + 1) + tcb) * RMAX + tr) * 3 + tc];
      const A y[3] = {v, v, v};
      epi(uP, bP, dP, P, k0 + tr, 32 * tcb, tc, tc + 1, y, false);
    }
  }
  if (MODE == EC_APPLY_DOT) {
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
    __syncthreads();
    if (lane == 0) red[tid >> 5] = dot;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < nthr / 32; w++) s += red[w];
      partials[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 sweep, residual and product with packed arithmetic. The schedule and
// the arithmetic are those of fine_ec_kernel, but each thread carries two z
// groups of its CTA (groups 2 tz and 2 tz + 1, "lanes" A and B) as the two
// halves of float2 values, so every add, multiply and multiply-add of the
// operator is one f32x2 instruction (sm_100 and later) for two elements. A
// lane's rows outside its group, and element rows outside the grid, get the
// modulus E = 0 and read their node values from a clamped (valid) row of the
// staged slab: they contribute exact zeros, and the arithmetic needs no
// per-lane branch. Indices are 32-bit (the plan requires 3 * nodes < 2^31).
__device__ __forceinline__ float2 pk_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 pk_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 pk_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pk_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 pk_shfl_down(float2 v, int d) {
  return make_float2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
}

template <int MODE, int RMAX, int MINB>
__global__ void __launch_bounds__(256, MINB) fine_pk_kernel(EcGeom g, const float* __restrict__ E,
                                                            const float* __restrict__ in, float* __restrict__ out,
                                                            const float* __restrict__ bv,
                                                            const float* __restrict__ invD, float omega) {
  constexpr int NST = 3;  // slab stages: planes L, L+1 in use, L+2 in flight
  static_assert(3 * RMAX <= 16, "one shared-column item per thread");
  static_assert(MODE != EC_APPLY_DOT, "the packed kernel has no dot product");
  constexpr bool HASB = (MODE == EC_JACOBI || MODE == EC_RESID);
  constexpr bool HASD = (MODE == EC_JACOBI);
  extern __shared__ __align__(16) unsigned char smem[];
  const int t = threadIdx.x, tz = threadIdx.y;
  const int nyt = blockDim.x, npr = blockDim.y, nzg = 2 * npr;
  const int nthr = nyt * npr, tid = t + nyt * tz;
  const int lane = t & 31, nwy = nyt >> 5;
  const int ny = g.ny, nz = g.nz, ey = g.ey, ez = g.ez;
  const int row3 = 3 * ny;
  {
    const long rs = (long)blockIdx.z * g.vstride;
    in += rs;
    out += rs;
    if (HASB) bv += rs;
  }
  const int gfirst = blockIdx.x * nzg;
  const int glast = min(gfirst + nzg, g.ngz) - 1;
  int K0, K1, dum;
  ec_rows(g, gfirst, K0, dum);
  ec_rows(g, glast, dum, K1);
  // lane A: group gfirst + 2 tz, lane B: the next one; a missing group has
  // the empty row range [K1, K1)
  int k0A = K1, k1A = K1, k0B = K1, k1B = K1;
  if (gfirst + 2 * tz <= glast) ec_rows(g, gfirst + 2 * tz, k0A, k1A);
  if (gfirst + 2 * tz + 1 <= glast) ec_rows(g, gfirst + 2 * tz + 1, k0B, k1B);
  const int nrowA = k1A - k0A, nrowB = k1B - k0B;
  const int nrow = max(nrowA, nrowB);
  const bool tact = nrow > 0;
  const int kmin = max(K0 - 1, 0), kmax = min(K1, nz - 1);
  const int slab_n = (kmax - kmin + 1) * row3;
  const int own_n = (K1 - K0) * row3;
  const int ekmin = max(K0 - 1, 0), ekmax = min(K1 - 1, ez - 1);
  const int e_n = (ekmax - ekmin + 1) * ey;
  const bool stage_own = g.own_bytes > 0;

  const int i0 = blockIdx.y * g.cx;
  const int i1 = min(i0 + g.cx, g.nx);
  const int Ls = max(i0 - 1, 0), Le = min(i1, g.ex);

  unsigned char* sl = smem;
  unsigned char* sb = sl + NST * g.slab_bytes;
  unsigned char* sd = sb + 2 * g.own_bytes;
  unsigned char* se = sd + 2 * g.own_bytes;
  float2* bnd_nb = reinterpret_cast<float2*>(se + 2 * g.e_bytes);  // [npr][nwy][RMAX][6]
  float2* bnd_own = bnd_nb + npr * nwy * RMAX * 6;                  // [npr][nwy][RMAX][6]
  float2* carry_b = bnd_own + npr * nwy * RMAX * 6;                 // [npr][nwy + 1][RMAX][3]
  // b and invD of the thread's own nodes in this layer, copied by the thread
  // itself when the layer starts: slot i of thread tid at [i * nthr + tid],
  // i = ((r * 2 + array) * 3 + c) * 2 + lane
  float* slot = reinterpret_cast<float*>(carry_b + npr * (nwy + 1) * RMAX * 3);
  const bool own_pt = HASB && g.pt_bytes > 0;

  auto slab_src = [&](int p) { return in + ((long)p * nz + kmin) * row3; };
  auto own_src = [&](const float* v, int p) { return v + ((long)p * nz + K0) * row3; };
  auto e_src = [&](int L) { return E + ((long)L * ez + ekmin) * ey; };
  auto issue_slab = [&](int p) { ec_stage<float>(sl + (p % NST) * g.slab_bytes, slab_src(p), slab_n, tid, nthr); };
  auto issue_own = [&](int p) {
    if (HASB && stage_own) ec_stage<float>(sb + (p & 1) * g.own_bytes, own_src(bv, p), own_n, tid, nthr);
    if (HASD && stage_own) ec_stage<float>(sd + (p & 1) * g.own_bytes, own_src(invD, p), own_n, tid, nthr);
  };
  auto issue_e = [&](int L) { ec_stage<float>(se + (L & 1) * g.e_bytes, e_src(L), e_n, tid, nthr); };
  auto slab_at = [&](int p) { return ec_view<float>(sl + (p % NST) * g.slab_bytes, slab_src(p)); };
  auto own_at = [&](unsigned char* base, const float* v, int p) -> const float* {
    if (!stage_own) return nullptr;
    return ec_view<float>(base + (p & 1) * g.own_bytes, own_src(v, p));
  };
  for (int q = tid; q < npr * (nwy + 1) * RMAX * 3; q += nthr) carry_b[q] = make_float2(0.f, 0.f);

  const float2 om2 = make_float2(omega, omega);
  // output components [c0, c1) of plane P, node row r of both lanes, column j;
  // from_slot: b and invD from the thread's slots (its own column t + 1)
  auto epi = [&](const float* uP, const float* bP, const float* dP, int P, int r, int j, int c0, int c1,
                 const float2* y, bool from_slot) {
    if (P < i0) return;
    const bool vA = r < nrowA, vB = r < nrowB;
    // rows of a lane past its group are read clamped (and not stored)
    const int krA = min(k0A + r, K1 - 1), krB = min(k0B + r, K1 - 1);
    const int liA = (krA - kmin) * row3 + 3 * j, liB = (krB - kmin) * row3 + 3 * j;
    const int loA = (krA - K0) * row3 + 3 * j, loB = (krB - K0) * row3 + 3 * j;
    const int nA = ((P * nz + krA) * ny + j) * 3, nB = ((P * nz + krB) * ny + j) * 3;
    const bool fixed = P == 0 && (j < g.lim || j >= ny - g.lim);  // identity rows
#pragma unroll
    for (int c = 0; c < 3; c++) {
      if (c < c0 || c >= c1) continue;
      const float2 u = make_float2(uP[liA + c], uP[liB + c]);
      const float2 yc = fixed ? u : y[c];
      float2 o = yc;
      if (HASB) {
        const int sb0 = ((r * 2 + 0) * 3 + c) * 2, sd0 = ((r * 2 + 1) * 3 + c) * 2;
        const float2 b = from_slot ? make_float2(slot[sb0 * nthr + tid], slot[(sb0 + 1) * nthr + tid])
                         : stage_own ? make_float2(bP[loA + c], bP[loB + c])
                                     : make_float2(bv[nA + c], bv[nB + c]);
        const float2 rr = pk_sub(b, yc);
        if (MODE == EC_RESID) o = rr;
        if (MODE == EC_JACOBI) {
          const float2 d = from_slot ? make_float2(slot[sd0 * nthr + tid], slot[(sd0 + 1) * nthr + tid])
                           : stage_own ? make_float2(dP[loA + c], dP[loB + c])
                                       : make_float2(invD[nA + c], invD[nB + c]);
          o = pk_fma(pk_mul(om2, d), rr, u);
        }
      }
      if (vA) out[nA + c] = o.x;
      if (vB) out[nB + c] = o.y;
    }
  };
  // the columns shared by two warps (0, 32, 64, ...): one (column, row,
  // component) item per thread of the thread row, both lanes at once
  const int ncb = ey / 32 + 1;
  const bool tail = tact && t < ncb * nrow * 3;
  const int tc = tail ? t % 3 : 0, tr = tail ? (t / 3) % nrow : 0, tcb = tail ? t / (3 * nrow) : 0;

  issue_slab(Ls);
  issue_slab(Ls + 1);
  issue_own(Ls);
  issue_e(Ls);
  cp_async_commit();

  float2 carry[RMAX][3];
#pragma unroll
  for (int r = 0; r < RMAX; r++) carry[r][0] = carry[r][1] = carry[r][2] = make_float2(0.f, 0.f);
  const bool lact = tact && t < ey;
  const int tt = min(t, ey - 1);  // column pair read by the thread (an idle thread reads a valid one)
  // the thread's own b and invD entries of plane L (column t + 1, rows of both lanes)
  const bool pt_thread = own_pt && lact && lane != 31;
  auto issue_pt = [&](int L) {
    if (!pt_thread || L < i0) return;
#pragma unroll
    for (int r = 0; r < RMAX; r++)
#pragma unroll
      for (int ln = 0; ln < 2; ln++) {
        if (r >= (ln ? nrowB : nrowA)) continue;
        const long n = (((long)L * nz + (ln ? k0B : k0A) + r) * ny + t + 1) * 3;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          cp_async4(&slot[(((r * 2 + 0) * 3 + c) * 2 + ln) * nthr + tid], bv + n + c);
          if (HASD) cp_async4(&slot[(((r * 2 + 1) * 3 + c) * 2 + ln) * nthr + tid], invD + n + c);
        }
      }
  };

  for (int L = Ls; L < Le; ++L) {
    issue_pt(L);
    cp_async_commit();
    if (L + 2 <= Le) issue_slab(L + 2);
    if (L + 1 <= Le) issue_own(L + 1);
    if (L + 1 < Le) issue_e(L + 1);
    cp_async_commit();
    cp_async_wait<2>();  // this layer's slot copies and the next stages may still be in flight
    __syncthreads();
    const float* EL = ec_view<float>(se + (L & 1) * g.e_bytes, e_src(L)) + tt;
    const float* u0 = slab_at(L);
    const float* u1 = slab_at(L + 1);
    const float* bL = HASB ? own_at(sb, bv, L) : nullptr;
    const float* dL = HASD ? own_at(sd, invD, L) : nullptr;

    if (tact) {
      // y and x butterflies of node rows krA, krB: X[(bx*2 + by)*3 + c]
      auto xrow = [&](int krA, int krB, float2* X) {
        const int oA = (min(max(krA, kmin), kmax) - kmin) * row3 + 3 * tt;
        const int oB = (min(max(krB, kmin), kmax) - kmin) * row3 + 3 * tt;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const float2 a0 = make_float2(u0[oA + c], u0[oB + c]), a1 = make_float2(u0[oA + 3 + c], u0[oB + 3 + c]);
          const float2 b0 = make_float2(u1[oA + c], u1[oB + c]), b1 = make_float2(u1[oA + 3 + c], u1[oB + 3 + c]);
          const float2 s0 = pk_add(a0, a1), d0 = pk_sub(a1, a0), s1 = pk_add(b0, b1), d1 = pk_sub(b1, b0);
          X[c] = pk_add(s0, s1);
          X[3 + c] = pk_add(d0, d1);
          X[6 + c] = pk_sub(s1, s0);
          X[9 + c] = pk_sub(d1, d0);
        }
      };
      // modulus of element row k0 - 1 + q of each lane (0 outside its group or the grid)
      auto emod = [&](int q) {
        const int eA = k0A - 1 + q, eB = k0B - 1 + q;
        const bool okA = lact && q <= nrowA && eA >= 0 && eA < ez;
        const bool okB = lact && q <= nrowB && eB >= 0 && eB < ez;
        return make_float2(okA ? EL[(eA - ekmin) * ey] : 0.f, okB ? EL[(eB - ekmin) * ey] : 0.f);
      };
      float2 Xp[12], Xn[12], accp[12], accn[12];
      xrow(k0A - 1, k0B - 1, Xp);
#pragma unroll
      for (int a = 0; a < 12; a++) accp[a] = make_float2(0.f, 0.f);
#define PK_K(i) c_kz2[i]
#define PK_D2(i, a, j, b) pk_fma(PK_K(j), Z[b], pk_mul(PK_K(i), Z[a]))
#define PK_D3(i, a, j, b, k, c) pk_fma(PK_K(k), Z[c], PK_D2(i, a, j, b))
#define PK_ONE(q, w1)                  \
  {                                    \
    const float2 w = w1;               \
    accp[q] = pk_fma(nE, w, accp[q]);  \
    accn[q] = pk_mul(Ee, w);           \
  }
#define PK_TWO(q, w0e, w1e)                                \
  {                                                        \
    const float2 w0 = w0e, w1 = w1e;                       \
    accp[q] = pk_fma(Ee, pk_sub(w0, w1), accp[q]);         \
    accn[q] = pk_mul(Ee, pk_add(w0, w1));                  \
  }
#pragma unroll
      for (int q = 0; q <= RMAX; q++) {
        if (q > nrow) break;
        xrow(k0A + q, k0B + q, Xn);
        const float2 Ee = emod(q);
        const float2 nE = make_float2(-Ee.x, -Ee.y);
        float2 Z[24];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int c = 0; c < 3; c++) {
            // a = bx*2 + by  ->  b = bx*4 + by*2 + bz = 2a + bz
            Z[(2 * a) * 3 + c] = pk_add(Xp[a * 3 + c], Xn[a * 3 + c]);
            Z[(2 * a + 1) * 3 + c] = pk_sub(Xn[a * 3 + c], Xp[a * 3 + c]);
          }
        // w = KZ Z by pairs (bz = 0, 1) of each (bx, by, c): node row ek takes
        // E (w0 - w1), node row ek + 1 takes E (w0 + w1)
        PK_ONE(0, PK_D2(0, 3, 1, 14));
        PK_ONE(1, PK_D2(2, 4, 3, 8));
        PK_ONE(2, PK_D3(4, 5, 5, 7, 6, 12));
        PK_TWO(3, PK_D2(7, 6, 8, 13), PK_D3(9, 9, 10, 16, 11, 20));
        PK_TWO(4, PK_D3(12, 5, 13, 7, 14, 12), PK_D2(15, 10, 16, 15));
        PK_TWO(5, PK_D2(17, 4, 18, 8), PK_D2(19, 11, 20, 18));
        PK_TWO(6, PK_D3(21, 5, 22, 7, 23, 12), PK_D2(24, 10, 25, 15));
        PK_TWO(7, PK_D2(26, 6, 27, 13), PK_D3(28, 9, 29, 16, 30, 20));
        PK_TWO(8, PK_D2(31, 3, 32, 14), PK_D2(33, 17, 34, 19));
        PK_TWO(9, PK_D2(35, 11, 36, 18), pk_mul(PK_K(37), Z[21]));
        PK_TWO(10, PK_D2(38, 17, 39, 19), pk_mul(PK_K(40), Z[22]));
        PK_TWO(11, PK_D3(41, 9, 42, 16, 43, 20), pk_mul(PK_K(44), Z[23]));
        if (q >= 1) {
          // node row k0 + r of each lane is complete: x and y butterflies back
          const int r = q - 1;
          if (q == 1) cp_async_wait<1>();  // the thread's slot copies of this layer
          float2 own0[3], own1[3], nb0[3], nb1[3];
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const float2 p0s = pk_sub(accp[c], accp[6 + c]), p0d = pk_sub(accp[3 + c], accp[9 + c]);
            const float2 p1s = pk_add(accp[c], accp[6 + c]), p1d = pk_add(accp[3 + c], accp[9 + c]);
            own0[c] = pk_add(p0s, p0d);  // plane L,   column t + 1
            own1[c] = pk_add(p1s, p1d);  // plane L+1, column t + 1
            nb0[c] = pk_sub(p0s, p0d);   // plane L,   column t
            nb1[c] = pk_sub(p1s, p1d);   // plane L+1, column t
          }
          float2 rv0[3], rv1[3];
#pragma unroll
          for (int c = 0; c < 3; c++) {
            rv0[c] = pk_shfl_down(nb0[c], 1);
            rv1[c] = pk_shfl_down(nb1[c], 1);
          }
          const int bo = ((tz * nwy + (t >> 5)) * RMAX + r) * 6;
          if (lane == 0) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
              bnd_nb[bo + c] = nb0[c];
              bnd_nb[bo + 3 + c] = nb1[c];
            }
          }
          if (lane == 31) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
              bnd_own[bo + c] = own0[c];
              bnd_own[bo + 3 + c] = own1[c];
            }
          } else if (lact) {
            float2 y[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
              y[c] = pk_add(pk_add(carry[r][c], own0[c]), rv0[c]);
              carry[r][c] = pk_add(own1[c], rv1[c]);
            }
            epi(u0, bL, dL, L, r, t + 1, 0, 3, y, own_pt);
          }
        }
#pragma unroll
        for (int a = 0; a < 12; a++) {
          Xp[a] = Xn[a];
          accp[a] = accn[a];
        }
      }
#undef PK_TWO
#undef PK_ONE
#undef PK_D3
#undef PK_D2
#undef PK_K
    }
    __syncthreads();
    // columns 0, 32, 64, ...: the own share of lane 31 of the warp on the
    // left plus the share of lane 0 of the warp on the right
    if (tail) {
      const int j = 32 * tcb;
      float2 o0 = make_float2(0.f, 0.f), o1 = o0, n0 = o0, n1 = o0;
      if (tcb >= 1) {
        const int bo = ((tz * nwy + tcb - 1) * RMAX + tr) * 6;
        o0 = bnd_own[bo + tc];
        o1 = bnd_own[bo + 3 + tc];
      }
      if (j < ey) {
        const int bo = ((tz * nwy + tcb) * RMAX + tr) * 6;
        n0 = bnd_nb[bo + tc];
        n1 = bnd_nb[bo + 3 + tc];
      }
      float2& cr = carry_b[((tz * (nwy + 1) + tcb) * RMAX + tr) * 3 + tc];
      const float2 v = pk_add(pk_add(cr, o0), n0);
      cr = pk_add(o1, n1);
      const float2 y[3] = {v, v, v};  // only component tc is stored
      epi(u0, bL, dL, L, tr, j, tc, tc + 1, y, false);
    }
    __syncthreads();
  }
  cp_async_wait<0>();
  __syncthreads();
  if (i1 == g.nx && tact) {
    // last plane (x = nelx): only layer nelx-1 touches it, its share is the carry
    const int P = g.ex;
    const float* uP = slab_at(P);
    const float* bP = HASB ? own_at(sb, bv, P) : nullptr;
    const float* dP = HASD ? own_at(sd, invD, P) : nullptr;
    if (lact && lane != 31) {
#pragma unroll
      for (int r = 0; r < RMAX; r++)
        if (r < nrow) epi(uP, bP, dP, P, r, t + 1, 0, 3, carry[r], false);
    }
    if (tail) {
      const float2 v = carry_b[((tz * (nwy + 1) + tcb) * RMAX + tr) * 3 + tc];
      const float2 y[3] = {v, v, v};
      epi(uP, bP, dP, P, tr, 32 * tcb, tc, tc + 1, y, false);
    }
  }
}

// ---------------------------------------------------------------------------
// host side: plan, shared-memory size, launch

constexpr int kEcRmax = 5;

static long roundup16(long b) { return (b + 15) / 16 * 16; }

// shape-only part of the plan (no launch); false if the grid is outside the
// kernel's envelope (nely + 1 columns in one CTA of at most 256 threads)
bool ec_plan(tp_ctx* c, int nzg, int ncx, EcPlan* P) {
  const Level& L = c->L[0];
  EcPlan p;
  p.nyt = (L.ey + 31) / 32 * 32;
  if (p.nyt > 256 || L.ex < 1 || L.ey < 1 || L.ez < 1) return false;
  p.nzg = std::max(1, std::min(nzg, 256 / p.nyt));
  p.ngz = (L.nz + kEcRmax - 1) / kEcRmax;
  p.zbase = L.nz / p.ngz;
  p.zextra = L.nz % p.ngz;
  if (p.zbase + (p.zextra > 0) > kEcRmax) return false;
  p.ncx = std::max(1, std::min(ncx, L.nx));
  p.cx = (L.nx + p.ncx - 1) / p.ncx;
  p.ncx = (L.nx + p.cx - 1) / p.cx;
  p.ok = true;
  *P = p;
  return true;
}

// plan of the packed FP32 kernel: npr thread rows of two z groups each
static bool pk_plan(tp_ctx* c, int npr, int ncx, EcPlan* P) {
  EcPlan p;
  if (!ec_plan(c, 1, ncx, &p)) return false;
  if (3L * c->L[0].nnodes >= (1L << 31)) return false;  // 32-bit indices
  npr = std::max(1, std::min(npr, std::min(256 / p.nyt, (p.ngz + 1) / 2)));
  p.nzg = 2 * npr;
  p.pk = 1;
  *P = p;
  return true;
}

// Defaults before any tuning: FP32 (bandwidth-bound) aims at about three
// CTAs per SM, FP64 (FP64-pipe-bound) at two; x chunks make up the count.
void ec_default_plans(tp_ctx* c) {
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  for (int m = 0; m < 4; m++) {
    c->ec_f32[m] = EcPlan();
    c->ec_f64[m] = EcPlan();
  }
  if (!c->ec_ok) return;
  for (int prec = 0; prec < 2; prec++) {
    EcPlan p;
    const int nzg = prec == 0 ? 2 : 1;
    if (!ec_plan(c, nzg, 1, &p)) return;
    const int zctas = (p.ngz + p.nzg - 1) / p.nzg;
    const int want = (prec == 0 ? 3 : 2) * sms;
    ec_plan(c, nzg, (want + zctas - 1) / zctas, &p);
    p.estage = prec == 0 ? 0 : 1;
    for (int m = 0; m < 4; m++) (prec == 0 ? c->ec_f32 : c->ec_f64)[m] = p;
  }
  for (int m = 0; m < 4; m++) c->ec_ds[m] = c->ec_f64[m];
}

// FP32 plans of the sweep, residual and product: the packed kernel's
// defaults (on) or the one-group kernel's (off); tp_autotune re-tunes them
void ec_select_packed(tp_ctx* c, bool on) {
  if (!c->ec_ok) return;
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  for (int m = 0; m < 4; m++) {
    if (m == FM_APPLY_DOT) continue;
    EcPlan p;
    if (on) {
      if (!pk_plan(c, 1, 1, &p)) continue;
      const int zctas = (p.ngz + p.nzg - 1) / p.nzg;
      pk_plan(c, 1, (2 * sms + zctas - 1) / zctas, &p);
    } else {
      if (!ec_plan(c, 2, 1, &p)) continue;
      const int zctas = (p.ngz + p.nzg - 1) / p.nzg;
      ec_plan(c, 2, (3 * sms + zctas - 1) / zctas, &p);
      p.estage = 0;
    }
    c->ec_f32[m] = p;
  }
}

static EcGeom ec_geom(const tp_ctx* c, const EcPlan& p, size_t tsize, bool own, long vstride, bool pt = false) {
  const Level& L = c->L[0];
  EcGeom g;
  g.nx = L.nx;
  g.ny = L.ny;
  g.nz = L.nz;
  g.ex = L.ex;
  g.ey = L.ey;
  g.ez = L.ez;
  g.lim = L.lim;
  g.ngz = p.ngz;
  g.zbase = p.zbase;
  g.zextra = p.zextra;
  g.cx = p.cx;
  g.vstride = vstride;
  const long rows = (long)p.nzg * (p.zbase + (p.zextra > 0 ? 1 : 0));
  const long row_bytes = 3L * L.ny * (long)tsize;
  g.slab_bytes = (int)roundup16((rows + 2) * row_bytes + 32);
  g.own_bytes = own ? (int)roundup16(rows * row_bytes + 32) : 0;
  g.e_bytes = (p.estage || tsize != sizeof(float)) ? (int)roundup16((rows + 1) * (long)L.ey * (long)tsize + 32) : 0;
  // b and invD slots: RMAX rows x 2 arrays x 3 components per z group and
  // column (a packed-kernel thread holds two groups)
  g.pt_bytes = pt ? (int)(p.nyt * p.nzg * kEcRmax * 6 * sizeof(float)) : 0;
  return g;
}

static size_t ec_smem(const EcGeom& g, const EcPlan& p, size_t tsize) {
  const int nwy = p.nyt / 32;
  return 3 * (size_t)g.slab_bytes + 4 * (size_t)g.own_bytes + 2 * (size_t)g.e_bytes + (size_t)g.pt_bytes +
         tsize * (size_t)(2 * p.nzg * nwy * kEcRmax * 6 + p.nzg * (nwy + 1) * kEcRmax * 3);
}

template <typename T, typename A, int MODE>
static int ec_launch_as(tp_ctx* c, const EcPlan& p, const T* E, const T* in, T* out, const T* b, const T* invD,
                        T omega, int nrhs, long vstride) {
  const bool hasb = MODE == EC_JACOBI || MODE == EC_RESID;
  const EcGeom g = ec_geom(c, p, sizeof(T), hasb && p.own == 1, vstride, hasb && p.own == 2 && sizeof(T) == 4);
  const size_t smem = ec_smem(g, p, sizeof(T));
  // the register-capped form exists for FP32 vectors (three CTAs per SM)
  const bool capped = std::is_same<T, float>::value && p.occ3;
  constexpr int kMinB = std::is_same<T, float>::value ? 2 : 1;
  auto kern = fine_ec_kernel<T, A, MODE, kEcRmax, kMinB, true, false>;
  const bool pt = std::is_same<T, float>::value && hasb && p.own == 2;
  if constexpr (std::is_same<T, float>::value) {
    constexpr bool HB = MODE == EC_JACOBI || MODE == EC_RESID;
    if (pt) {
      if constexpr (HB) {
        if (capped)
          kern = p.estage ? fine_ec_kernel<T, A, MODE, kEcRmax, 3, true, true>
                          : fine_ec_kernel<T, A, MODE, kEcRmax, 3, false, true>;
        else
          kern = p.estage ? fine_ec_kernel<T, A, MODE, kEcRmax, kMinB, true, true>
                          : fine_ec_kernel<T, A, MODE, kEcRmax, kMinB, false, true>;
      }
    } else if (capped) {
      kern = p.estage ? fine_ec_kernel<T, A, MODE, kEcRmax, 3, true, false>
                      : fine_ec_kernel<T, A, MODE, kEcRmax, 3, false, false>;
    } else if (!p.estage) {
      kern = fine_ec_kernel<T, A, MODE, kEcRmax, kMinB, false, false>;
    }
  }
  const int form = (pt ? 4 : 0) + (capped ? 2 : 0) + (p.estage ? 1 : 0);
  static size_t set_for[8] = {};  // largest size the attribute was raised to, per form
  if (smem > 48 * 1024 && smem > set_for[form]) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
      cudaGetLastError();  // not sticky: the error is reported through c->err
      c->err = "fine_ec: shared memory request of " + std::to_string(smem) + " bytes refused";
      return 0;
    }
    set_for[form] = smem;
  }
  const dim3 grid((unsigned)((p.ngz + p.nzg - 1) / p.nzg), (unsigned)p.ncx, (unsigned)nrhs);
  kern<<<grid, dim3(p.nyt, p.nzg), smem, c->s>>>(g, E, in, out, b, invD, omega, c->d_red);
  TP_CHECK_LAUNCH(c, "fine_ec");
  return (int)(grid.x * grid.y);  // partials per right-hand side
}

// the packed FP32 kernel: p.nzg groups per CTA, two per thread row
template <int MODE>
static int pk_launch(tp_ctx* c, const EcPlan& p, const float* E, const float* in, float* out, const float* b,
                     const float* invD, float omega, int nrhs, long vstride) {
  const bool hasb = MODE == EC_JACOBI || MODE == EC_RESID;
  const EcGeom g = ec_geom(c, p, sizeof(float), hasb && p.own == 1, vstride, hasb && p.own == 2);
  const size_t smem = ec_smem(g, p, sizeof(float));
  // occ3 selects the form whose registers are capped for two 256-thread CTAs per SM
  auto kern = p.occ3 ? fine_pk_kernel<MODE, kEcRmax, 2> : fine_pk_kernel<MODE, kEcRmax, 1>;
  static size_t set_for[2] = {0, 0};
  const int form = p.occ3 ? 1 : 0;
  if (smem > 48 * 1024 && smem > set_for[form]) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
      cudaGetLastError();
      c->err = "fine_pk: shared memory request of " + std::to_string(smem) + " bytes refused";
      return 0;
    }
    set_for[form] = smem;
  }
  const dim3 grid((unsigned)((p.ngz + p.nzg - 1) / p.nzg), (unsigned)p.ncx, (unsigned)nrhs);
  kern<<<grid, dim3(p.nyt, p.nzg / 2), smem, c->s>>>(g, E, in, out, b, invD, omega);
  TP_CHECK_LAUNCH(c, "fine_pk");
  return (int)(grid.x * grid.y);
}

// double vectors are worked on in double-single when the context asks for it
template <typename T, int MODE>
static int ec_launch(tp_ctx* c, const EcPlan& p, const T* E, const T* in, T* out, const T* b, const T* invD,
                     T omega, int nrhs, long vstride) {
  if constexpr (std::is_same<T, double>::value)
    if (c->fine_ds) return ec_launch_as<T, Dsf, MODE>(c, p, E, in, out, b, invD, omega, nrhs, vstride);
  return ec_launch_as<T, T, MODE>(c, p, E, in, out, b, invD, omega, nrhs, vstride);
}

template <typename T>
const EcPlan& ec_plan_for(const tp_ctx* c, int mode) {
  return sizeof(T) == 8 ? (c->fine_ds ? c->ec_ds[mode] : c->ec_f64[mode]) : c->ec_f32[mode];
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// one launch of plan p for mode (the packed FP32 kernel where the plan says so)
template <typename T>
static int ec_run(tp_ctx* c, int mode, const EcPlan& p, const T* E, const T* in, T* out, const T* b,
                  const T* invD, T omega, int nr, long vs) {
  if constexpr (std::is_same<T, float>::value) {
    if (p.pk && mode != EC_APPLY_DOT) {
      switch (mode) {
        case EC_APPLY: return pk_launch<EC_APPLY>(c, p, E, in, out, b, invD, omega, nr, vs);
        case EC_JACOBI: return pk_launch<EC_JACOBI>(c, p, E, in, out, b, invD, omega, nr, vs);
        default: return pk_launch<EC_RESID>(c, p, E, in, out, b, invD, omega, nr, vs);
      }
    }
  }
  switch (mode) {
    case EC_APPLY: return ec_launch<T, EC_APPLY>(c, p, E, in, out, b, invD, omega, nr, vs);
    case EC_APPLY_DOT: return ec_launch<T, EC_APPLY_DOT>(c, p, E, in, out, b, invD, omega, nr, vs);
    case EC_JACOBI: return ec_launch<T, EC_JACOBI>(c, p, E, in, out, b, invD, omega, nr, vs);
    default: return ec_launch<T, EC_RESID>(c, p, E, in, out, b, invD, omega, nr, vs);
  }
}

// nr right-hand sides, consecutive columns of ndof(0). Only the first column
// needs a 16-byte aligned base: the staging of a later column may start up to
// 15 bytes early, inside the column before it.
template <typename T>
int fine_ec(tp_ctx* c, int mode, const T* E, const T* in, T* out, const T* b, const T* invD, T omega, int nr) {
  const EcPlan& p = ec_plan_for<T>(c, mode);
  const long vs = c->L[0].ndof;
  if (!p.ok || !aligned16(in) || (b && !aligned16(b)) || (invD && !aligned16(invD))) return -1;
  return ec_run<T>(c, mode, p, E, in, out, b, invD, omega, nr, vs);
}

template int fine_ec<double>(tp_ctx*, int, const double*, const double*, double*, const double*, const double*,
                             double, int);
template int fine_ec<float>(tp_ctx*, int, const float*, const float*, float*, const float*, const float*, float,
                            int);

}  // namespace tp

// ---------------------------------------------------------------------------
// The small autotuner: for each precision and fused mode, time the candidate
// launch shapes on the context's own grid and keep the fastest.
namespace {

template <typename T>
float ec_time(tp_ctx* c, int mode, const tp::EcPlan& p, const T* E, const T* in, T* out, const T* b,
              const T* d) {
  using namespace tp;
  int smax = 0;
  cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
  const bool hasb = mode == FM_JACOBI || mode == FM_RESID;
  if (ec_smem(ec_geom(c, p, sizeof(T), hasb && p.own == 1, 0, hasb && p.own == 2), p, sizeof(T)) > (size_t)smax)
    return 1e30f;  // does not fit
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto run = [&]() { return ec_run<T>(c, mode, p, E, in, out, b, d, T(0.6), 1, 0); };
  run();
  cudaEventRecord(e0, c->s);
  const int reps = 3;
  for (int r = 0; r < reps; r++) run();
  cudaEventRecord(e1, c->s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return c->err.empty() ? ms / reps : 1e30f;
}

template <typename T>
void ec_tune(tp_ctx* c, tp::EcPlan* plans, const T* E, const T* in, T* out, const T* b, const T* d, int sms,
             double* ms_out) {
  using namespace tp;
  constexpr bool f32 = std::is_same<T, float>::value;
  for (int mode = 0; mode < 4; mode++) {
    EcPlan best = plans[mode];
    float tbest = 1e30f;
    // family 0: one z group per thread row; family 1 (FP32 sweeps, residuals
    // and products): the packed kernel, two z groups per thread row
    const int nfam = (f32 && mode != FM_APPLY_DOT) ? 2 : 1;
    for (int fam = 0; fam < nfam; fam++)
      for (int nz1 = 1; nz1 <= 4; nz1 *= 2) {
        EcPlan p;
        auto plan = [&](int ncx) { return fam ? pk_plan(c, nz1, ncx, &p) : ec_plan(c, nz1, ncx, &p); };
        if (!plan(1) || p.nzg != (fam ? 2 * nz1 : nz1)) continue;
        const int zctas = (p.ngz + p.nzg - 1) / p.nzg;
        int last_ncx = -1;
        for (int mult = 1; mult <= 6; mult++) {
          if (!plan((mult * sms + zctas - 1) / zctas) || p.ncx == last_ncx) continue;
          last_ncx = p.ncx;
          const int nown = (mode == FM_JACOBI || mode == FM_RESID) ? (f32 ? 3 : 2) : 1;
          const int nocc = f32 ? 2 : 1;
          const int nes = (f32 && !fam) ? 2 : 1;  // FP32 one-group kernel: E staged or in registers
          for (int own = 0; own < nown; own++)
            for (int occ = 0; occ < nocc; occ++)
              for (int es = 0; es < nes; es++) {
                p.own = own;
                p.occ3 = occ;
                p.estage = nes == 2 ? es : 1;
                const float ms = ec_time<T>(c, mode, p, E, in, out, b, d);
                if (ms < tbest) {
                  tbest = ms;
                  best = p;
                }
              }
        }
      }
    plans[mode] = best;
    if (ms_out) ms_out[mode] = tbest;
  }
}

}  // namespace

extern "C" tp_status tp_autotune(tp_ctx* c, double* ms_out) {
  using namespace tp;
  if (!c) return TP_ERR_ARG;
  if (ms_out)
    for (int i = 0; i < 8; i++) ms_out[i] = 0.0;
  if (!c->ec_ok || !c->ec_f64[0].ok) return TP_OK;
  graph_free(c);  // a captured CG loop keeps the launch shapes it was recorded with
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  // the double-vector plans of the arithmetic in use (FP64 or double-single)
  ec_tune<double>(c, c->fine_ds ? c->ec_ds : c->ec_f64, c->d_E, c->d_p, c->d_q, c->d_r, c->invD[0], sms,
                  ms_out ? ms_out + 4 : nullptr);
  if (c->mgf_r[0] && c->invDf[0])
    ec_tune<float>(c, c->ec_f32, c->d_Ef, c->mgf_z[0], c->mgf_t[0], c->mgf_r[0], c->invDf[0], sms, ms_out);
  cudaError_t e = cudaStreamSynchronize(c->s);
  if (e != cudaSuccess) {
    c->err = std::string("autotune: ") + cudaGetErrorString(e);
    return TP_ERR_CUDA;
  }
  return c->err.empty() ? TP_OK : TP_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// Launch plans of the element-centric level-0 kernel, read and set by the
// caller (to keep a tuning between runs, or to choose one by hand).
namespace {
tp::EcPlan* plan_slot(tp_ctx* c, int vec, int mode) {
  if (vec == 0) return &c->ec_f32[mode];
  return c->fine_ds ? &c->ec_ds[mode] : &c->ec_f64[mode];
}
}  // namespace

extern "C" tp_status tp_get_fine_plan(tp_ctx* c, int vec, int mode, int* plan) {
  using namespace tp;
  if (!c || vec < 0 || vec > 1 || mode < 0 || mode > 3 || !plan) return TP_ERR_ARG;
  const EcPlan& p = *plan_slot(c, vec, mode);
  if (!p.ok) return TP_ERR_STATE;
  plan[0] = p.nzg;
  plan[1] = p.ncx;
  plan[2] = p.own;
  plan[3] = p.occ3;
  plan[4] = p.pk;
  plan[5] = p.estage;
  plan[6] = p.nyt;
  return TP_OK;
}

extern "C" tp_status tp_set_fine_plan(tp_ctx* c, int vec, int mode, const int* plan) {
  using namespace tp;
  if (!c || vec < 0 || vec > 1 || mode < 0 || mode > 3 || !plan || !c->ec_ok) return TP_ERR_ARG;
  const int groups = plan[0], ncx = plan[1], own = plan[2], occ = plan[3], pk = plan[4], es = plan[5];
  const bool hasb = mode == FM_JACOBI || mode == FM_RESID;
  if (groups < 1 || ncx < 1 || own < 0 || own > (vec == 0 ? 2 : 1) || (own && !hasb) || occ < 0 || occ > 1 ||
      pk < 0 || pk > 1 || (pk && (vec != 0 || mode == FM_APPLY_DOT || groups % 2)) || (occ && vec != 0) ||
      es < 0 || es > 1 || (!es && (vec != 0 || pk)))
    return TP_ERR_ARG;
  EcPlan p;
  const bool ok = pk ? pk_plan(c, groups / 2, ncx, &p) : ec_plan(c, groups, ncx, &p);
  if (!ok || p.nzg != groups || p.ncx != ncx) return TP_ERR_ARG;
  p.own = own;
  p.occ3 = occ;
  p.estage = es;
  const size_t tsize = vec == 0 ? sizeof(float) : sizeof(double);
  int smax = 0;
  cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
  if (ec_smem(ec_geom(c, p, tsize, hasb && own == 1, 0, hasb && own == 2), p, tsize) > (size_t)smax)
    return TP_ERR_ARG;
  *plan_slot(c, vec, mode) = p;
  graph_free(c);  // a captured CG loop keeps the launch shapes it was recorded with
  return TP_OK;
}
