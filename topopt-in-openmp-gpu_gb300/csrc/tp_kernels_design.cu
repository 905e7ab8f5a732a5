// Design-variable operations of the loop at stencil_optimization.c:148-189:
// compliance and sensitivity (stencil_methods.c:808-862), the density filter
// and its adjoint (stencil_optimization.c:228-395), the volume
// (gpu_definitions.c:94-108) and the OC bisection with the change measure
// (gpu_definitions.c:110-157). FP64 on FP64 data, all reductions two-pass
// and order-fixed; in the mixed form the element energies of the compliance
// pass are formed in double-single arithmetic (the level-0 operator's), the
// rest in FP64.
#include <cmath>
#include <vector>

#include "tp_dsf.cuh"
#include "tp_internal.h"

namespace tp {

__constant__ double c_ke0_design[576];
__constant__ double c_kz_design[45];
__constant__ float c_kzd_design[45][2];  // c_kz_design as double-single pairs
static bool g_kz_design = false;

void set_design_ke(const double* ke0) {
  cudaMemcpyToSymbol(c_ke0_design, ke0, sizeof(double) * 576);
  g_kz_design = false;
}
void set_design_kz(const double* kz45) {
  cudaMemcpyToSymbol(c_kz_design, kz45, sizeof(double) * 45);
  float d[45][2];
  for (int i = 0; i < 45; i++) {
    d[i][0] = (float)kz45[i];
    d[i][1] = (float)(kz45[i] - (double)d[i][0]);
  }
  cudaMemcpyToSymbol(c_kzd_design, d, sizeof(d));
  g_kz_design = true;
}

__host__ __device__ constexpr int dloc_dx(int q) { return (q == 1 || q == 2 || q == 5 || q == 6) ? 1 : 0; }
__host__ __device__ constexpr int dloc_dy(int q) { return (q == 0 || q == 1 || q == 4 || q == 5) ? 1 : 0; }
__host__ __device__ constexpr int dloc_dz(int q) { return q >= 4 ? 1 : 0; }

__device__ __forceinline__ double bsum256(double v) {
  __shared__ double sh[8];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < 8; w++) s += sh[w];
  __syncthreads();
  return s;
}
__device__ __forceinline__ double bmax256(double v) {
  __shared__ double sh[8];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < 8; w++) s = fmax(s, sh[w]);
  __syncthreads();
  return s;
}

struct DGeom {
  int ex, ey, ez, nx, ny, nz;
};
static DGeom dgeom(const tp_ctx* c) {
  const Level& L = c->L[0];
  return DGeom{L.ex, L.ey, L.ez, L.nx, L.ny, L.nz};
}

constexpr int kMaxBlocks = 4096;

// The per-axis sum/difference transform of an element's 8 nodal 3-vectors
// (v in the reference's local node order, z[(bx*4 + by*2 + bz)*3 + c]): three
// butterfly stages, x, y, z. The rigid-translation entries (b = 0) are not
// formed: KZ's row and column 0..2 vanish.
template <typename V>
__device__ __forceinline__ void t8_transform(const V* v, V* z) {
  // local node of corner (dx, dy, dz): dz*4 + (dy ? (dx ? 1 : 0) : (dx ? 2 : 3))
#pragma unroll
  for (int c = 0; c < 3; c++) {
    V a[2][2][2];  // [dy][dz][bx]
#pragma unroll
    for (int dy = 0; dy < 2; dy++)
#pragma unroll
      for (int dz = 0; dz < 2; dz++) {
        const V v0 = v[3 * (dz * 4 + (dy ? 0 : 3)) + c], v1 = v[3 * (dz * 4 + (dy ? 1 : 2)) + c];
        a[dy][dz][0] = v0 + v1;
        a[dy][dz][1] = v1 - v0;
      }
    V b[2][2][2];  // [bx][dz][by]
#pragma unroll
    for (int bx = 0; bx < 2; bx++)
#pragma unroll
      for (int dz = 0; dz < 2; dz++) {
        b[bx][dz][0] = a[0][dz][bx] + a[1][dz][bx];
        b[bx][dz][1] = a[1][dz][bx] - a[0][dz][bx];
      }
#pragma unroll
    for (int bx = 0; bx < 2; bx++)
#pragma unroll
      for (int by = 0; by < 2; by++) {
        if (bx || by) z[(bx * 4 + by * 2) * 3 + c] = b[bx][0][by] + b[bx][1][by];
        z[(bx * 4 + by * 2 + 1) * 3 + c] = b[bx][1][by] - b[bx][0][by];
      }
  }
}

// out_e = -3 (E0-Emin) x_e^2 w_e^T KE u_e (penalty 3, stencil_methods.c:855-858);
// with w = u, also the compliance partials sum_e E_e u_e^T KE u_e. With nr
// load cases (columns vs apart) the compliance and its sensitivity are the
// sums over the cases. SF: the energy as (T u)^T KZ (T w) -- the butterfly
// and the 45 non-zeros -- instead of the dense 24 x 24 product (a quarter
// of the FP64 instructions; equal to rounding).
template <bool COMPLIANCE, bool SF>
__global__ void sens_kernel(DGeom g, const double* __restrict__ x, const double* __restrict__ u,
                            const double* __restrict__ w, double* __restrict__ out,
                            double* __restrict__ partials, int nr, long vs) {
  const long ne = (long)g.ex * g.ey * g.ez;
  const double Ed = 1.0 - 1e-6;
  double csum = 0.0;
  for (long e = blockIdx.x * 256L + threadIdx.x; e < ne; e += (long)gridDim.x * 256) {
    const int j = e % g.ey;
    const int k = (e / g.ey) % g.ez;
    const int i = e / ((long)g.ey * g.ez);
    const double xe = x[e];
    double d = 0.0;
    for (int r = 0; r < nr; r++) {
      double ue[24], we[24];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const long n = ((long)(i + dloc_dx(q)) * g.nz + (k + dloc_dz(q))) * g.ny + (j + dloc_dy(q));
#pragma unroll
        for (int c = 0; c < 3; c++) {
          ue[3 * q + c] = u[r * vs + 3 * n + c];
          we[3 * q + c] = COMPLIANCE ? ue[3 * q + c] : w[3 * n + c];
        }
      }
      if (SF) {
        double zu[24], zw[24];
        t8_transform(ue, zu);
        if (COMPLIANCE) {
#pragma unroll
          for (int q = 3; q < 24; q++) zw[q] = zu[q];
        } else {
          t8_transform(we, zw);
        }
        double en = 0.0;
#define TP_KZ_TERM(i, rr, ss) en += c_kz_design[i] * zu[rr] * zw[ss];
        TP_KZ_PATTERN(TP_KZ_TERM)
#undef TP_KZ_TERM
        if (COMPLIANCE) csum += en * (1e-6 + xe * xe * xe * Ed);
        d += en * (-3.0 * Ed * xe * xe);
      } else {
#pragma unroll
        for (int ii = 0; ii < 8; ii++) {
          double cl = 0.0;
#pragma unroll
          for (int a = 0; a < 3; a++) {
            double t = 0.0;
#pragma unroll
            for (int b = 0; b < 24; b++) t += c_ke0_design[(ii * 3 + a) * 24 + b] * ue[b];
            cl += we[3 * ii + a] * t;
          }
          if (COMPLIANCE) csum += cl * (1e-6 + xe * xe * xe * Ed);
          d += cl * (-3.0 * Ed * xe * xe);
        }
      }
    }
    out[e] = d;
  }
  if (COMPLIANCE) {
    const double s = bsum256(csum);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
  }
}

// The compliance pass of the mixed form: the element energy (T u)^T KZ (T u)
// of sens_kernel<true, true> in double-single arithmetic (on this part an
// FP64 instruction holds its sub-partition's FP64 unit ~67 cycles, so the
// FP64 kernel is bound by that unit: about a tenth of its time), the
// penalty terms and the sums in FP64.
__global__ void sens_ds_kernel(DGeom g, const double* __restrict__ x, const double* __restrict__ u,
                               double* __restrict__ out, double* __restrict__ partials, int nr, long vs) {
  const long ne = (long)g.ex * g.ey * g.ez;
  const double Ed = 1.0 - 1e-6;
  double csum = 0.0;
  for (long e = blockIdx.x * 256L + threadIdx.x; e < ne; e += (long)gridDim.x * 256) {
    const int j = e % g.ey;
    const int k = (e / g.ey) % g.ez;
    const int i = e / ((long)g.ey * g.ez);
    const double xe = x[e];
    double d = 0.0;
    for (int r = 0; r < nr; r++) {
      Dsf ue[24], zu[24];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const long n = ((long)(i + dloc_dx(q)) * g.nz + (k + dloc_dz(q))) * g.ny + (j + dloc_dy(q));
#pragma unroll
        for (int c = 0; c < 3; c++) ue[3 * q + c] = ds_from(u[r * vs + 3 * n + c]);
      }
      t8_transform(ue, zu);
      Dsf en(0.f);
#define TP_KZ_TERM(i, rr, ss) en += Dsf(c_kzd_design[i][0], c_kzd_design[i][1]) * zu[rr] * zu[ss];
      TP_KZ_PATTERN(TP_KZ_TERM)
#undef TP_KZ_TERM
      const double ed = ds_to(en);
      csum += ed * (1e-6 + xe * xe * xe * Ed);
      d += ed * (-3.0 * Ed * xe * xe);
    }
    out[e] = d;
  }
  const double s = bsum256(csum);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

static int blocks_for(long n) {
  long b = (n + 255) / 256;
  if (b > kMaxBlocks) b = kMaxBlocks;
  if (b < 1) b = 1;
  return (int)b;
}

void compliance(tp_ctx* c, const double* u, double* dc, int* nblocks, int nr) {
  ProfScope ps(c, P_DESIGN);
  const DGeom g = dgeom(c);
  const long ne = (long)g.ex * g.ey * g.ez;
  const int nb = blocks_for(ne);
  if (c->ec_ok && g_kz_design && c->fine_ds)
    sens_ds_kernel<<<nb, 256, 0, c->s>>>(g, c->d_xphys, u, dc, c->d_red, nr, c->L[0].ndof);
  else if (c->ec_ok && g_kz_design)
    sens_kernel<true, true><<<nb, 256, 0, c->s>>>(g, c->d_xphys, u, nullptr, dc, c->d_red, nr, c->L[0].ndof);
  else
    sens_kernel<true, false><<<nb, 256, 0, c->s>>>(g, c->d_xphys, u, nullptr, dc, c->d_red, nr, c->L[0].ndof);
  TP_CHECK_LAUNCH(c, "compliance");
  *nblocks = nb;
}

void element_sens(tp_ctx* c, const double* u, const double* w, double* out) {
  ProfScope ps(c, P_DESIGN);
  const DGeom g = dgeom(c);
  const long ne = (long)g.ex * g.ey * g.ez;
  if (c->ec_ok && g_kz_design)
    sens_kernel<false, true><<<blocks_for(ne), 256, 0, c->s>>>(g, c->d_xphys, u, w, out, nullptr, 1, 0);
  else
    sens_kernel<false, false><<<blocks_for(ne), 256, 0, c->s>>>(g, c->d_xphys, u, w, out, nullptr, 1, 0);
  TP_CHECK_LAUNCH(c, "element_sens");
}

// ----------------------------------------------------------------------------
// Filter neighbourhood: [i-(ceil(rmin)-1), i+ceil(rmin)] clipped to the grid
// (stencil_optimization.c:254-269), weights max(0, rmin - |d|), loops in the
// reference's x, z, y order. The weight depends only on the offset, so the
// nonzero weights are tabulated once per radius on the host (IEEE sqrt, the
// same bits as the reference's expression) with their offsets, in that loop
// order; skipping the zero weights (and the test for them, an FP64 compare
// per offset) leaves every sum and its order unchanged.
struct FBox {
  int nw;               // nonzero weights
  const double* w;      // nw weights, then nw packed offsets (di, dk, dj) as doubles
};
constexpr int kFilterSmem = 512;  // weights staged in shared memory (rmin <= 4 always fits)

template <int MODE>  // 0: Hs, 1: forward H x / Hs, 2: adjoint H (v) with v already / Hs
__global__ void filter_kernel(DGeom g, FBox fb, const double* __restrict__ in, const double* __restrict__ hs,
                              double* __restrict__ out, double* __restrict__ partials) {
  __shared__ double sw[kFilterSmem];
  __shared__ int soff[kFilterSmem];  // (di + 64) << 16 | (dk + 64) << 8 | (dj + 64)
  const bool staged = fb.nw <= kFilterSmem;  // else read from global memory
  for (int q = threadIdx.x; staged && q < fb.nw; q += blockDim.x) {
    sw[q] = fb.w[q];
    soff[q] = (int)fb.w[fb.nw + q];
  }
  __syncthreads();
  const long ne = (long)g.ex * g.ey * g.ez;
  double vsum = 0.0;
  for (long e = blockIdx.x * 256L + threadIdx.x; e < ne; e += (long)gridDim.x * 256) {
    const int j = e % g.ey;
    const int k = (e / g.ey) % g.ez;
    const int i = e / ((long)g.ey * g.ez);
    double o = 0.0, h = 0.0;
    for (int q = 0; q < fb.nw; q++) {
      const int of = staged ? soff[q] : (int)__ldg(fb.w + fb.nw + q);
      const int i2 = i + (of >> 16) - 64, k2 = k + ((of >> 8) & 255) - 64, j2 = j + (of & 255) - 64;
      if (i2 < 0 || i2 >= g.ex || k2 < 0 || k2 >= g.ez || j2 < 0 || j2 >= g.ey) continue;
      const double wq = staged ? sw[q] : __ldg(fb.w + q);
      if (MODE == 0) h += wq;
      if (MODE != 0) o += wq * in[((long)i2 * g.ez + k2) * g.ey + j2];
    }
    if (MODE == 0) out[e] = h;
    if (MODE == 1) {
      const double v = o / hs[e];
      out[e] = v;
      vsum += v;
    }
    if (MODE == 2) out[e] = o;
  }
  if (MODE == 1) {
    const double s = bsum256(vsum);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
  }
}

__global__ void div_kernel(long n, const double* __restrict__ v, const double* __restrict__ hs, double* __restrict__ t) {
  const long e = blockIdx.x * 256L + threadIdx.x;
  if (e < n) t[e] = v[e] / hs[e];
}

static FBox fbox(const tp_ctx* c) { return FBox{c->fw_n, c->d_fw}; }

// (re)tabulates the weights of the context's radius and the row sums Hs
void filter_hs(tp_ctx* c, double* hs) {
  ProfScope ps(c, P_DESIGN);
  const int cr = (int)std::ceil(c->p.rmin);
  std::vector<double> wt, of;
  for (int di = -(cr - 1); di <= cr; di++)
    for (int dk = -(cr - 1); dk <= cr; dk++)
      for (int dj = -(cr - 1); dj <= cr; dj++) {
        const unsigned d2 = (unsigned)(di * di + dj * dj + dk * dk);
        const double v = c->p.rmin - std::sqrt((double)d2);
        if (v > 0.0) {
          wt.push_back(v);
          of.push_back((double)(((di + 64) << 16) | ((dk + 64) << 8) | (dj + 64)));
        }
      }
  c->fw_n = (int)wt.size();
  std::vector<double> w(wt);
  w.insert(w.end(), of.begin(), of.end());
  dev_free(c->d_fw);
  c->d_fw = nullptr;
  if (dev_malloc(&c->d_fw, sizeof(double) * w.size()) != cudaSuccess) {
    c->err = "cudaMalloc of the filter weights failed";
    return;
  }
  cudaMemcpyAsync(c->d_fw, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice, c->s);
  cudaStreamSynchronize(c->s);
  const DGeom g = dgeom(c);
  filter_kernel<0><<<blocks_for((long)g.ex * g.ey * g.ez), 256, 0, c->s>>>(g, fbox(c), nullptr, nullptr, hs, nullptr);
  TP_CHECK_LAUNCH(c, "filter_hs");
}

// forward filter; leaves sum(out) partials for the volume in d_red
int filter_fwd_blocks(const tp_ctx* c) {
  const DGeom g = dgeom(c);
  return blocks_for((long)g.ex * g.ey * g.ez);
}
void filter_fwd(tp_ctx* c, const double* x, double* out) {
  ProfScope ps(c, P_DESIGN);
  const DGeom g = dgeom(c);
  filter_kernel<1><<<filter_fwd_blocks(c), 256, 0, c->s>>>(g, fbox(c), x, c->d_hs, out, c->d_red);
  TP_CHECK_LAUNCH(c, "filter_fwd");
}

void filter_adj(tp_ctx* c, double* v, double* tmp) {
  ProfScope ps(c, P_DESIGN);
  const DGeom g = dgeom(c);
  const long ne = (long)g.ex * g.ey * g.ez;
  div_kernel<<<grid_for(ne, 256), 256, 0, c->s>>>(ne, v, c->d_hs, tmp);
  filter_kernel<2><<<blocks_for(ne), 256, 0, c->s>>>(g, fbox(c), tmp, nullptr, v, nullptr);
  TP_CHECK_LAUNCH(c, "filter_adj");
}

__global__ void sum_kernel(long n, const double* __restrict__ v, double* __restrict__ partials) {
  double s = 0.0;
  for (long e = blockIdx.x * 256L + threadIdx.x; e < n; e += (long)gridDim.x * 256) s += v[e];
  s = bsum256(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

void volume_partials(tp_ctx* c, const double* xphys, int* nblocks) {
  ProfScope ps(c, P_DESIGN);
  const long ne = (long)c->L[0].ex * c->L[0].ey * c->L[0].ez;
  const int nb = blocks_for(ne);
  sum_kernel<<<nb, 256, 0, c->s>>>(ne, xphys, c->d_red);
  TP_CHECK_LAUNCH(c, "volume");
  *nblocks = nb;
}

// ----------------------------------------------------------------------------
// The bisection takes at most kOcCap steps (then oc_bisect reports that it
// did not finish); a step after the cap, or after the interval is narrow
// enough, returns at once.
constexpr int kOcCap = 240;

// OC: xnew = max(0, max(x - move, min(1, min(x + move, x*sqrt(-dc/(dv*lmid))))))
// with the reference's MAX/MIN macros (a > b ? a : b), move = 0.2.
__device__ __forceinline__ double oc_xnew(double x, double dc, double dv, double lmid) {
  const double move = 0.2;
  const double xs = x * sqrt(-dc / (dv * lmid));
  const double a = (x + move > xs) ? xs : x + move;  // MIN(x + move, xs)
  const double b = (1.0 > a) ? a : 1.0;              // MIN(1.0, a)
  const double cc = (x - move > b) ? x - move : b;   // MAX(x - move, b)
  return (0.0 > cc) ? 0.0 : cc;                      // MAX(0.0, cc)
}

// The bisection steps only need the volume change sum_e dv_e (xnew_e - x_e)
// at each trial lmid. x sqrt(-dc/(dv lmid)) = B / sqrt(lmid) with
// B = x sqrt(-dc/dv) formed once per update, which takes the division and the
// square root of every element out of the ~50 steps (they agree with the
// reference's expression to a few ulp; the final pass below evaluates the
// reference's expression itself at the chosen lmid). The reference's nested
// MAX/MIN equal max(lo, min(hi, xs)) with lo = max(0, x - move) and
// hi = min(1, x + move) -- min and max do not round -- and lo, hi are formed
// once too. FP64 instructions are what a step costs on this part: lo, hi and
// xs are non-negative, so the clamp is an integer comparison of their bit
// patterns (the same values as fmin/fmax; a NaN xs, from a positive dc,
// counts as +inf, as fmin treats it), which leaves three per element
// (multiply, subtract, multiply-add). The sum keeps the reference's form
// dv (xnew - x) and its fold order: near the root gt is small, and another
// rounding of it can turn a bisection decision.
// max(lo, min(hi, v)) for 0 <= lo <= hi finite and any v: a NaN v gives hi
// (+inf here, as fmin ignores it), a negative v or -0 (B = -0 when the
// filtered dc is +0) gives lo (+0 here)
__device__ __forceinline__ double oc_clamp(double lo, double hi, double v) {
  long long iv = __double_as_longlong(v);
  if (iv < 0) iv = (iv & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL ? 0x7ff0000000000000LL : 0;
  else if (iv > 0x7ff0000000000000LL) iv = 0x7ff0000000000000LL;
  const long long il = __double_as_longlong(lo), ih = __double_as_longlong(hi);
  iv = iv < ih ? iv : ih;
  return __longlong_as_double(iv > il ? iv : il);
}
__global__ void oc_prep_kernel(long n, const double* __restrict__ x, const double* __restrict__ dc,
                               const double* __restrict__ dv, double* __restrict__ B, double* __restrict__ lo,
                               double* __restrict__ hi, double* __restrict__ scal) {
  const long e = blockIdx.x * 256L + threadIdx.x;
  if (e >= n) return;
  const double move = 0.2, xe = x[e], dve = dv[e];
  B[e] = xe * sqrt(-dc[e] / dve);
  lo[e] = fmax(0.0, xe - move);
  hi[e] = fmin(1.0, xe + move);
  if (!(dve > 0.0)) scal[S_DVBAD] = 1.0;  // the first phase's search needs every dv > 0
}

// one bisection step: partial sums of dv*(xnew - x) at lmid = (l1 + l2)/2;
// B = nullptr evaluates the reference's expression per element instead
__global__ void oc_step_kernel(long n, const double* __restrict__ x, const double* __restrict__ dc,
                               const double* __restrict__ dv, const double* __restrict__ B,
                               const double* __restrict__ lo, const double* __restrict__ hi,
                               double* __restrict__ scal, double* __restrict__ partials) {
  if (scal[S_OCDONE] != 0.0 || scal[S_TMP0] >= (double)kOcCap) return;
  const double lmid = 0.5 * (scal[S_L2] + scal[S_L1]);
  // 1/sqrt(lmid), formed once per step by the kernel that set l1 and l2 (FP64
  // division and square root are slow enough here to matter once per thread)
  const double rl = scal[S_RL];
  double s = 0.0;
  for (long e = blockIdx.x * 256L + threadIdx.x; e < n; e += (long)gridDim.x * 256) {
    const double xe = x[e];
    const double xn = B ? oc_clamp(lo[e], hi[e], B[e] * rl) : oc_xnew(xe, dc[e], dv[e], lmid);
    s += dv[e] * (xn - xe);
  }
  s = bsum256(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// gt = sum + g (g in scal[S_G]); l1 or l2 <- lmid; done when (l2-l1)/(l1+l2) <= 1e-6
__device__ __forceinline__ double oc_gt(const double* __restrict__ partials, int nb, const double* scal) {
  __shared__ double sh[256];
  const int per = (nb + 255) / 256;
  const int b0 = threadIdx.x * per;
  double s = 0.0;
  for (int i = b0; i < b0 + per && i < nb; i++) s += partials[i];
  return fold256(s, false, sh) + scal[S_G];
}

__global__ void oc_finish_kernel(const double* __restrict__ partials, int nb, double* __restrict__ scal) {
  if (scal[S_OCDONE] != 0.0 || scal[S_TMP0] >= (double)kOcCap) return;
  const double gt = oc_gt(partials, nb, scal);
  if (threadIdx.x == 0) {
    const double l1 = scal[S_L1], l2 = scal[S_L2];
    const double lmid = 0.5 * (l2 + l1);
    double nl1 = l1, nl2 = l2;
    if (gt > 0)
      nl1 = lmid;
    else
      nl2 = lmid;
    scal[S_L1] = nl1;
    scal[S_L2] = nl2;
    scal[S_LMID] = lmid;
    scal[S_GT] = gt;
    scal[S_OCDONE] = ((nl2 - nl1) / (nl1 + nl2) > 1e-6) ? 0.0 : 1.0;
    scal[S_RL] = 1.0 / sqrt(0.5 * (nl2 + nl1));
    scal[S_TMP0] += 1.0;  // steps taken
  }
}

// The bisection's first phase, searched. From l1 = 0, l2 = 1e9 the bisection
// halves l2 (step n tries lmid = 1e9 2^-n exactly: l2 + 0 and the halving do
// not round) while gt(lmid) <= 0, and sets l1 at the first step n* with
// gt > 0. With every dv > 0, gt as evaluated is a non-increasing function of
// lmid: each xnew is a non-decreasing function of 1/sqrt(lmid) (rounding is
// monotone, and a NaN term is NaN at every lmid), and the sum adds monotone
// terms in a fixed order. So n* is found by a binary search over n in
// ceil(log2(cap + 1)) probes of the same step kernel, each run with the l1,
// l2 and 1/sqrt(lmid) that sequential step n would have, and the state after
// step n* is set as the sequential steps leave it: the same decisions, the
// same bits, in 8 passes over the elements instead of n* (~40 at
// 256x128x128). A probe after the search has ended returns at once.
constexpr int kOcProbes = 8;  // 2^8 > kOcCap + 1
static_assert((1 << kOcProbes) > kOcCap + 1, "probes cover the first phase");

__device__ __forceinline__ double oc_l2_before(int n) { return ldexp(1e9, -(n - 1)); }  // l2 before step n

__global__ void oc_search_init_kernel(double* scal) {
  // a dv that is not positive leaves the first phase to the sequential steps
  scal[S_BLO] = 1.0;
  scal[S_BHI] = scal[S_DVBAD] != 0.0 ? 1.0 : (double)(kOcCap + 1);
}

__global__ void oc_probe_set_kernel(double* scal) {
  const int lo = (int)scal[S_BLO], hi = (int)scal[S_BHI];
  if (lo >= hi) {
    scal[S_OCDONE] = 1.0;  // the probe's step and finish return at once
    return;
  }
  const int mid = (lo + hi) / 2;
  const double l2 = oc_l2_before(mid);
  scal[S_L1] = 0.0;
  scal[S_L2] = l2;
  scal[S_RL] = 1.0 / sqrt(0.5 * (l2 + 0.0));
  scal[S_OCDONE] = 0.0;
  scal[S_TMP0] = 0.0;
  scal[S_TMP1] = (double)mid;
}

__global__ void oc_probe_finish_kernel(const double* __restrict__ partials, int nb, double* __restrict__ scal) {
  if (scal[S_OCDONE] != 0.0) return;
  const double gt = oc_gt(partials, nb, scal);
  if (threadIdx.x == 0) {
    const int mid = (int)scal[S_TMP1];
    if (gt > 0)
      scal[S_BHI] = (double)mid;
    else
      scal[S_BLO] = (double)(mid + 1);
  }
}

// the state the sequential steps 1 .. n* leave (or, with no n* within the
// cap, steps 1 .. cap); with the search skipped, the state before step 1
__global__ void oc_search_done_kernel(double* scal) {
  if (scal[S_DVBAD] != 0.0) {
    scal[S_L1] = 0.0;
    scal[S_L2] = 1e9;
    scal[S_OCDONE] = ((1e9 - 0.0) / (0.0 + 1e9) > 1e-6) ? 0.0 : 1.0;
    scal[S_TMP0] = 0.0;
    scal[S_LMID] = 0.0;
    scal[S_RL] = 1.0 / sqrt(0.5 * (1e9 + 0.0));
    return;
  }
  const int n = (int)scal[S_BLO];  // == hi
  double nl1, nl2;
  if (n > kOcCap) {  // cap halvings, no root bracketed
    nl1 = 0.0;
    nl2 = oc_l2_before(kOcCap + 1);
    scal[S_TMP0] = (double)kOcCap;
  } else {
    nl1 = oc_l2_before(n + 1);  // lmid of step n
    nl2 = oc_l2_before(n);
    scal[S_TMP0] = (double)n;
  }
  scal[S_LMID] = n > kOcCap ? nl2 : nl1;
  scal[S_L1] = nl1;
  scal[S_L2] = nl2;
  scal[S_OCDONE] = ((nl2 - nl1) / (nl1 + nl2) > 1e-6) ? 0.0 : 1.0;
  scal[S_RL] = 1.0 / sqrt(0.5 * (nl2 + nl1));
}

// the search, enqueued: 3 + 2 kOcProbes small launches and kOcProbes passes
static void oc_search_enqueue(tp_ctx* c, long ne, int nb, const double* x, const double* dc, const double* dv,
                              const double* B, const double* lo, const double* hi) {
  oc_search_init_kernel<<<1, 1, 0, c->s>>>(c->d_scal);
  for (int q = 0; q < kOcProbes; q++) {
    oc_probe_set_kernel<<<1, 1, 0, c->s>>>(c->d_scal);
    oc_step_kernel<<<nb, 256, 0, c->s>>>(ne, x, dc, dv, B, lo, hi, c->d_scal, c->d_red);
    oc_probe_finish_kernel<<<1, 256, 0, c->s>>>(c->d_red, nb, c->d_scal);
  }
  oc_search_done_kernel<<<1, 1, 0, c->s>>>(c->d_scal);
}

// final pass at the last lmid: xnew, max |x - xnew| partials, x <- xnew
__global__ void oc_apply_kernel(long n, double* __restrict__ x, double* __restrict__ xnew,
                                const double* __restrict__ dc, const double* __restrict__ dv,
                                const double* __restrict__ scal, double* __restrict__ partials, int commit) {
  const double lmid = scal[S_LMID];
  double m = 0.0;
  for (long e = blockIdx.x * 256L + threadIdx.x; e < n; e += (long)gridDim.x * 256) {
    const double xo = x[e];
    const double xn = oc_xnew(xo, dc[e], dv[e], lmid);
    xnew[e] = xn;
    m = fmax(m, fabs(xo - xn));
    if (commit) x[e] = xn;
  }
  m = bmax256(m);
  if (threadIdx.x == 0) partials[blockIdx.x] = m;
}

__global__ void oc_set_g_kernel(double* scal, double g) { scal[S_G] = g; }

// the constraint value of the loop (stencil_optimization.c:158-160): the
// volume sum divided by the element count, minus volfrac
__global__ void oc_g_from_volume_kernel(double* scal, double nelem, double volfrac) {
  scal[S_G] = scal[S_VOL] / nelem - volfrac;
}

// loop condition of the bisection graph: another batch of steps while the
// interval is not yet narrow enough and the step cap is not reached
__global__ void oc_cond_kernel(const double* scal, cudaGraphConditionalHandle h, int cap) {
  const bool go = scal[S_OCDONE] == 0.0 && scal[S_TMP0] < (double)cap;
  cudaGraphSetConditional(h, go ? 1u : 0u);
}

__global__ void oc_init_kernel(double* scal) {
  scal[S_DVBAD] = 0.0;
  scal[S_L1] = 0.0;
  scal[S_L2] = 1e9;
  scal[S_OCDONE] = ((1e9 - 0.0) / (0.0 + 1e9) > 1e-6) ? 0.0 : 1.0;
  scal[S_TMP0] = 0.0;
  scal[S_LMID] = 0.0;
  scal[S_RL] = 1.0 / sqrt(0.5 * (1e9 + 0.0));
}

// Bisection over any n design variables; leaves xnew, S_CHANGE and, when
// commit is set, x <- xnew. Returns 0, or -1 if the bisection did not finish
// within its step cap.
int oc_bisect(tp_ctx* c, long ne, double* x, double* xnew, const double* dc, const double* dv, double g,
              bool commit) {
  ProfScope ps(c, P_DESIGN);
  const int nb = blocks_for(ne);
  oc_init_kernel<<<1, 1, 0, c->s>>>(c->d_scal);
  oc_set_g_kernel<<<1, 1, 0, c->s>>>(c->d_scal, g);
  const double *B = nullptr, *lo = nullptr, *hi = nullptr;
  if (ne > c->ocb_n) {
    // a longer array than the context's design (the reference-signature
    // update_solution passes the padded element count): the scratch grows
    // once; without it every step evaluates the reference's expression per
    // element (an FP64 division and square root each)
    double* nb = nullptr;
    if (dev_malloc(&nb, sizeof(double) * 3 * (size_t)ne) == cudaSuccess) {
      cudaStreamSynchronize(c->s);
      dev_free(c->d_ocb);
      c->mem_bytes += 24L * (ne - c->ocb_n);
      c->d_ocb = nb;
      c->ocb_n = ne;
      oc_graph_free(c);  // the captured bisection holds the old scratch
    }
  }
  if (c->d_ocb && ne <= c->ocb_n) {
    double* b = c->d_ocb;
    oc_prep_kernel<<<grid_for(ne, 256), 256, 0, c->s>>>(ne, x, dc, dv, b, b + ne, b + 2 * ne, c->d_scal);
    B = b;
    lo = b + ne;
    hi = b + 2 * ne;
    oc_search_enqueue(c, ne, nb, x, dc, dv, B, lo, hi);
  }
  const int kBatch = 24;
  for (;;) {
    for (int q = 0; q < kBatch; q++) {
      oc_step_kernel<<<nb, 256, 0, c->s>>>(ne, x, dc, dv, B, lo, hi, c->d_scal, c->d_red);
      oc_finish_kernel<<<1, 256, 0, c->s>>>(c->d_red, nb, c->d_scal);
    }
    // S_OCDONE and S_TMP0 (steps taken) are adjacent
    cudaMemcpyAsync(c->h_scal + S_OCDONE, c->d_scal + S_OCDONE, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->s);
    cudaStreamSynchronize(c->s);
    if (c->h_scal[S_OCDONE] != 0.0) break;
    if (c->h_scal[S_TMP0] >= (double)kOcCap) return -1;
  }
  oc_apply_kernel<<<nb, 256, 0, c->s>>>(ne, x, xnew, dc, dv, c->d_scal, c->d_red, commit ? 1 : 0);
  finish_sum(c, nb, S_CHANGE, 1);
  TP_CHECK_LAUNCH(c, "oc_update");
  return 0;
}

int oc_update(tp_ctx* c, double g) {
  const long ne = (long)c->L[0].ex * c->L[0].ey * c->L[0].ez;
  return oc_bisect(c, ne, c->d_x, c->d_xnew, c->d_dc, c->d_dv, g, true);
}

void constraint_from_volume(tp_ctx* c) {
  const double ne = (double)((long)c->L[0].ex * c->L[0].ey * c->L[0].ez);
  oc_g_from_volume_kernel<<<1, 1, 0, c->s>>>(c->d_scal, ne, c->p.volfrac);
}

// The bisection of the context's own design arrays as a CUDA graph: one
// conditional WHILE node whose body is kOcBody bisection steps (each a
// partial-sum kernel and the kernel that halves the interval; steps after
// the interval is narrow enough return at once) and the condition kernel.
// It takes the same steps as oc_bisect, with no host check between them; the
// cap is the same 240 steps.
constexpr int kOcBody = 8;

void oc_graph_free(tp_ctx* c) {
  if (c->oc_exec) cudaGraphExecDestroy(c->oc_exec);
  c->oc_exec = nullptr;
}

static bool oc_graph_build(tp_ctx* c) {
  oc_graph_free(c);
  const long ne = (long)c->L[0].ex * c->L[0].ey * c->L[0].ez;
  const int nb = blocks_for(ne);
  double* b = c->d_ocb;
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
  cudaGraphConditionalHandle h;
  bool ok = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  ok = ok && cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) == cudaSuccess;
  if (ok) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    ok = cudaStreamBeginCaptureToGraph(c->s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    if (ok) {
      for (int q = 0; q < kOcBody; q++) {
        oc_step_kernel<<<nb, 256, 0, c->s>>>(ne, c->d_x, c->d_dc, c->d_dv, b, b + ne, b + 2 * ne, c->d_scal,
                                             c->d_red);
        oc_finish_kernel<<<1, 256, 0, c->s>>>(c->d_red, nb, c->d_scal);
      }
      oc_cond_kernel<<<1, 1, 0, c->s>>>(c->d_scal, h, kOcCap);
      cudaGraph_t out = nullptr;
      ok = cudaStreamEndCapture(c->s, &out) == cudaSuccess;
    }
  }
  if (ok) ok = cudaGraphInstantiate(&c->oc_exec, g, 0) == cudaSuccess;
  cudaGraphDestroy(g);
  if (!ok) {
    c->oc_exec = nullptr;
    cudaGetLastError();
  }
  return ok;
}

bool oc_update_graph(tp_ctx* c) {
  const long ne = (long)c->L[0].ex * c->L[0].ey * c->L[0].ez;
  if (!c->d_ocb || ne > c->ocb_n) return false;
  if (!c->oc_exec && !oc_graph_build(c)) return false;
  ProfScope ps(c, P_DESIGN);
  const int nb = blocks_for(ne);
  double* b = c->d_ocb;
  oc_init_kernel<<<1, 1, 0, c->s>>>(c->d_scal);
  oc_prep_kernel<<<grid_for(ne, 256), 256, 0, c->s>>>(ne, c->d_x, c->d_dc, c->d_dv, b, b + ne, b + 2 * ne,
                                                      c->d_scal);
  oc_search_enqueue(c, ne, nb, c->d_x, c->d_dc, c->d_dv, b, b + ne, b + 2 * ne);
  cudaGraphLaunch(c->oc_exec, c->s);
  oc_apply_kernel<<<nb, 256, 0, c->s>>>(ne, c->d_x, c->d_xnew, c->d_dc, c->d_dv, c->d_scal, c->d_red, 1);
  finish_sum(c, nb, S_CHANGE, 1);
  TP_CHECK_LAUNCH(c, "oc_update_graph");
  return true;
}

// max |x - xnew| into S_CHANGE, then x <- xnew (gpu_definitions.c:110-125)
__global__ void change_kernel(long n, double* __restrict__ x, const double* __restrict__ xnew,
                              double* __restrict__ partials) {
  double m = 0.0;
  for (long e = blockIdx.x * 256L + threadIdx.x; e < n; e += (long)gridDim.x * 256) {
    m = fmax(m, fabs(x[e] - xnew[e]));
    x[e] = xnew[e];
  }
  m = bmax256(m);
  if (threadIdx.x == 0) partials[blockIdx.x] = m;
}

void vec_change(tp_ctx* c, long n, double* x, const double* xnew) {
  ProfScope ps(c, P_DESIGN);
  const int nb = blocks_for(n);
  change_kernel<<<nb, 256, 0, c->s>>>(n, x, xnew, c->d_red);
  finish_sum(c, nb, S_CHANGE, 1);
  TP_CHECK_LAUNCH(c, "vec_change");
}

void vec_sum(tp_ctx* c, long n, const double* v, int slot) {
  ProfScope ps(c, P_DESIGN);
  const int nb = blocks_for(n);
  sum_kernel<<<nb, 256, 0, c->s>>>(n, v, c->d_red);
  finish_sum(c, nb, slot, 0);
  TP_CHECK_LAUNCH(c, "vec_sum");
}

}  // namespace tp
