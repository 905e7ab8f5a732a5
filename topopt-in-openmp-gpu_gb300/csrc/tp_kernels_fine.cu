// Level-0 operator: the matrix-free hex8 stencil y = K(rho) u
// (stencil_methods.c:7-428), with its fused consumers (Jacobi sweep,
// residual, CG matvec + dot) and the fine Jacobi diagonal (:693-773).
//
// One CTA owns a TX x TZ x TY block of nodes. It stages the input nodes of
// the block plus a one-node halo and the E(rho) of the touching elements in
// shared memory (coalesced along y), then each thread gathers the 27
// neighbour nodes of its node and applies the 64 "spokes" (node, element,
// node) of the element stiffness KE, scaled by E of the element:
//   y_n = sum_{e ni n} E_e * KE[rows of n in e, :] * u_e.
// KE lives in constant memory and every index is a compile-time constant
// after unrolling, so the 576 multiply-adds take KE as an immediate
// constant-bank operand. Elements outside the grid have E = 0 (the
// reference's halo), fixed DOFs return the input (:420-427).
#include "tp_internal.h"

namespace tp {

__constant__ double c_ke0[576];
__constant__ float c_ke0f[576];

void set_fine_ke(const double* ke0) {
  float f[576];
  set_fine_kz(ke0, nullptr);
  for (int i = 0; i < 576; i++) f[i] = (float)ke0[i];
  cudaMemcpyToSymbol(c_ke0, ke0, sizeof(double) * 576);
  cudaMemcpyToSymbol(c_ke0f, f, sizeof(float) * 576);
}

template <typename T>
__device__ __forceinline__ T ke0(int idx);
template <>
__device__ __forceinline__ double ke0<double>(int idx) { return c_ke0[idx]; }
template <>
__device__ __forceinline__ float ke0<float>(int idx) { return c_ke0f[idx]; }

// local node number of the node at offset (dx,dy,dz) from an element's
// (i, j, k) corner, in the order of getEdof_halo (stencil_utility.h:19-52)
__host__ __device__ constexpr int loc(int dx, int dy, int dz) {
  return dz * 4 + (dy ? (dx ? 1 : 0) : (dx ? 2 : 3));
}

struct FineGeom {
  int nx, ny, nz, ex, ey, ez, lim;
};

constexpr int TY = 32, TZ = 4, TX = 2, NT = TX * TY * TZ;
constexpr int SY = TY + 2, SZ = TZ + 2, SX = TX + 2;
constexpr int EY = TY + 1, EZ = TZ + 1, EX = TX + 1;

enum { M_APPLY = 0, M_APPLY_DOT = 1, M_JACOBI = 2, M_RESID = 3 };

template <typename T>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int warp = tid >> 5;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (tid == 0)
    for (int w = 0; w < NT / 32; w++) s += sh[w];
  return s;
}

template <typename T, int MODE>
__global__ void __launch_bounds__(NT)
    fine_kernel(FineGeom g, const T* __restrict__ E, const T* __restrict__ in,
                T* __restrict__ out, const T* __restrict__ b, const T* __restrict__ invD,
                T omega, double* __restrict__ partials) {
  __shared__ T su[SX][SZ][SY * 3];
  __shared__ T sE[EX][EZ][EY];
  const int tj = threadIdx.x, tk = threadIdx.y, ti = threadIdx.z;
  const int j0 = blockIdx.x * TY, k0 = blockIdx.y * TZ, i0 = blockIdx.z * TX;
  const int tid = tj + TY * (tk + TZ * ti);

  for (int idx = tid; idx < SX * SZ * SY * 3; idx += NT) {
    const int c = idx % (SY * 3);
    const int rest = idx / (SY * 3);
    const int sk = rest % SZ, si = rest / SZ;
    const int gi = i0 - 1 + si, gk = k0 - 1 + sk, gj = j0 - 1 + c / 3;
    T v = T(0);
    if (gi >= 0 && gi < g.nx && gk >= 0 && gk < g.nz && gj >= 0 && gj < g.ny)
      v = in[3 * (((long)gi * g.nz + gk) * g.ny + gj) + c % 3];
    su[si][sk][c] = v;
  }
  for (int idx = tid; idx < EX * EZ * EY; idx += NT) {
    const int sj = idx % EY;
    const int rest = idx / EY;
    const int sk = rest % EZ, si = rest / EZ;
    const int gi = i0 - 1 + si, gk = k0 - 1 + sk, gj = j0 - 1 + sj;
    T v = T(0);
    if (gi >= 0 && gi < g.ex && gk >= 0 && gk < g.ez && gj >= 0 && gj < g.ey)
      v = E[((long)gi * g.ez + gk) * g.ey + gj];
    sE[si][sk][sj] = v;
  }
  __syncthreads();

  const int i = i0 + ti, k = k0 + tk, j = j0 + tj;
  const bool active = (i < g.nx) && (k < g.nz) && (j < g.ny);

  T acc[8][3];
#pragma unroll
  for (int e = 0; e < 8; e++) acc[e][0] = acc[e][1] = acc[e][2] = T(0);

#pragma unroll
  for (int m = 0; m < 27; m++) {
    const int mx = m / 9 - 1, mz = (m / 3) % 3 - 1, my = m % 3 - 1;
    const T u0 = su[ti + 1 + mx][tk + 1 + mz][3 * (tj + 1 + my) + 0];
    const T u1 = su[ti + 1 + mx][tk + 1 + mz][3 * (tj + 1 + my) + 1];
    const T u2 = su[ti + 1 + mx][tk + 1 + mz][3 * (tj + 1 + my) + 2];
#pragma unroll
    for (int e = 0; e < 8; e++) {
      const int ex = -(e & 1), ez = -((e >> 1) & 1), ey = -((e >> 2) & 1);
      const int rx = mx - ex, ry = my - ey, rz = mz - ez;
      if (rx < 0 || rx > 1 || ry < 0 || ry > 1 || rz < 0 || rz > 1) continue;
      const int qn = loc(-ex, -ey, -ez), qm = loc(rx, ry, rz);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const int row = (3 * qn + c) * 24 + 3 * qm;
        acc[e][c] += ke0<T>(row + 0) * u0 + ke0<T>(row + 1) * u1 + ke0<T>(row + 2) * u2;
      }
    }
  }
  T y[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int e = 0; e < 8; e++) {
    const int ex = -(e & 1), ez = -((e >> 1) & 1), ey = -((e >> 2) & 1);
    const T Ee = sE[ti + 1 + ex][tk + 1 + ez][tj + 1 + ey];
    y[0] += Ee * acc[e][0];
    y[1] += Ee * acc[e][1];
    y[2] += Ee * acc[e][2];
  }
  const T* uc = &su[ti + 1][tk + 1][3 * (tj + 1)];
  const bool fixed = (i == 0) && (j < g.lim || j >= g.ny - g.lim);
  if (fixed) {
    y[0] = uc[0];
    y[1] = uc[1];
    y[2] = uc[2];
  }
  const long n = ((long)i * g.nz + k) * g.ny + j;
  double dotv = 0.0;
  if (active) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      if (MODE == M_APPLY || MODE == M_APPLY_DOT) out[3 * n + c] = y[c];
      if (MODE == M_JACOBI) out[3 * n + c] = uc[c] + omega * invD[3 * n + c] * (b[3 * n + c] - y[c]);
      if (MODE == M_RESID) out[3 * n + c] = b[3 * n + c] - y[c];
      if (MODE == M_APPLY_DOT) dotv += (double)uc[c] * (double)y[c];
    }
  }
  if (MODE == M_APPLY_DOT) {
    __shared__ double sh[NT / 32];
    const double s = block_sum<T>(dotv, sh);
    if (tid == 0) partials[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
  }
}

static FineGeom geom(const tp_ctx* c) {
  const Level& L = c->L[0];
  return FineGeom{L.nx, L.ny, L.nz, L.ex, L.ey, L.ez, L.lim};
}
static dim3 fine_grid(const tp_ctx* c) {
  const Level& L = c->L[0];
  return dim3((L.ny + TY - 1) / TY, (L.nz + TZ - 1) / TZ, (L.nx + TX - 1) / TX);
}

// The element-centric kernel (tp_kernels_fine_ec.cu) takes every call it
// has a plan for; this node-centric kernel covers the rest (y extents above
// 256 elements, unaligned vectors) and serves as its cross-check.
template <typename T>
void fine_apply(tp_ctx* c, const T* E, const T* in, T* out, int nr) {
  ProfScope ps(c, sizeof(T) == 8 ? P_FINE_APPLY_F64 : P_FINE_APPLY_F32);
  if (c->fine_variant == 0 && fine_ec<T>(c, FM_APPLY, E, in, out, nullptr, nullptr, T(0), nr) >= 0) return;
  const long vs = c->L[0].ndof;
  for (int r = 0; r < nr; r++)
    fine_kernel<T, M_APPLY><<<fine_grid(c), dim3(TY, TZ, TX), 0, c->s>>>(geom(c), E, in + r * vs, out + r * vs,
                                                                         nullptr, nullptr, T(0), nullptr);
  TP_CHECK_LAUNCH(c, "fine_apply");
}
template <typename T>
int fine_apply_dot(tp_ctx* c, const T* E, const T* in, T* out, int nr) {
  ProfScope ps(c, sizeof(T) == 8 ? P_FINE_APPLY_F64 : P_FINE_APPLY_F32);
  if (c->fine_variant == 0) {
    const int nb = fine_ec<T>(c, FM_APPLY_DOT, E, in, out, nullptr, nullptr, T(0), nr);
    if (nb >= 0) return nb;
  }
  const long vs = c->L[0].ndof;
  for (int r = 0; r < nr; r++)
    fine_kernel<T, M_APPLY_DOT><<<fine_grid(c), dim3(TY, TZ, TX), 0, c->s>>>(
        geom(c), E, in + r * vs, out + r * vs, nullptr, nullptr, T(0), c->d_red + (long)r * fine_blocks(c));
  TP_CHECK_LAUNCH(c, "fine_apply_dot");
  return fine_blocks(c);
}
template <typename T>
void fine_jacobi(tp_ctx* c, const T* E, const T* invD, const T* b, const T* u, T* unew, T omega, int nr) {
  ProfScope ps(c, sizeof(T) == 8 ? P_FINE_JACOBI_F64 : P_FINE_JACOBI_F32);
  if (c->fine_variant == 0 && fine_ec<T>(c, FM_JACOBI, E, u, unew, b, invD, omega, nr) >= 0) return;
  const long vs = c->L[0].ndof;
  for (int r = 0; r < nr; r++)
    fine_kernel<T, M_JACOBI><<<fine_grid(c), dim3(TY, TZ, TX), 0, c->s>>>(geom(c), E, u + r * vs, unew + r * vs,
                                                                          b + r * vs, invD, omega, nullptr);
  TP_CHECK_LAUNCH(c, "fine_jacobi");
}
template <typename T>
void fine_resid(tp_ctx* c, const T* E, const T* b, const T* u, T* d, int nr) {
  ProfScope ps(c, sizeof(T) == 8 ? P_FINE_RESID_F64 : P_FINE_RESID_F32);
  if (c->fine_variant == 0 && fine_ec<T>(c, FM_RESID, E, u, d, b, nullptr, T(0), nr) >= 0) return;
  const long vs = c->L[0].ndof;
  for (int r = 0; r < nr; r++)
    fine_kernel<T, M_RESID><<<fine_grid(c), dim3(TY, TZ, TX), 0, c->s>>>(geom(c), E, u + r * vs, d + r * vs,
                                                                         b + r * vs, nullptr, T(0), nullptr);
  TP_CHECK_LAUNCH(c, "fine_resid");
}

int fine_blocks(const tp_ctx* c) {
  const dim3 g = fine_grid(c);
  return (int)(g.x * g.y * g.z);
}

template void fine_apply<double>(tp_ctx*, const double*, const double*, double*, int);
template void fine_apply<float>(tp_ctx*, const float*, const float*, float*, int);
template int fine_apply_dot<double>(tp_ctx*, const double*, const double*, double*, int);
template void fine_jacobi<double>(tp_ctx*, const double*, const double*, const double*, const double*, double*, double,
                                  int);
template void fine_jacobi<float>(tp_ctx*, const float*, const float*, const float*, const float*, float*, float, int);
template void fine_resid<double>(tp_ctx*, const double*, const double*, const double*, double*, int);
template void fine_resid<float>(tp_ctx*, const float*, const float*, const float*, float*, int);

// inverse Jacobi diagonal of level 0: 1 / sum_e E_e KE[r][r], 1 at fixed DOFs
__global__ void fine_diag_kernel(FineGeom g, const double* __restrict__ E, double* __restrict__ invD) {
  const long n = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (n >= (long)g.nx * g.ny * g.nz) return;
  const int j = n % g.ny;
  const int k = (n / g.ny) % g.nz;
  const int i = n / ((long)g.ny * g.nz);
  double d[3] = {0, 0, 0};
#pragma unroll
  for (int e = 0; e < 8; e++) {
    const int ex = -(e & 1), ez = -((e >> 1) & 1), ey = -((e >> 2) & 1);
    const int ei = i + ex, ek = k + ez, ej = j + ey;
    if (ei < 0 || ei >= g.ex || ek < 0 || ek >= g.ez || ej < 0 || ej >= g.ey) continue;
    const double Ee = E[((long)ei * g.ez + ek) * g.ey + ej];
    const int qn = loc(-ex, -ey, -ez);
#pragma unroll
    for (int c = 0; c < 3; c++) d[c] += Ee * c_ke0[(3 * qn + c) * 25];
  }
  const bool fixed = (i == 0) && (j < g.lim || j >= g.ny - g.lim);
#pragma unroll
  for (int c = 0; c < 3; c++) invD[3 * n + c] = fixed ? 1.0 : 1.0 / d[c];
}

void fine_inv_diag(tp_ctx* c, double* invD) {
  ProfScope ps(c, P_ASSEMBLE);
  const long nn = c->L[0].nnodes;
  fine_diag_kernel<<<grid_for(nn, 256), 256, 0, c->s>>>(geom(c), c->d_E, invD);
  TP_CHECK_LAUNCH(c, "fine_inv_diag");
}

// E = Emin + rho^3 (E0 - Emin) (stencil_methods.c:96-97), E0 = 1, Emin = 1e-6
__global__ void compute_E_kernel(long ne, const double* __restrict__ x, double* __restrict__ E,
                                 float* __restrict__ Ef) {
  const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const double xe = x[e];
  const double v = 1e-6 + xe * xe * xe * (1.0 - 1e-6);
  E[e] = v;
  Ef[e] = (float)v;
}

void compute_E(tp_ctx* c) {
  const long ne = (long)c->L[0].ex * c->L[0].ey * c->L[0].ez;
  compute_E_kernel<<<grid_for(ne, 256), 256, 0, c->s>>>(ne, c->d_xphys, c->d_E, c->d_Ef);
  TP_CHECK_LAUNCH(c, "compute_E");
}

}  // namespace tp
