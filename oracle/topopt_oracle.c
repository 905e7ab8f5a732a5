/*
 * CPU oracle: plain-C FP64 restatement of the reference's hot path.
 * TEST INFRASTRUCTURE ONLY (see topopt_oracle.h). Each function cites the
 * reference lines it follows. Built with -ffp-contract=off so that x86 and
 * aarch64 hosts give the same bits.
 */
#include "topopt_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

#define OR_MAX(a, b) ((a) > (b) ? (a) : (b))
#define OR_MIN(a, b) ((a) > (b) ? (b) : (a))

/* local node q of a hex element -> offset (dx, dy, dz) from its (i, j, k)
 * corner, in the order of getEdof_halo (stencil_utility.h:19-52) */
static const int kLocal[8][3] = {{0, 1, 0}, {1, 1, 0}, {1, 0, 0}, {0, 0, 0},
                                 {0, 1, 1}, {1, 1, 1}, {1, 0, 1}, {0, 0, 1}};

static inline int lx(const OrGrid *g, int l) { return g->nelx >> l; }
static inline int ly(const OrGrid *g, int l) { return g->nely >> l; }
static inline int lz(const OrGrid *g, int l) { return g->nelz >> l; }

size_t or_nnodes(const OrGrid *g, int l) {
  return (size_t)(lx(g, l) + 1) * (ly(g, l) + 1) * (lz(g, l) + 1);
}
size_t or_nelem(const OrGrid *g) { return (size_t)g->nelx * g->nely * g->nelz; }

/* ------------------------------------------------------------------------ */
/* Element stiffness: getC (local_matrix.c:7-29), getB (:33-247),
 * getKEsubspace (:251-319). The float operations and their order are kept,
 * with the reference's two dgemm calls written as triple loops. */
static void or_getC(double C[6][6], double nu) {
  const double t1 = (1.0 - nu) / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double t2 = nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double t3 = 1.0 / (2.0 * (1.0 + nu));
  memset(C, 0, sizeof(double) * 36);
  C[0][0] = C[1][1] = C[2][2] = t1;
  C[3][3] = C[4][4] = C[5][5] = t3;
  C[0][1] = C[1][0] = C[0][2] = C[2][0] = C[1][2] = C[2][1] = t2;
}

static void or_getB(double B[6][24], double *jdet, const double iso[3],
                    const double xe[24]) {
  const double xi = iso[0], eta = iso[1], zeta = iso[2];
  double d[8][3]; /* d/dxi, d/deta, d/dzeta of the 8 trilinear functions */
  d[0][0] = -0.125 * (1 - eta) * (1 - zeta);
  d[0][1] = -0.125 * (1 - xi) * (1 - zeta);
  d[0][2] = -0.125 * (1 - xi) * (1 - eta);
  d[1][0] = 0.125 * (1 - eta) * (1 - zeta);
  d[1][1] = -0.125 * (1 + xi) * (1 - zeta);
  d[1][2] = -0.125 * (1 + xi) * (1 - eta);
  d[2][0] = 0.125 * (1 + eta) * (1 - zeta);
  d[2][1] = 0.125 * (1 + xi) * (1 - zeta);
  d[2][2] = -0.125 * (1 + xi) * (1 + eta);
  d[3][0] = -0.125 * (1 + eta) * (1 - zeta);
  d[3][1] = 0.125 * (1 - xi) * (1 - zeta);
  d[3][2] = -0.125 * (1 - xi) * (1 + eta);
  d[4][0] = -0.125 * (1 - eta) * (1 + zeta);
  d[4][1] = -0.125 * (1 - xi) * (1 + zeta);
  d[4][2] = 0.125 * (1 - xi) * (1 - eta);
  d[5][0] = 0.125 * (1 - eta) * (1 + zeta);
  d[5][1] = -0.125 * (1 + xi) * (1 + zeta);
  d[5][2] = 0.125 * (1 + xi) * (1 - eta);
  d[6][0] = 0.125 * (1 + eta) * (1 + zeta);
  d[6][1] = 0.125 * (1 + xi) * (1 + zeta);
  d[6][2] = 0.125 * (1 + xi) * (1 + eta);
  d[7][0] = -0.125 * (1 + eta) * (1 + zeta);
  d[7][1] = 0.125 * (1 - xi) * (1 + zeta);
  d[7][2] = 0.125 * (1 - xi) * (1 + eta);

  double Nt[9][24];
  memset(Nt, 0, sizeof Nt);
  for (int c = 0; c < 3; c++)
    for (int q = 0; q < 8; q++)
      for (int r = 0; r < 3; r++) Nt[3 * c + r][3 * q + c] = d[q][r];

  double jac[3][3];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      double s = d[0][r] * xe[c];
      for (int q = 1; q < 8; q++) s = s + d[q][r] * xe[3 * q + c];
      jac[r][c] = s;
    }
  /* the reference's determinant reads jac[1][2] twice (local_matrix.c:204);
   * the Jacobian of an axis-aligned box is diagonal, so it is kept as is */
  *jdet = jac[0][0] * (jac[1][1] * jac[2][2] - jac[1][2] * jac[1][2]) -
          jac[0][1] * (jac[1][0] * jac[2][2] - jac[1][2] * jac[2][0]) +
          jac[0][2] * (jac[1][0] * jac[2][1] - jac[1][1] * jac[2][0]);
  double ji[9][9];
  memset(ji, 0, sizeof ji);
  const double inv = 1.0 / (*jdet);
  ji[0][0] = inv * (jac[1][1] * jac[2][2] - jac[1][2] * jac[1][2]);
  ji[0][1] = inv * -1.0 * (jac[1][0] * jac[2][2] - jac[1][2] * jac[2][0]);
  ji[0][2] = inv * (jac[1][0] * jac[2][1] - jac[1][1] * jac[2][0]);
  ji[1][0] = inv * -1.0 * (jac[0][1] * jac[2][2] - jac[0][2] * jac[2][1]);
  ji[1][1] = inv * (jac[0][0] * jac[2][2] - jac[0][2] * jac[2][0]);
  ji[1][2] = inv * -1.0 * (jac[0][0] * jac[2][1] - jac[0][1] * jac[2][0]);
  ji[2][0] = inv * (jac[0][1] * jac[1][2] - jac[0][2] * jac[1][1]);
  ji[2][1] = inv * -1.0 * (jac[0][0] * jac[1][2] - jac[0][2] * jac[1][0]);
  ji[2][2] = inv * (jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0]);
  for (int k = 1; k < 3; k++)
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) ji[3 * k + i][3 * k + j] = ji[i][j];

  double partial[9][24];
  for (int m = 0; m < 9; m++)
    for (int n = 0; n < 24; n++) {
      double acc = 0.0;
      for (int k = 0; k < 9; k++) acc += ji[m][k] * Nt[k][n];
      partial[m][n] = 1.0 * acc + 0.0;
    }
  /* strain rows: xx, yy, zz, xy, yz, zx (the L matrix of local_matrix.c:100-108) */
  static const int Lrows[6][2] = {{0, -1}, {4, -1}, {8, -1}, {1, 3}, {5, 7}, {2, 6}};
  for (int m = 0; m < 6; m++)
    for (int n = 0; n < 24; n++) {
      /* dgemm with the 0/1 matrix L: the k loop adds exact zeros except at
       * the listed rows, in ascending k order */
      double acc = 0.0;
      for (int k = 0; k < 9; k++) {
        const double Lmk = (k == Lrows[m][0] || k == Lrows[m][1]) ? 1.0 : 0.0;
        acc += Lmk * partial[k][n];
      }
      B[m][n] = 1.0 * acc + 0.0;
    }
}

void or_ke(double nu, int l, double *KE) {
  const int ncell = 1 << l;
  const int ip = 10;
  const double a = 0.5 * ncell, b = 0.5 * ncell, c = 0.5 * ncell;
  const double xe[24] = {-a, -b, -c, a, -b, -c, a, b, -c, -a, b, -c,
                         -a, -b, c,  a, -b, c,  a, b, c,  -a, b, c};
  double C[6][6];
  or_getC(C, nu);
  const double spacing = 2.0 / (double)ncell / (double)ip;
  const double vol = spacing * spacing * spacing;
  memset(KE, 0, sizeof(double) * 576 * ncell * ncell * ncell);
#pragma omp parallel for collapse(3) schedule(static)
  for (int ii = 0; ii < ncell; ii++)
    for (int kk = 0; kk < ncell; kk++)
      for (int jj = 0; jj < ncell; jj++) {
        double *K = KE + 576 * (ncell * ncell * ii + ncell * kk + jj);
        double B[6][24], P[24][6], jdet, iso[3];
        double igp = -1.0 + spacing / 2.0 + 2.0 / (double)ncell * ((double)ii);
        for (int a1 = 0; a1 < ip; a1++) {
          double jgp = -1.0 + spacing / 2.0 + 2.0 / (double)ncell * ((double)jj);
          for (int a2 = 0; a2 < ip; a2++) {
            double kgp = -1.0 + spacing / 2.0 + 2.0 / (double)ncell * ((double)kk);
            for (int a3 = 0; a3 < ip; a3++) {
              iso[0] = igp;
              iso[1] = -1.0 * jgp; /* the reference flips eta (local_matrix.c:297-298) */
              iso[2] = kgp;
              or_getB(B, &jdet, iso, xe);
              for (int m = 0; m < 24; m++)
                for (int n = 0; n < 6; n++) {
                  double acc = 0.0;
                  for (int k = 0; k < 6; k++) acc += B[k][m] * C[k][n];
                  P[m][n] = 1.0 * acc + 0.0;
                }
              const double alpha = jdet * vol;
              for (int m = 0; m < 24; m++)
                for (int n = 0; n < 24; n++) {
                  double acc = 0.0;
                  for (int k = 0; k < 6; k++) acc += P[m][k] * B[k][n];
                  K[24 * m + n] = alpha * acc + K[24 * m + n];
                }
              kgp += spacing;
            }
            jgp += spacing;
          }
          igp += spacing;
        }
      }
}

/* ------------------------------------------------------------------------ */
/* Boundary conditions: two y-edge strips of the x=0 face, per level
 * (stencil_grid_utility.c:34-59). */
int or_fixed_dofs(const OrGrid *g, int l, long *out) {
  const int ny = ly(g, l) + 1, nz = lz(g, l) + 1;
  const int lim = ly(g, l) / 4 + 1;
  int q = 0;
  for (int k = 0; k < nz; k++) {
    for (int j = 0; j < lim; j++)
      for (int c = 0; c < 3; c++, q++)
        if (out) out[q] = 3L * ((long)k * ny + j) + c;
    for (int j = ny - lim; j < ny; j++)
      for (int c = 0; c < 3; c++, q++)
        if (out) out[q] = 3L * ((long)k * ny + j) + c;
  }
  return q;
}

/* Cantilever load: -1 in z spread over the z=0 face nodes of the elements
 * within radius ny/5 of (x=nelx, y=(nely-1)/2) (stencil_optimization.c:37-95). */
void or_load(const OrGrid *g, double *F) {
  const int nelx = g->nelx, nely = g->nely;
  const int ny = nely + 1, nz = g->nelz + 1;
  memset(F, 0, sizeof(double) * 3 * or_nnodes(g, 0));
  const double radius = ((double)ny) / 5.0, r2 = radius * radius;
  const double cx = (double)nelx, cy = ((double)nely - 1.0) / 2.0;
  int cnt = 0;
  for (int i = 0; i < nelx; i++)
    for (int j = 0; j < nely; j++) {
      const double dx = (double)i - cx, dy = (double)j - cy;
      if (dx * dx + dy * dy < r2) cnt++;
    }
  const double f = -1.0 / (4.0 * (double)cnt);
  for (int i = 0; i < nelx; i++)
    for (int j = 0; j < nely; j++) {
      const double dx = (double)i - cx, dy = (double)j - cy;
      if (dx * dx + dy * dy < r2) {
        /* nodes (i+1,j+1), (i+1,j), (i,j+1), (i,j) of the z=0 face */
        F[3 * (((size_t)(i + 1) * nz + 0) * ny + (j + 1)) + 2] += f;
        F[3 * (((size_t)(i + 1) * nz + 0) * ny + j) + 2] += f;
        F[3 * (((size_t)i * nz + 0) * ny + (j + 1)) + 2] += f;
        F[3 * (((size_t)i * nz + 0) * ny + j) + 2] += f;
      }
    }
}

OrGrid *or_create(int nelx, int nely, int nelz, int nl) {
  OrGrid *g = calloc(1, sizeof(OrGrid));
  g->nelx = nelx; g->nely = nely; g->nelz = nelz; g->nl = nl;
  g->E0 = 1; g->Emin = 1e-6; g->nu = 0.3; /* stencil_grid_utility.c:69-72 */
  for (int l = 0; l < nl; l++) {
    const int nc = 1 << l;
    g->ke[l] = malloc(sizeof(double) * 576 * nc * nc * nc);
    or_ke(g->nu, l, g->ke[l]);
    g->nfixed[l] = or_fixed_dofs(g, l, NULL);
    g->fixed[l] = malloc(sizeof(long) * g->nfixed[l]);
    or_fixed_dofs(g, l, g->fixed[l]);
    g->isfixed[l] = calloc(3 * or_nnodes(g, l), 1);
    for (int q = 0; q < g->nfixed[l]; q++) g->isfixed[l][g->fixed[l][q]] = 1;
  }
  return g;
}

void or_destroy(OrGrid *g) {
  for (int l = 0; l < g->nl; l++) {
    free(g->ke[l]);
    free(g->fixed[l]);
    free(g->isfixed[l]);
  }
  free(g);
}

/* ------------------------------------------------------------------------ */
static inline double escale(const OrGrid *g, double x) {
  return g->Emin + x * x * x * (g->E0 - g->Emin);
}

/* element matrix of coarse element (i,k,j) of level l: sum over its ncell^3
 * fine sub-cells of E(x_fine) * KE_l[cell] (stencil_methods.c:484-501) */
static void element_matrix(const OrGrid *g, int l, const double *x, int i, int k,
                           int j, double Ke[576]) {
  const int nc = 1 << l;
  memset(Ke, 0, sizeof(double) * 576);
  for (int ii = 0; ii < nc; ii++)
    for (int kk = 0; kk < nc; kk++)
      for (int jj = 0; jj < nc; jj++) {
        const size_t e = ((size_t)(i * nc + ii) * g->nelz + (k * nc + kk)) * g->nely + (j * nc + jj);
        const double E = escale(g, x[e]);
        const double *K = g->ke[l] + 576 * (nc * nc * ii + nc * kk + jj);
        for (int q = 0; q < 576; q++) Ke[q] += E * K[q];
      }
}

static inline void element_dofs(int ny, int nz, int i, int k, int j, size_t dof[24]) {
  for (int q = 0; q < 8; q++) {
    const size_t n = ((size_t)(i + kLocal[q][0]) * nz + (k + kLocal[q][2])) * ny + (j + kLocal[q][1]);
    dof[3 * q] = 3 * n;
    dof[3 * q + 1] = 3 * n + 1;
    dof[3 * q + 2] = 3 * n + 2;
  }
}

/* out = K_l(x) in, identity rows at fixed DOFs, columns NOT zeroed: the
 * reference's level-0 stencil (stencil_methods.c:7-428) and level-l subspace
 * operator (:436-519) have these semantics. mask != NULL zeroes the input at
 * fixed DOFs first (the assembled CSR levels, stencil_assembly.c:226-259). */
static void apply_impl(const OrGrid *g, int l, const double *x, const double *in,
                       double *out, int masked) {
  const int ex = lx(g, l), ey = ly(g, l), ez = lz(g, l);
  const int ny = ey + 1, nz = ez + 1;
  const size_t ndof = 3 * or_nnodes(g, l);
  const unsigned char *fx = g->isfixed[l];
  memset(out, 0, sizeof(double) * ndof);
  for (int bx = 0; bx < 2; bx++)
    for (int bz = 0; bz < 2; bz++)
      for (int by = 0; by < 2; by++) {
#pragma omp parallel for collapse(2) schedule(static)
        for (int i = bx; i < ex; i += 2)
          for (int k = bz; k < ez; k += 2)
            for (int j = by; j < ey; j += 2) {
              double Ke[576], ue[24];
              size_t dof[24];
              element_matrix(g, l, x, i, k, j, Ke);
              element_dofs(ny, nz, i, k, j, dof);
              for (int a = 0; a < 24; a++)
                ue[a] = (masked && fx[dof[a]]) ? 0.0 : in[dof[a]];
              for (int a = 0; a < 24; a++) {
                double s = 0.0;
                for (int b = 0; b < 24; b++) s += Ke[24 * a + b] * ue[b];
                out[dof[a]] += s;
              }
            }
      }
  for (int q = 0; q < g->nfixed[l]; q++) out[g->fixed[l][q]] = in[g->fixed[l][q]];
}

void or_apply(const OrGrid *g, int l, const double *x, const double *in, double *out) {
  apply_impl(g, l, x, in, out, 0);
}
void or_apply_masked(const OrGrid *g, int l, const double *x, const double *in, double *out) {
  apply_impl(g, l, x, in, out, 1);
}

/* inverse Jacobi diagonal, every level (stencil_methods.c:693-773) */
void or_inv_diag(const OrGrid *g, int l, const double *x, double *invD) {
  const int ex = lx(g, l), ey = ly(g, l), ez = lz(g, l);
  const int ny = ey + 1, nz = ez + 1;
  const size_t ndof = 3 * or_nnodes(g, l);
  memset(invD, 0, sizeof(double) * ndof);
  const int nc = 1 << l;
  for (int bx = 0; bx < 2; bx++)
    for (int bz = 0; bz < 2; bz++)
      for (int by = 0; by < 2; by++) {
#pragma omp parallel for collapse(2) schedule(static)
        for (int i = bx; i < ex; i += 2)
          for (int k = bz; k < ez; k += 2)
            for (int j = by; j < ey; j += 2) {
              size_t dof[24];
              element_dofs(ny, nz, i, k, j, dof);
              for (int ii = 0; ii < nc; ii++)
                for (int kk = 0; kk < nc; kk++)
                  for (int jj = 0; jj < nc; jj++) {
                    const size_t e = ((size_t)(i * nc + ii) * g->nelz + (k * nc + kk)) * g->nely + (j * nc + jj);
                    const double E = escale(g, x[e]);
                    const double *K = g->ke[l] + 576 * (nc * nc * ii + nc * kk + jj);
                    for (int a = 0; a < 24; a++) invD[dof[a]] += E * K[24 * a + a];
                  }
            }
      }
  for (int q = 0; q < g->nfixed[l]; q++) invD[g->fixed[l][q]] = 1.0;
  for (size_t q = 0; q < ndof; q++) invD[q] = 1.0 / invD[q];
}

/* full-weighting restriction, coarse level l+1 <- fine level l
 * (stencil_methods.c:595-688): weights 1, .5, .25, .125 by squared distance */
void or_restrict(const OrGrid *g, int l, const double *fine, double *coarse) {
  static const double vals[4] = {1.0, 0.5, 0.25, 0.125};
  const int nxf = lx(g, l) + 1, nyf = ly(g, l) + 1, nzf = lz(g, l) + 1;
  const int nxc = lx(g, l + 1) + 1, nyc = ly(g, l + 1) + 1, nzc = lz(g, l + 1) + 1;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ic = 0; ic < nxc; ic++)
    for (int kc = 0; kc < nzc; kc++)
      for (int jc = 0; jc < nyc; jc++) {
        double acc[3] = {0, 0, 0};
        const int i1 = 2 * ic, j1 = 2 * jc, k1 = 2 * kc;
        for (int i = i1 - 1; i < i1 + 2; i++)
          for (int k = k1 - 1; k < k1 + 2; k++)
            for (int j = j1 - 1; j < j1 + 2; j++) {
              if (i < 0 || i >= nxf || j < 0 || j >= nyf || k < 0 || k >= nzf) continue;
              const int d2 = (i1 - i) * (i1 - i) + (j1 - j) * (j1 - j) + (k1 - k) * (k1 - k);
              const size_t n = ((size_t)i * nzf + k) * nyf + j;
              for (int c = 0; c < 3; c++) acc[c] += vals[d2] * fine[3 * n + c];
            }
        const size_t nc = ((size_t)ic * nzc + kc) * nyc + jc;
        for (int c = 0; c < 3; c++) coarse[3 * nc + c] = acc[c];
      }
}

/* trilinear prolongation, fine level l <- coarse level l+1
 * (stencil_methods.c:521-590) */
void or_prolong(const OrGrid *g, int l, const double *coarse, double *fine) {
  const int nxf = lx(g, l) + 1, nyf = ly(g, l) + 1, nzf = lz(g, l) + 1;
  const int nyc = ly(g, l + 1) + 1, nzc = lz(g, l + 1) + 1;
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < nxf; i++)
    for (int k = 0; k < nzf; k++)
      for (int j = 0; j < nyf; j++) {
        const int i1 = i >> 1, i2 = (i + 1) >> 1;
        const int j1 = j >> 1, j2 = (j + 1) >> 1;
        const int k1 = k >> 1, k2 = (k + 1) >> 1;
#define CN(a, b, c) (((size_t)(a) * nzc + (b)) * nyc + (c))
        const size_t c1 = CN(i1, k1, j2), c2 = CN(i2, k1, j2), c3 = CN(i2, k1, j1),
                     c4 = CN(i1, k1, j1), c5 = CN(i1, k2, j2), c6 = CN(i2, k2, j2),
                     c7 = CN(i2, k2, j1), c8 = CN(i1, k2, j1);
#undef CN
        const size_t n = ((size_t)i * nzf + k) * nyf + j;
        for (int c = 0; c < 3; c++)
          fine[3 * n + c] = 0.125 * coarse[3 * c1 + c] + 0.125 * coarse[3 * c2 + c] +
                            0.125 * coarse[3 * c3 + c] + 0.125 * coarse[3 * c4 + c] +
                            0.125 * coarse[3 * c5 + c] + 0.125 * coarse[3 * c6 + c] +
                            0.125 * coarse[3 * c7 + c] + 0.125 * coarse[3 * c8 + c];
      }
}

/* damped Jacobi sweeps u += omega*invD*(b - K u) (stencil_solvers.c:11-122);
 * levels >= 2 use the assembled, BC-masked operator */
void or_smooth(const OrGrid *g, int l, const double *x, int nswp, double omega,
               const double *invD, const double *b, double *u, double *tmp) {
  const size_t ndof = 3 * or_nnodes(g, l);
  for (int s = 0; s < nswp; s++) {
    apply_impl(g, l, x, u, tmp, l >= 2);
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < ndof; q++) u[q] += omega * invD[q] * (b[q] - tmp[q]);
  }
}

/* ------------------------------------------------------------------------ */
/* Coarsest level: the assembled operator with fixed rows and columns zeroed
 * and a unit diagonal (stencil_assembly.c:126-259), factored by a dense band
 * Cholesky in natural node order (standing in for CHOLMOD,
 * stencil_assembly.c:428-503). */
int or_coarse_factor(const OrGrid *g, int l, const double *x, OrCoarse *cs) {
  const int ex = lx(g, l), ey = ly(g, l), ez = lz(g, l);
  const int ny = ey + 1, nz = ez + 1;
  const size_t n = 3 * or_nnodes(g, l);
  const size_t bw = 3 * ((size_t)nz * ny + ny + 1) + 2;
  const size_t w = bw + 1;
  cs->l = l;
  cs->n = n;
  cs->bw = bw;
  cs->band = calloc(n * w, sizeof(double));
  double *B = cs->band;
  const unsigned char *fx = g->isfixed[l];
  for (int i = 0; i < ex; i++)
    for (int k = 0; k < ez; k++)
      for (int j = 0; j < ey; j++) {
        double Ke[576];
        size_t dof[24];
        element_matrix(g, l, x, i, k, j, Ke);
        element_dofs(ny, nz, i, k, j, dof);
        for (int a = 0; a < 24; a++)
          for (int b = 0; b < 24; b++)
            if (dof[a] >= dof[b]) B[dof[b] * w + (dof[a] - dof[b])] += Ke[24 * a + b];
      }
  for (size_t c = 0; c < n; c++)
    for (size_t r = c; r < n && r <= c + bw; r++)
      if (fx[r] || fx[c]) B[c * w + (r - c)] = (r == c) ? 1.0 : 0.0;
  int status = 0;
  for (size_t j = 0; j < n; j++) {
    double d = B[j * w];
    if (!(d > 0.0)) {
      status = -1;
      d = 1.0;
    }
    d = sqrt(d);
    B[j * w] = d;
    const size_t last = OR_MIN(j + bw, n - 1);
    for (size_t i = j + 1; i <= last; i++) B[j * w + (i - j)] /= d;
#pragma omp parallel for schedule(static) if (last - j > 64)
    for (long cc = (long)j + 1; cc <= (long)last; cc++) {
      const double ljc = B[j * w + ((size_t)cc - j)];
      double *col = B + (size_t)cc * w - (size_t)cc;
      const double *lj = B + j * w - j;
      for (size_t r = (size_t)cc; r <= last; r++) col[r] -= lj[r] * ljc;
    }
  }
  return status;
}

void or_coarse_solve(const OrCoarse *cs, const double *rhs, double *x) {
  const size_t n = cs->n, bw = cs->bw, w = bw + 1;
  const double *L = cs->band;
  memcpy(x, rhs, n * sizeof(double));
  for (size_t j = 0; j < n; j++) {
    x[j] /= L[j * w];
    const size_t last = OR_MIN(j + bw, n - 1);
    for (size_t i = j + 1; i <= last; i++) x[i] -= L[j * w + (i - j)] * x[j];
  }
  for (size_t jj = n; jj-- > 0;) {
    const size_t last = OR_MIN(jj + bw, n - 1);
    double s = x[jj];
    for (size_t i = jj + 1; i <= last; i++) s -= L[jj * w + (i - jj)] * x[i];
    x[jj] = s / L[jj * w];
  }
}

void or_coarse_free(OrCoarse *cs) {
  free(cs->band);
  cs->band = NULL;
}

/* factor + solve in one call, for checks of the coarse direct solve */
int or_coarse_direct(const OrGrid *g, int l, const double *x, const double *rhs, double *sol) {
  OrCoarse cs;
  const int st = or_coarse_factor(g, l, x, &cs);
  or_coarse_solve(&cs, rhs, sol);
  or_coarse_free(&cs);
  return st;
}

/* ------------------------------------------------------------------------ */
/* V-cycle (stencil_solvers.c:129-252) and PCG (:259-397) */
typedef struct {
  double *r[OR_MAXL], *z[OR_MAXL], *d[OR_MAXL], *invD[OR_MAXL];
  OrCoarse cs;
} OrMG;

static void vcycle(const OrGrid *g, const double *x, int l, OrMG *m, int nswp,
                   double omega) {
  const int nl = g->nl;
  const size_t nd = 3 * or_nnodes(g, l);
  memset(m->z[l], 0, nd * sizeof(double));
  or_smooth(g, l, x, nswp, omega, m->invD[l], m->r[l], m->z[l], m->d[l]);
  apply_impl(g, l, x, m->z[l], m->d[l], l >= 2);
  for (size_t q = 0; q < nd; q++) m->d[l][q] = m->r[l][q] - m->d[l][q];
  or_restrict(g, l, m->d[l], m->r[l + 1]);
  if (nl == l + 2)
    or_coarse_solve(&m->cs, m->r[l + 1], m->z[l + 1]);
  else
    vcycle(g, x, l + 1, m, nswp, omega);
  or_prolong(g, l, m->z[l + 1], m->d[l]);
  for (size_t q = 0; q < nd; q++) m->z[l][q] += m->d[l][q];
  or_smooth(g, l, x, nswp, omega, m->invD[l], m->r[l], m->z[l], m->d[l]);
}

static double dot(const double *a, const double *b, size_t n) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (size_t q = 0; q < n; q++) s += a[q] * b[q];
  return s;
}

int or_solve(const OrGrid *g, const double *x, const double *b, double *u,
             int nswp, double tol, int *iters, double *relres) {
  const int nl = g->nl;
  const size_t nd = 3 * or_nnodes(g, 0);
  OrMG m;
  memset(&m, 0, sizeof m);
  for (int l = 0; l < nl; l++) {
    const size_t n = 3 * or_nnodes(g, l);
    m.r[l] = calloc(n, sizeof(double));
    m.z[l] = calloc(n, sizeof(double));
    m.d[l] = calloc(n, sizeof(double));
    m.invD[l] = calloc(n, sizeof(double));
    or_inv_diag(g, l, x, m.invD[l]);
  }
  int status = or_coarse_factor(g, nl - 1, x, &m.cs);
  double *r = m.r[0], *z = m.z[0];
  double *p = calloc(nd, sizeof(double)), *q = calloc(nd, sizeof(double));
  memcpy(z, u, nd * sizeof(double));
  or_apply(g, 0, x, z, r);
  for (size_t i = 0; i < nd; i++) r[i] = b[i] - r[i];
  const double omega = 0.6;
  const double bnorm = sqrt(dot(b, b, nd));
  double rhoold = 0.0;
  int it = 0;
  for (int iter = 0; iter < 1000; iter++) {
    vcycle(g, x, 0, &m, nswp, omega);
    const double rho = dot(r, z, nd);
    if (iter == 0)
      memcpy(p, z, nd * sizeof(double));
    else {
      const double beta = rho / rhoold;
      for (size_t i = 0; i < nd; i++) p[i] = beta * p[i] + z[i];
    }
    or_apply(g, 0, x, p, q);
    const double dpr = dot(p, q, nd);
    const double alpha = rho / dpr;
    rhoold = rho;
    for (size_t i = 0; i < nd; i++) u[i] += alpha * p[i];
    for (size_t i = 0; i < nd; i++) r[i] -= alpha * q[i];
    const double rr = sqrt(dot(r, r, nd)) / bnorm;
    it = iter;
    *relres = (float)rr; /* the reference reports it through a float */
    if (rr < tol) break;
  }
  *iters = it;
  for (int l = 0; l < nl; l++) {
    free(m.r[l]); free(m.z[l]); free(m.d[l]); free(m.invD[l]);
  }
  or_coarse_free(&m.cs);
  free(p); free(q);
  return status;
}

/* ------------------------------------------------------------------------ */
/* compliance and sensitivity (stencil_methods.c:808-862), penalty 3 */
double or_compliance(const OrGrid *g, const double *x, const double *u, double *dc) {
  const int ex = g->nelx, ey = g->nely, ez = g->nelz;
  const int ny = ey + 1, nz = ez + 1;
  const double *KE = g->ke[0];
  const double Ed = g->E0 - g->Emin;
  double c = 0.0;
#pragma omp parallel for collapse(2) reduction(+ : c) schedule(static)
  for (int i = 0; i < ex; i++)
    for (int k = 0; k < ez; k++)
      for (int j = 0; j < ey; j++) {
        size_t dof[24];
        element_dofs(ny, nz, i, k, j, dof);
        const size_t e = ((size_t)i * ez + k) * ey + j;
        const double xe = x[e];
        double d = 0.0;
        for (int ii = 0; ii < 8; ii++) {
          double cl = 0.0;
          for (int a = 0; a < 3; a++) {
            double t = 0.0;
            for (int b = 0; b < 24; b++) t += KE[(ii * 3 + a) * 24 + b] * u[dof[b]];
            cl += u[dof[3 * ii + a]] * t;
          }
          c += cl * (g->Emin + xe * xe * xe * Ed);
          d += cl * (-3.0 * Ed * xe * xe);
        }
        dc[e] = d;
      }
  return c;
}

/* density filter and its adjoint (stencil_optimization.c:228-395); the
 * neighbourhood box is [i-(ceil(rmin)-1), i+ceil(rmin)] clipped to the grid,
 * with weights max(0, rmin - |d|) */
static void filter_box(const OrGrid *g, double rmin, int i, int n, int *lo, int *hi) {
  const int c = (int)ceil(rmin);
  *lo = OR_MAX(i - (c - 1), 0);
  *hi = OR_MIN(i + c + 1, n); /* exclusive */
}

void or_filter(const OrGrid *g, double rmin, const double *x, double *out) {
  const int ex = g->nelx, ey = g->nely, ez = g->nelz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < ex; i++)
    for (int k = 0; k < ez; k++)
      for (int j = 0; j < ey; j++) {
        double o = 0.0, hs = 0.0;
        int i0, i1, k0, k1, j0, j1;
        filter_box(g, rmin, i, ex, &i0, &i1);
        filter_box(g, rmin, k, ez, &k0, &k1);
        filter_box(g, rmin, j, ey, &j0, &j1);
        for (int i2 = i0; i2 < i1; i2++)
          for (int k2 = k0; k2 < k1; k2++)
            for (int j2 = j0; j2 < j1; j2++) {
              const unsigned d2 = (unsigned)((i - i2) * (i - i2) + (j - j2) * (j - j2) + (k - k2) * (k - k2));
              const double w = OR_MAX(0.0, rmin - sqrt((double)d2));
              o += w * x[((size_t)i2 * ez + k2) * ey + j2];
              hs += w;
            }
        out[((size_t)i * ez + k) * ey + j] = o / hs;
      }
}

void or_filter_T(const OrGrid *g, double rmin, double *v) {
  const int ex = g->nelx, ey = g->nely, ez = g->nelz;
  const size_t ne = or_nelem(g);
  double *tmp = malloc(sizeof(double) * ne);
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < ex; i++)
    for (int k = 0; k < ez; k++)
      for (int j = 0; j < ey; j++) {
        double hs = 0.0;
        int i0, i1, k0, k1, j0, j1;
        filter_box(g, rmin, i, ex, &i0, &i1);
        filter_box(g, rmin, k, ez, &k0, &k1);
        filter_box(g, rmin, j, ey, &j0, &j1);
        for (int i2 = i0; i2 < i1; i2++)
          for (int k2 = k0; k2 < k1; k2++)
            for (int j2 = j0; j2 < j1; j2++) {
              const unsigned d2 = (unsigned)((i - i2) * (i - i2) + (j - j2) * (j - j2) + (k - k2) * (k - k2));
              hs += OR_MAX(0.0, rmin - sqrt((double)d2));
            }
        const size_t e = ((size_t)i * ez + k) * ey + j;
        tmp[e] = v[e] / hs;
      }
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < ex; i++)
    for (int k = 0; k < ez; k++)
      for (int j = 0; j < ey; j++) {
        double s = 0.0;
        int i0, i1, k0, k1, j0, j1;
        filter_box(g, rmin, i, ex, &i0, &i1);
        filter_box(g, rmin, k, ez, &k0, &k1);
        filter_box(g, rmin, j, ey, &j0, &j1);
        for (int i2 = i0; i2 < i1; i2++)
          for (int k2 = k0; k2 < k1; k2++)
            for (int j2 = j0; j2 < j1; j2++) {
              const unsigned d2 = (unsigned)((i - i2) * (i - i2) + (j - j2) * (j - j2) + (k - k2) * (k - k2));
              const double w = OR_MAX(0.0, rmin - sqrt((double)d2));
              s += w * tmp[((size_t)i2 * ez + k2) * ey + j2];
            }
        v[((size_t)i * ez + k) * ey + j] = s;
      }
  free(tmp);
}

/* OC bisection on the volume multiplier (gpu_definitions.c:127-157) */
void or_oc_update(const OrGrid *g, const double *x, const double *dv,
                  const double *dc, double gvol, double *xnew) {
  const size_t ne = or_nelem(g);
  double l1 = 0.0, l2 = 1e9;
  const double move = 0.2;
  while ((l2 - l1) / (l1 + l2) > 1e-6) {
    const double lmid = 0.5 * (l2 + l1);
    double gt = 0.0;
#pragma omp parallel for reduction(+ : gt) schedule(static)
    for (size_t e = 0; e < ne; e++) {
      const double xs = x[e] * sqrt(-dc[e] / (dv[e] * lmid));
      const double a = OR_MIN(x[e] + move, xs);
      const double b = OR_MIN(1.0, a);
      const double c = OR_MAX(x[e] - move, b);
      xnew[e] = OR_MAX(0.0, c);
      gt += dv[e] * (xnew[e] - x[e]);
    }
    gt += gvol;
    if (gt > 0)
      l1 = lmid;
    else
      l2 = lmid;
  }
}

double or_volume(const OrGrid *g, const double *xPhys) {
  const size_t ne = or_nelem(g);
  double v = 0.0;
#pragma omp parallel for reduction(+ : v) schedule(static)
  for (size_t e = 0; e < ne; e++) v += xPhys[e];
  return v;
}

/* max |x - xnew| through a float accumulator, then x <- xnew
 * (gpu_definitions.c:110-125) */
float or_change(const OrGrid *g, double *x, const double *xnew) {
  const size_t ne = or_nelem(g);
  float ch = 0.0f;
  for (size_t e = 0; e < ne; e++) {
    const double d = fabs(x[e] - xnew[e]);
    ch = (float)OR_MAX((double)ch, d);
    x[e] = xnew[e];
  }
  return ch;
}

/* ------------------------------------------------------------------------ */
/* the design loop (stencil_optimization.c:97-189) */
int or_run(int nelx, int nely, int nelz, double volfrac, double rmin, int nl,
           double cgtol, int max_iterations, OrHistory *h, double *xPhys_out,
           double *u_out) {
  OrGrid *g = or_create(nelx, nely, nelz, nl);
  const size_t ne = or_nelem(g), nd = 3 * or_nnodes(g, 0);
  double *F = malloc(nd * sizeof(double)), *U = calloc(nd, sizeof(double));
  or_load(g, F);
  double *x = malloc(ne * sizeof(double)), *xPhys = malloc(ne * sizeof(double));
  double *xnew = calloc(ne, sizeof(double)), *dc = calloc(ne, sizeof(double));
  double *dv = malloc(ne * sizeof(double));
  for (size_t e = 0; e < ne; e++) {
    x[e] = volfrac;
    xPhys[e] = volfrac;
    dv[e] = 1.0;
  }
  or_filter_T(g, rmin, dv);
  int loop = 0;
  float change = 1.0f;
  while (change > 1e-2 && loop < max_iterations) {
    loop++;
    const double t_iter = omp_get_wtime();
    int cgiter;
    double cgres;
    or_solve(g, xPhys, F, U, 4, cgtol, &cgiter, &cgres);
    double vol = or_volume(g, xPhys);
    const double c = or_compliance(g, xPhys, U, dc);
    or_filter_T(g, rmin, dc);
    vol /= (double)((size_t)nelx * nely * nelz);
    const double gv = vol - volfrac;
    or_oc_update(g, x, dv, dc, gv, xnew);
    change = or_change(g, x, xnew);
    or_filter(g, rmin, x, xPhys);
    if (h && loop <= 1024) {
      h->c[loop - 1] = c;
      h->vol[loop - 1] = vol;
      h->change[loop - 1] = change;
      h->cgiters[loop - 1] = cgiter;
      h->seconds[loop - 1] = omp_get_wtime() - t_iter;
      h->relres[loop - 1] = cgres;
    }
  }
  if (h) h->loops = loop;
  if (xPhys_out) memcpy(xPhys_out, xPhys, ne * sizeof(double));
  if (u_out) memcpy(u_out, U, nd * sizeof(double));
  free(F); free(U); free(x); free(xPhys); free(xnew); free(dc); free(dv);
  or_destroy(g);
  return loop;
}
