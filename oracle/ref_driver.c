/*
 * Flat C entry points over the reference's OWN functions, compiled together
 * with (mechanically patched copies of) the reference's sources by
 * oracle/build_ref.sh into oracle/_ref/libref{32,64}.so.
 *
 * TEST INFRASTRUCTURE ONLY: used here, in this container, to generate the
 * golden fixtures under tests/golden/ and to pin the oracle restatement
 * (oracle/topopt_oracle.c). Nothing in the product library links or calls it.
 *
 * All arrays crossing this interface are double and use the UNPADDED
 * canonical layout: node (i,k,j) of level l at n = (i*nz_l + k)*ny_l + j,
 * DOF 3n+c; fine element (i,k,j) at (i*nelz + k)*nely + j. The driver
 * converts to the reference's halo/padded layout (gpu_definitions.c:67-92)
 * and to its CTYPE/DTYPE.
 */
#include "definitions.h"
#include "gpu_definitions.h"
#include "local_matrix.h"
#include "stencil_assembly.h"
#include "stencil_grid_utility.h"
#include "stencil_methods.h"
#include "stencil_optimization.h"
#include "stencil_solvers.h"
#include "stencil_utility.h"

#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  struct gridContext gc;
  struct gpuGrid gpu;
  int nl;
} RefCtx;

static void dims(const RefCtx *c, int l, int *nelx, int *nely, int *nelz,
                 int *wx, int *wy, int *wz, uint_fast32_t *ndof) {
  int ncell;
  computePadding(&c->gc, l, &ncell, wx, wy, wz, ndof);
  *nelx = (int)c->gc.nelx / ncell;
  *nely = (int)c->gc.nely / ncell;
  *nelz = (int)c->gc.nelz / ncell;
}

void *ref_create(int nelx, int nely, int nelz, int nl) {
  RefCtx *c = calloc(1, sizeof(RefCtx));
  c->nl = nl;
  setupGC(&c->gc, nl, nelx, nely, nelz);
  c->gpu.num_targets = 1;
  gridContextToGPUGrid(&c->gc, &c->gpu, nl, 0);
  return c;
}

void ref_destroy(void *p) {
  RefCtx *c = p;
  freeGC(&c->gc, c->nl);
  freeGPUGrid(&c->gpu, c->nl);
  free(c);
}

/* ---- layout conversion ---- */
static CTYPE *vec_to_padded(const RefCtx *c, int l, const double *v) {
  int ex, ey, ez, wx, wy, wz;
  uint_fast32_t ndof;
  dims(c, l, &ex, &ey, &ez, &wx, &wy, &wz, &ndof);
  CTYPE *p = calloc(ndof, sizeof(CTYPE));
  const int nx = ex + 1, ny = ey + 1, nz = ez + 1;
  if (v)
    for (int i = 0; i < nx; i++)
      for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
          for (int d = 0; d < 3; d++)
            p[3 * ((size_t)(i + 1) * wy * wz + (size_t)(k + 1) * wy + (j + 1)) + d] =
                (CTYPE)v[3 * (((size_t)i * nz + k) * ny + j) + d];
  return p;
}

static void vec_from_padded(const RefCtx *c, int l, const CTYPE *p, double *v) {
  int ex, ey, ez, wx, wy, wz;
  uint_fast32_t ndof;
  dims(c, l, &ex, &ey, &ez, &wx, &wy, &wz, &ndof);
  const int nx = ex + 1, ny = ey + 1, nz = ez + 1;
  for (int i = 0; i < nx; i++)
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++)
        for (int d = 0; d < 3; d++)
          v[3 * (((size_t)i * nz + k) * ny + j) + d] =
              (double)p[3 * ((size_t)(i + 1) * wy * wz + (size_t)(k + 1) * wy + (j + 1)) + d];
}

static size_t nelem_padded(const RefCtx *c) {
  return (size_t)(c->gc.wrapx - 1) * (c->gc.wrapy - 1) * (c->gc.wrapz - 1);
}

static DTYPE *el_to_padded(const RefCtx *c, const double *x) {
  const size_t ne = nelem_padded(c);
  DTYPE *p = calloc(ne, sizeof(DTYPE));
  const int ex = c->gc.nelx, ey = c->gc.nely, ez = c->gc.nelz;
  const int wy = c->gc.wrapy - 1, wz = c->gc.wrapz - 1;
  if (x)
    for (int i = 0; i < ex; i++)
      for (int k = 0; k < ez; k++)
        for (int j = 0; j < ey; j++)
          p[(size_t)(i + 1) * wy * wz + (size_t)(k + 1) * wy + (j + 1)] =
              (DTYPE)x[((size_t)i * ez + k) * ey + j];
  return p;
}

static void el_from_padded(const RefCtx *c, const DTYPE *p, double *x) {
  const int ex = c->gc.nelx, ey = c->gc.nely, ez = c->gc.nelz;
  const int wy = c->gc.wrapy - 1, wz = c->gc.wrapz - 1;
  for (int i = 0; i < ex; i++)
    for (int k = 0; k < ez; k++)
      for (int j = 0; j < ey; j++)
        x[((size_t)i * ez + k) * ey + j] =
            (double)p[(size_t)(i + 1) * wy * wz + (size_t)(k + 1) * wy + (j + 1)];
}

/* ---- set-up data ---- */
int ref_sizeof_ctype(void) { return (int)sizeof(CTYPE); }
int ref_sizeof_dtype(void) { return (int)sizeof(DTYPE); }

void ref_ke(void *p, int l, double *out) {
  RefCtx *c = p;
  const int ncell = 1 << l;
  memcpy(out, c->gc.precomputedKE[l], sizeof(double) * 576 * ncell * ncell * ncell);
}

/* fixed DOFs of level l as canonical DOF indices, in the reference's order */
int ref_fixed_dofs(void *p, int l, long *out) {
  RefCtx *c = p;
  int ex, ey, ez, wx, wy, wz;
  uint_fast32_t ndof;
  dims(c, l, &ex, &ey, &ez, &wx, &wy, &wz, &ndof);
  const int n = (int)c->gc.fixedDofs[l].n;
  for (int q = 0; q < n && out; q++) {
    const long idx = (long)c->gc.fixedDofs[l].idx[q];
    out[q] = haloToTrue((int)idx, wy, wz, ey + 1, ez + 1);
  }
  return n;
}

/* ---- operators ---- */
void ref_matvec(void *p, int l, const double *x, const double *in, double *out) {
  RefCtx *c = p;
  DTYPE *xp = el_to_padded(c, x);
  CTYPE *ip = vec_to_padded(c, l, in);
  CTYPE *op = vec_to_padded(c, l, NULL);
  if (l == 0)
    applyStateOperator_stencil(&c->gpu.target[0], xp, ip, op);
  else
    applyStateOperatorSubspace_halo(&c->gpu.target[0], l, xp, ip, op);
  vec_from_padded(c, l, op, out);
  free(xp); free(ip); free(op);
}

/* assembled CSR operator of level l >= 2 (zeroed fixed rows/cols) */
void ref_matvec_csr(void *p, int l, const double *x, const double *in, double *out) {
  RefCtx *c = p;
  DTYPE *xp = el_to_padded(c, x);
  CTYPE *ip = vec_to_padded(c, l, in);
  CTYPE *op = vec_to_padded(c, l, NULL);
  int ex, ey, ez, wx, wy, wz;
  uint_fast32_t ndof;
  dims(c, l, &ex, &ey, &ez, &wx, &wy, &wz, &ndof);
  MTYPE *tmp = calloc(ndof, sizeof(MTYPE));
  struct CSRMatrix M;
  allocateSubspaceMatrix(c->gc, l, &M);
  assembleSubspaceMatrix(c->gc, l, xp, M, tmp);
  applyStateOperatorSubspaceMatrix(c->gc, l, M, ip, op);
  vec_from_padded(c, l, op, out);
  freeSubspaceMatrix(&M);
  free(tmp); free(xp); free(ip); free(op);
}

/* assembled CSR matrix of level l in canonical (unpadded) numbering */
long ref_csr(void *p, int l, const double *x, int *rowptr, int *col, double *val) {
  RefCtx *c = p;
  DTYPE *xp = el_to_padded(c, x);
  int ex, ey, ez, wx, wy, wz;
  uint_fast32_t ndof;
  dims(c, l, &ex, &ey, &ez, &wx, &wy, &wz, &ndof);
  MTYPE *tmp = calloc(ndof, sizeof(MTYPE));
  struct CSRMatrix M;
  allocateSubspaceMatrix(c->gc, l, &M);
  assembleSubspaceMatrix(c->gc, l, xp, M, tmp);
  const long nnz = (long)M.nnz;
  if (rowptr) {
    memcpy(rowptr, M.rowOffsets, sizeof(int) * (M.nrows + 1));
    memcpy(col, M.colIndex, sizeof(int) * nnz);
    memcpy(val, M.vals, sizeof(double) * nnz);
  }
  freeSubspaceMatrix(&M);
  free(tmp); free(xp);
  return nnz;
}

void ref_inv_diag(void *p, int l, const double *x, double *out) {
  RefCtx *c = p;
  DTYPE *xp = el_to_padded(c, x);
  int ex, ey, ez, wx, wy, wz;
  uint_fast32_t ndof;
  dims(c, l, &ex, &ey, &ez, &wx, &wy, &wz, &ndof);
  MTYPE *d = calloc(ndof, sizeof(MTYPE));
  assembleInvertedMatrixDiagonalSubspace_halo(&c->gpu.target[0], xp, l, d);
  const int nx = ex + 1, ny = ey + 1, nz = ez + 1;
  for (int i = 0; i < nx; i++)
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++)
        for (int q = 0; q < 3; q++)
          out[3 * (((size_t)i * nz + k) * ny + j) + q] =
              d[3 * ((size_t)(i + 1) * wy * wz + (size_t)(k + 1) * wy + (j + 1)) + q];
  free(d); free(xp);
}

/* coarse (level l+1) <- fine (level l) */
void ref_restrict(void *p, int l, const double *fine, double *coarse) {
  RefCtx *c = p;
  CTYPE *fp = vec_to_padded(c, l, fine);
  CTYPE *cp = vec_to_padded(c, l + 1, NULL);
  projectToCoarserGrid_halo(&c->gpu.target[0], l, fp, cp);
  vec_from_padded(c, l + 1, cp, coarse);
  free(fp); free(cp);
}

/* fine (level l) <- coarse (level l+1) */
void ref_prolong(void *p, int l, const double *coarse, double *fine) {
  RefCtx *c = p;
  CTYPE *cp = vec_to_padded(c, l + 1, coarse);
  CTYPE *fp = vec_to_padded(c, l, NULL);
  projectToFinerGrid_halo(&c->gpu.target[0], l, cp, fp);
  vec_from_padded(c, l, fp, fine);
  free(fp); free(cp);
}

/* damped Jacobi, nswp sweeps, on level 0 (stencil) or level l>=1 (subspace) */
void ref_smooth(void *p, int l, const double *x, int nswp, double omega,
                const double *b, double *u) {
  RefCtx *c = p;
  int ex, ey, ez, wx, wy, wz;
  uint_fast32_t ndof;
  dims(c, l, &ex, &ey, &ez, &wx, &wy, &wz, &ndof);
  DTYPE *xp = el_to_padded(c, x);
  CTYPE *bp = vec_to_padded(c, l, b);
  CTYPE *up = vec_to_padded(c, l, u);
  CTYPE *tp = vec_to_padded(c, l, NULL);
  MTYPE *d = calloc(ndof, sizeof(MTYPE));
  assembleInvertedMatrixDiagonalSubspace_halo(&c->gpu.target[0], xp, l, d);
  if (l == 0)
    smoothDampedJacobi_halo(&c->gpu.target[0], xp, nswp, (CTYPE)omega, d, up, bp, tp);
  else
    smoothDampedJacobiSubspace_halo(&c->gpu.target[0], xp, l, nswp, (CTYPE)omega, d, up, bp, tp);
  vec_from_padded(c, l, up, u);
  free(d); free(xp); free(bp); free(up); free(tp);
}

void ref_compliance(void *p, const double *x, const double *u, double *cout,
                    double *dc) {
  RefCtx *c = p;
  DTYPE *xp = el_to_padded(c, x);
  CTYPE *ut = vec_to_padded(c, 0, u);
  uint_fast32_t ndof = 3 * c->gc.wrapx * c->gc.wrapy * c->gc.wrapz;
  STYPE *up = calloc(ndof, sizeof(STYPE));
  for (size_t q = 0; q < ndof; q++) up[q] = (STYPE)ut[q];
  /* STYPE is double in both flavours: copy u at full precision */
  {
    const int nx = c->gc.nelx + 1, ny = c->gc.nely + 1, nz = c->gc.nelz + 1;
    const int wy = c->gc.wrapy, wz = c->gc.wrapz;
    for (int i = 0; i < nx; i++)
      for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
          for (int d = 0; d < 3; d++)
            up[3 * ((size_t)(i + 1) * wy * wz + (size_t)(k + 1) * wy + (j + 1)) + d] =
                u[3 * (((size_t)i * nz + k) * ny + j) + d];
  }
  DTYPE *dcp = calloc(nelem_padded(c), sizeof(DTYPE));
  DTYPE cc = 0;
  getComplianceAndSensetivity_halo(&c->gpu.target[0], xp, up, &cc, dcp);
  *cout = (double)cc;
  el_from_padded(c, dcp, dc);
  free(xp); free(ut); free(up); free(dcp);
}

void ref_filter(void *p, double rmin, const double *x, double *out) {
  RefCtx *c = p;
  DTYPE *xp = el_to_padded(c, x);
  DTYPE *op = el_to_padded(c, NULL);
  applyDensityFilter(c->gc, (DTYPE)rmin, xp, op);
  el_from_padded(c, op, out);
  free(xp); free(op);
}

void ref_filter_T(void *p, double rmin, double *v) {
  RefCtx *c = p;
  DTYPE *vp = el_to_padded(c, v);
  applyDensityFilterGradient(c->gc, (DTYPE)rmin, vp);
  el_from_padded(c, vp, v);
  free(vp);
}

/* OC bisection step over the padded element array; dv is 1 on halo
 * elements and dc 0 there, as in the reference's driver. */
void ref_oc_update(void *p, const double *x, const double *dv, const double *dc,
                   double g, double *xnew) {
  RefCtx *c = p;
  const size_t ne = nelem_padded(c);
  DTYPE *xp = el_to_padded(c, x);
  DTYPE *dcp = el_to_padded(c, dc);
  DTYPE *dvp = el_to_padded(c, dv);
  DTYPE *xn = el_to_padded(c, NULL);
  {
    /* halo elements of dv are 1, as the driver initialises them */
    DTYPE *ones = el_to_padded(c, NULL);
    for (size_t q = 0; q < ne; q++) ones[q] = 1.0;
    const int ex = c->gc.nelx, ey = c->gc.nely, ez = c->gc.nelz;
    const int wy = c->gc.wrapy - 1, wz = c->gc.wrapz - 1;
    for (int i = 0; i < ex; i++)
      for (int k = 0; k < ez; k++)
        for (int j = 0; j < ey; j++) {
          const size_t q = (size_t)(i + 1) * wy * wz + (size_t)(k + 1) * wy + (j + 1);
          ones[q] = dvp[q];
        }
    free(dvp);
    dvp = ones;
  }
  update_solution(xp, xn, dvp, dcp, (int)ne, (DTYPE)g);
  el_from_padded(c, xn, xnew);
  free(xp); free(dcp); free(dvp); free(xn);
}

/* one preconditioned CG solve, warm-started from u (in/out) */
void ref_solve(void *p, const double *x, const double *b, double *u, int nswp,
               double tol, int *iters, double *relres) {
  RefCtx *c = p;
  const int nl = c->nl;
  struct SolverDataBuffer sd;
  allocateSolverData(c->gc, nl, &sd);
  initializeCholmod(c->gc, nl - 1, &sd.bottomSolver, sd.coarseMatrices[nl - 1]);
  DTYPE *xp = el_to_padded(c, x);
  CTYPE *bp = vec_to_padded(c, 0, b);
  uint_fast32_t ndof = 3 * c->gc.wrapx * c->gc.wrapy * c->gc.wrapz;
  STYPE *up = calloc(ndof, sizeof(STYPE));
  {
    const int nx = c->gc.nelx + 1, ny = c->gc.nely + 1, nz = c->gc.nelz + 1;
    const int wy = c->gc.wrapy, wz = c->gc.wrapz;
    for (int i = 0; i < nx; i++)
      for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
          for (int d = 0; d < 3; d++)
            up[3 * ((size_t)(i + 1) * wy * wz + (size_t)(k + 1) * wy + (j + 1)) + d] =
                u[3 * (((size_t)i * nz + k) * ny + j) + d];
  }
  int it = 0;
  float rr = 0;
  solveStateMG_halo(&c->gpu, xp, nswp, nl, (CTYPE)tol, &sd, &it, &rr, bp, up);
  {
    const int nx = c->gc.nelx + 1, ny = c->gc.nely + 1, nz = c->gc.nelz + 1;
    const int wy = c->gc.wrapy, wz = c->gc.wrapz;
    for (int i = 0; i < nx; i++)
      for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
          for (int d = 0; d < 3; d++)
            u[3 * (((size_t)i * nz + k) * ny + j) + d] =
                up[3 * ((size_t)(i + 1) * wy * wz + (size_t)(k + 1) * wy + (j + 1)) + d];
  }
  *iters = it;
  *relres = rr;
  finishCholmod(c->gc, nl - 1, &sd.bottomSolver, sd.coarseMatrices[nl - 1], 0);
  freeSolverData(&sd, nl);
  free(xp); free(bp); free(up);
}

/* the reference's cantilever load vector (stencil_optimization.c:37-95) is set
 * up inside top3dmgcg; this restates that block so the design loop below can
 * run the reference's functions in the driver's order */
static void cantilever_load(const struct gridContext *g, CTYPE *F) {
  const int nelx = g->nelx, nely = g->nely;
  const double forceMagnitude = -1;
  const int ny = nely + 1;
  const int k = 0;
  const double radius = ((double)ny) / 5.0;
  const double radius2 = radius * radius;
  const double center_x = (double)nelx;
  const double center_y = ((double)nely - 1.0) / 2.0;
  int num_elements = 0;
  for (int i = 0; i < nelx; i++)
    for (int j = 0; j < nely; j++) {
      const double dx = (double)i - center_x, dy = (double)j - center_y;
      if (dx * dx + dy * dy < radius2) num_elements++;
    }
  const double nodalForce = forceMagnitude / (4.0 * (double)num_elements);
  for (int i = 0; i < nelx; i++)
    for (int j = 0; j < nely; j++) {
      const int ii = i + 1, jj = j + 1, kk = k + 1;
      const double dx = (double)i - center_x, dy = (double)j - center_y;
      if (dx * dx + dy * dy < radius2) {
        const size_t wyz = (size_t)g->wrapy * g->wrapz;
        const size_t n1 = (ii + 1) * wyz + g->wrapy * kk + (jj + 1);
        const size_t n2 = (ii + 1) * wyz + g->wrapy * kk + jj;
        const size_t n3 = ii * wyz + g->wrapy * kk + (jj + 1);
        const size_t n4 = ii * wyz + g->wrapy * kk + jj;
        F[3 * n1 + 2] += nodalForce;
        F[3 * n2 + 2] += nodalForce;
        F[3 * n3 + 2] += nodalForce;
        F[3 * n4 + 2] += nodalForce;
      }
    }
}

void ref_load(void *p, double *F) {
  RefCtx *c = p;
  CTYPE *Fp = vec_to_padded(c, 0, NULL);
  cantilever_load(&c->gc, Fp);
  vec_from_padded(c, 0, Fp, F);
  free(Fp);
}

/* The design loop of top3dmgcg (stencil_optimization.c:97-189), run through
 * the reference's functions, recording the per-iteration history at full
 * precision. volfrac/rmin arrive as the float values main() passes. */
int ref_run(int nelx, int nely, int nelz, float volfrac_f, float rmin_f, int nl,
            float cgtol, int max_iterations, double *hist_c, double *hist_vol,
            double *hist_change, int *hist_cg, double *hist_relres,
            double *xphys_out, double *u_out) {
  const DTYPE volfrac = volfrac_f, rmin = rmin_f;
  RefCtx *c = ref_create(nelx, nely, nelz, nl);
  struct gridContext *gcp = &c->gc;
  const size_t nelem = nelem_padded(c);
  CTYPE *F;
  STYPE *U;
  allocateZeroPaddedStateField(*gcp, 0, &F);
  allocateZeroPaddedStateField_STYPE(*gcp, 0, &U);
  cantilever_load(gcp, F);
  DTYPE *dc = calloc(nelem, sizeof(DTYPE));
  DTYPE *dv = malloc(sizeof(DTYPE) * nelem);
  DTYPE *x = calloc(nelem, sizeof(DTYPE));
  DTYPE *xPhys = calloc(nelem, sizeof(DTYPE));
  DTYPE *xnew = calloc(nelem, sizeof(DTYPE));
  DTYPE cc = 0.0;
  for (size_t q = 0; q < nelem; q++) dv[q] = 1.0;
  for (int i = 1; i < gcp->nelx + 1; i++)
    for (int k = 1; k < gcp->nelz + 1; k++)
      for (int j = 1; j < gcp->nely + 1; j++) {
        const int idx = i * (gcp->wrapy - 1) * (gcp->wrapz - 1) + k * (gcp->wrapy - 1) + j;
        x[idx] = volfrac;
        xPhys[idx] = volfrac;
      }
  struct SolverDataBuffer sd;
  allocateSolverData(*gcp, nl, &sd);
  initializeCholmod(*gcp, nl - 1, &sd.bottomSolver, sd.coarseMatrices[nl - 1]);
  applyDensityFilterGradient(*gcp, rmin, dv);
  unsigned int loop = 0;
  float change = 1;
  DTYPE vol = 0.0;
  /* REF_VERBOSE=1 prints one progress line per design iteration to stderr,
   * the fields of the reference's verbose line (stencil_optimization.c:173-181) */
  const int verbose = getenv("REF_VERBOSE") != NULL;
  const double t0 = omp_get_wtime();
  while ((change > 1e-2) && (loop < (unsigned)max_iterations)) {
    loop++;
    int cgiter;
    float cgres;
    const int nswp = 4;
    solveStateMG_halo(&c->gpu, xPhys, nswp, nl, cgtol, &sd, &cgiter, &cgres, F, U);
    vol = compute_volume(*gcp, xPhys);
    getComplianceAndSensetivity_halo(&c->gpu.target[0], xPhys, U, &cc, dc);
    applyDensityFilterGradient(*gcp, rmin, dc);
    vol /= (DTYPE)(gcp->nelx * gcp->nely * gcp->nelz);
    DTYPE g = vol - volfrac;
    update_solution(x, xnew, dv, dc, (int)nelem, g);
    change = compute_change(x, xnew, (int)nelem);
    applyDensityFilter(*gcp, rmin, x, xPhys);
    hist_c[loop - 1] = cc;
    hist_vol[loop - 1] = vol;
    hist_change[loop - 1] = change;
    hist_cg[loop - 1] = cgiter;
    hist_relres[loop - 1] = cgres;
    if (verbose) {
      fprintf(stderr, "It.:%4u Obj.:%.17g Vol.:%.6f ch.:%.4f relres: %.4e iters: %4d time: %.3f\n",
              loop, (double)cc, (double)vol, change, cgres, cgiter, omp_get_wtime() - t0);
      fflush(stderr);
    }
  }
  if (xphys_out) el_from_padded(c, xPhys, xphys_out);
  if (u_out) {
    const int nx = gcp->nelx + 1, ny = gcp->nely + 1, nz = gcp->nelz + 1;
    const int wy = gcp->wrapy, wz = gcp->wrapz;
    for (int i = 0; i < nx; i++)
      for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
          for (int d = 0; d < 3; d++)
            u_out[3 * (((size_t)i * nz + k) * ny + j) + d] =
                U[3 * ((size_t)(i + 1) * wy * wz + (size_t)(k + 1) * wy + (j + 1)) + d];
  }
  finishCholmod(*gcp, nl - 1, &sd.bottomSolver, sd.coarseMatrices[nl - 1], 0);
  freeSolverData(&sd, nl);
  free(F); free(U); free(dc); free(dv); free(x); free(xPhys); free(xnew);
  ref_destroy(c);
  return (int)loop;
}

/* ---- timing samples of the reference's own design iteration ----
 * For the CPU baseline: the state of top3dmgcg (stencil_optimization.c:
 * 22-137) on one grid, and the parts of one design iteration timed with
 * omp_get_wtime around the reference's own calls only (no layout
 * conversion inside a timed span):
 *   ref_bench_fixed   solveStateMG_halo with its CG loop cut to one
 *                     iteration (a tolerance every residual meets): the
 *                     per-iteration assembly, diagonals and coarse factor,
 *                     the initial residual and one CG iteration
 *   ref_bench_cg      one more iteration of that CG loop, the body of
 *                     stencil_solvers.c:340-390 on the reference's functions
 *   ref_bench_design  the rest of the iteration, stencil_optimization.c:
 *                     157-178 (volume, compliance and sensitivities, filter
 *                     adjoint, OC update, change, filter)
 * A design iteration with n CG iterations costs fixed + (n - 1) cg + design. */
/* stencil_solvers.c:129-133; the reference's headers do not declare it */
void VcyclePreconditioner(const struct gpuGrid *gpu_gc, const DTYPE *x, const int nl, const int l,
                          MTYPE **const invD, struct CoarseSolverData *bottomSolverData,
                          const struct CSRMatrix *coarseMatrices, CTYPE omega, const int nswp, CTYPE **r,
                          CTYPE **z, CTYPE **d);

typedef struct {
  RefCtx *c;
  struct SolverDataBuffer sd;
  CTYPE *F;
  STYPE *U;
  DTYPE *dc, *dv, *x, *xPhys, *xnew;
  DTYPE volfrac, rmin;
  CTYPE rhoold;
  size_t nelem;
} RefBench;

void *ref_bench_create(int nelx, int nely, int nelz, int nl, float volfrac_f, float rmin_f) {
  RefBench *b = calloc(1, sizeof(RefBench));
  b->c = ref_create(nelx, nely, nelz, nl);
  struct gridContext *g = &b->c->gc;
  b->volfrac = volfrac_f;
  b->rmin = rmin_f;
  b->nelem = nelem_padded(b->c);
  allocateZeroPaddedStateField(*g, 0, &b->F);
  allocateZeroPaddedStateField_STYPE(*g, 0, &b->U);
  cantilever_load(g, b->F);
  b->dc = calloc(b->nelem, sizeof(DTYPE));
  b->dv = malloc(sizeof(DTYPE) * b->nelem);
  b->x = calloc(b->nelem, sizeof(DTYPE));
  b->xPhys = calloc(b->nelem, sizeof(DTYPE));
  b->xnew = calloc(b->nelem, sizeof(DTYPE));
  for (size_t q = 0; q < b->nelem; q++) b->dv[q] = 1.0;
  for (int i = 1; i < g->nelx + 1; i++)
    for (int k = 1; k < g->nelz + 1; k++)
      for (int j = 1; j < g->nely + 1; j++) {
        const size_t idx = (size_t)i * (g->wrapy - 1) * (g->wrapz - 1) + (size_t)k * (g->wrapy - 1) + j;
        b->x[idx] = b->volfrac;
        b->xPhys[idx] = b->volfrac;
      }
  allocateSolverData(*g, nl, &b->sd);
  initializeCholmod(*g, nl - 1, &b->sd.bottomSolver, b->sd.coarseMatrices[nl - 1]);
  applyDensityFilterGradient(*g, b->rmin, b->dv);
  return b;
}

void ref_bench_destroy(void *p) {
  RefBench *b = p;
  const int nl = b->c->nl;
  finishCholmod(b->c->gc, nl - 1, &b->sd.bottomSolver, b->sd.coarseMatrices[nl - 1], 0);
  freeSolverData(&b->sd, nl);
  free(b->F); free(b->U); free(b->dc); free(b->dv); free(b->x); free(b->xPhys); free(b->xnew);
  ref_destroy(b->c);
  free(b);
}

double ref_bench_fixed(void *p) {
  RefBench *b = p;
  int it = 0;
  float rr = 0;
  const double t0 = omp_get_wtime();
  solveStateMG_halo(&b->c->gpu, b->xPhys, 4, b->c->nl, (CTYPE)1e30, &b->sd, &it, &rr, b->F, b->U);
  const double t = omp_get_wtime() - t0;
  /* rho of the iteration just taken, the next iteration's rhoold */
  b->rhoold = innerProduct(b->sd.r, b->sd.z, 3 * (size_t)b->c->gc.wrapx * b->c->gc.wrapy * b->c->gc.wrapz);
  return t;
}

double ref_bench_cg(void *p) {
  RefBench *b = p;
  struct SolverDataBuffer *data = &b->sd;
  const struct gridContext *gc = &b->c->gc;
  const uint_fast32_t ndof = 3 * gc->wrapx * gc->wrapy * gc->wrapz;
  CTYPE *r = data->r, *pp = data->p, *q = data->q, *z = data->z;
  STYPE *u = b->U;
  const MTYPE omega = 0.6;
  const double t0 = omp_get_wtime();
  VcyclePreconditioner(&b->c->gpu, b->xPhys, b->c->nl, 0, data->invD, &data->bottomSolver,
                       data->coarseMatrices, omega, 4, data->rmg, data->zmg, data->dmg);
  const CTYPE rho = innerProduct(r, z, ndof);
  const CTYPE beta = rho / b->rhoold;
#pragma omp parallel for schedule(static)
  for (uint_fast32_t i = 0; i < ndof; i++) pp[i] = beta * pp[i] + z[i];
  applyStateOperator_stencil(&b->c->gpu.target[0], b->xPhys, pp, q);
  const CTYPE dpr = innerProduct(pp, q, ndof);
  const CTYPE alpha = rho / dpr;
  b->rhoold = rho;
#pragma omp parallel for schedule(static)
  for (uint_fast32_t i = 0; i < ndof; i++) u[i] += (STYPE)(alpha * pp[i]);
#pragma omp parallel for schedule(static)
  for (uint_fast32_t i = 0; i < ndof; i++) r[i] -= alpha * q[i];
  volatile CTYPE rn = norm(r, ndof);
  (void)rn;
  return omp_get_wtime() - t0;
}

double ref_bench_design(void *p, double *c_out) {
  RefBench *b = p;
  struct gridContext *g = &b->c->gc;
  DTYPE cc = 0.0;
  const double t0 = omp_get_wtime();
  DTYPE vol = compute_volume(*g, b->xPhys);
  getComplianceAndSensetivity_halo(&b->c->gpu.target[0], b->xPhys, b->U, &cc, b->dc);
  applyDensityFilterGradient(*g, b->rmin, b->dc);
  vol /= (DTYPE)(g->nelx * g->nely * g->nelz);
  const DTYPE gv = vol - b->volfrac;
  update_solution(b->x, b->xnew, b->dv, b->dc, (int)b->nelem, gv);
  volatile float change = compute_change(b->x, b->xnew, (int)b->nelem);
  (void)change;
  applyDensityFilter(*g, b->rmin, b->x, b->xPhys);
  const double t = omp_get_wtime() - t0;
  if (c_out) *c_out = (double)cc;
  return t;
}

/* milliseconds of single calls of the reference's kernels on the bench's
 * state: [0] fine matvec, [1] level-1 matvec, [2] restriction 0->1,
 * [3] prolongation 1->0, [4] inverse diagonal of level 0, [5] compliance and
 * sensitivities, [6] density filter, [7] filter adjoint */
void ref_bench_kernels(void *p, double *ms) {
  RefBench *b = p;
  struct gridContext *g = &b->c->gc;
  const struct gpuNode *node = &b->c->gpu.target[0];
  struct SolverDataBuffer *d = &b->sd;
  double t;
  DTYPE cc = 0;
  t = omp_get_wtime();
  applyStateOperator_stencil(node, b->xPhys, d->p, d->q);
  ms[0] = 1e3 * (omp_get_wtime() - t);
  t = omp_get_wtime();
  applyStateOperatorSubspace_halo(node, 1, b->xPhys, d->zmg[1], d->dmg[1]);
  ms[1] = 1e3 * (omp_get_wtime() - t);
  t = omp_get_wtime();
  projectToCoarserGrid_halo(node, 0, d->r, d->rmg[1]);
  ms[2] = 1e3 * (omp_get_wtime() - t);
  t = omp_get_wtime();
  projectToFinerGrid_halo(node, 0, d->zmg[1], d->dmg[0]);
  ms[3] = 1e3 * (omp_get_wtime() - t);
  t = omp_get_wtime();
  assembleInvertedMatrixDiagonalSubspace_halo(node, b->xPhys, 0, d->invD[0]);
  ms[4] = 1e3 * (omp_get_wtime() - t);
  t = omp_get_wtime();
  getComplianceAndSensetivity_halo(node, b->xPhys, b->U, &cc, b->dc);
  ms[5] = 1e3 * (omp_get_wtime() - t);
  t = omp_get_wtime();
  applyDensityFilter(*g, b->rmin, b->x, b->xnew);
  ms[6] = 1e3 * (omp_get_wtime() - t);
  t = omp_get_wtime();
  applyDensityFilterGradient(*g, b->rmin, b->dc);
  ms[7] = 1e3 * (omp_get_wtime() - t);
}
