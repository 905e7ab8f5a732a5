/*
 * CPU oracle: a plain-C, FP64 restatement of the reference's SIMP design loop
 * and its multigrid-preconditioned CG state solve (topopt/TopOpt-in-OpenMP-GPU).
 *
 * TEST INFRASTRUCTURE ONLY. The parity tests, smoke() and bench.py's CPU
 * baseline leg call it as the checker; the product library never links it.
 * It is pinned against the reference's own C (compiled by build_ref.sh) through
 * the golden fixtures in tests/golden/.
 *
 * Canonical (unpadded) layout used everywhere here:
 *   level l has nelx_l = nelx >> l elements in x (likewise y, z) and
 *   nx_l = nelx_l + 1 nodes; node (i,k,j) sits at n = (i*nz_l + k)*ny_l + j
 *   and owns DOFs 3n+0..2 (x,y,z); fine element (i,k,j) sits at
 *   (i*nelz + k)*nely + j. This is the reference's ordering
 *   (stencil_utility.h:19-52) with the halo and y-padding removed.
 */
#ifndef TOPOPT_ORACLE_H
#define TOPOPT_ORACLE_H

#include <stddef.h>

#define OR_MAXL 8

typedef struct {
  int nelx, nely, nelz, nl;
  double E0, Emin, nu;
  double *ke[OR_MAXL];       /* 576*ncell^3 doubles per level */
  long *fixed[OR_MAXL];      /* canonical fixed DOF indices */
  int nfixed[OR_MAXL];
  unsigned char *isfixed[OR_MAXL];
} OrGrid;

typedef struct {
  int loops;
  double c[1024], vol[1024], change[1024], relres[1024];
  int cgiters[1024];
  double seconds[1024]; /* wall time of each design iteration */
} OrHistory;

#ifdef __cplusplus
extern "C" {
#endif

OrGrid *or_create(int nelx, int nely, int nelz, int nl);
void or_destroy(OrGrid *g);

size_t or_nnodes(const OrGrid *g, int l);
size_t or_nelem(const OrGrid *g);

void or_ke(double nu, int l, double *KE);
int or_fixed_dofs(const OrGrid *g, int l, long *out);
void or_load(const OrGrid *g, double *F);

void or_apply(const OrGrid *g, int l, const double *x, const double *in, double *out);
void or_apply_masked(const OrGrid *g, int l, const double *x, const double *in, double *out);
void or_inv_diag(const OrGrid *g, int l, const double *x, double *invD);
void or_restrict(const OrGrid *g, int l, const double *fine, double *coarse);
void or_prolong(const OrGrid *g, int l, const double *coarse, double *fine);
void or_smooth(const OrGrid *g, int l, const double *x, int nswp, double omega,
               const double *invD, const double *b, double *u, double *tmp);

/* coarsest-level banded Cholesky of the assembled, BC-modified operator */
typedef struct {
  int l;
  size_t n, bw;
  double *band;
} OrCoarse;
int or_coarse_factor(const OrGrid *g, int l, const double *x, OrCoarse *cs);
void or_coarse_solve(const OrCoarse *cs, const double *rhs, double *sol);
void or_coarse_free(OrCoarse *cs);
int or_coarse_direct(const OrGrid *g, int l, const double *x, const double *rhs, double *sol);

int or_solve(const OrGrid *g, const double *x, const double *b, double *u,
             int nswp, double tol, int *iters, double *relres);

double or_compliance(const OrGrid *g, const double *x, const double *u, double *dc);
void or_filter(const OrGrid *g, double rmin, const double *x, double *out);
void or_filter_T(const OrGrid *g, double rmin, double *v);
void or_oc_update(const OrGrid *g, const double *x, const double *dv,
                  const double *dc, double gvol, double *xnew);
double or_volume(const OrGrid *g, const double *xPhys);
float or_change(const OrGrid *g, double *x, const double *xnew);

int or_run(int nelx, int nely, int nelz, double volfrac, double rmin, int nl,
           double cgtol, int max_iterations, OrHistory *h, double *xPhys_out,
           double *u_out);

#ifdef __cplusplus
}
#endif
#endif
