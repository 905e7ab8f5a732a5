/*
 * Dense banded Cholesky standing in for the CHOLMOD calls of the reference's
 * coarsest-level solver (stencil_assembly.c:366-503). Test infrastructure for
 * the CPU oracle only. The matrix arrives as CSC with stype=1 ("use the upper
 * triangle", stencil_assembly.c:373-381); the factor is stored as the lower
 * band of L, column by column.
 */
#include "cholmod.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int cholmod_start(cholmod_common *c) {
  memset(c, 0, sizeof(*c));
  return 1;
}
int cholmod_finish(cholmod_common *c) {
  (void)c;
  return 1;
}
int cholmod_print_common(const char *name, cholmod_common *c) {
  printf("%s: banded Cholesky stand-in, status %d\n", name, c->status);
  return 1;
}

cholmod_sparse *cholmod_allocate_sparse(size_t nrow, size_t ncol, size_t nzmax,
                                        int sorted, int packed, int stype,
                                        int xtype, cholmod_common *c) {
  (void)sorted; (void)packed; (void)xtype; (void)c;
  cholmod_sparse *A = calloc(1, sizeof(cholmod_sparse));
  A->nrow = nrow;
  A->ncol = ncol;
  A->nzmax = nzmax;
  A->stype = stype;
  A->p = calloc(ncol + 1, sizeof(int));
  A->i = calloc(nzmax, sizeof(int));
  A->x = calloc(nzmax, sizeof(double));
  return A;
}

int cholmod_free_sparse(cholmod_sparse **A, cholmod_common *c) {
  (void)c;
  if (A && *A) {
    free((*A)->p);
    free((*A)->i);
    free((*A)->x);
    free(*A);
    *A = NULL;
  }
  return 1;
}

cholmod_dense *cholmod_allocate_dense(size_t nrow, size_t ncol, size_t d,
                                      int xtype, cholmod_common *c) {
  (void)xtype; (void)c;
  cholmod_dense *X = calloc(1, sizeof(cholmod_dense));
  X->nrow = nrow;
  X->ncol = ncol;
  X->d = d;
  X->x = calloc(d * ncol, sizeof(double));
  return X;
}

int cholmod_free_dense(cholmod_dense **X, cholmod_common *c) {
  (void)c;
  if (X && *X) {
    free((*X)->x);
    free(*X);
    *X = NULL;
  }
  return 1;
}

/* The "analysis" is the half bandwidth of the upper-triangle pattern. */
cholmod_factor *cholmod_analyze(cholmod_sparse *A, cholmod_common *c) {
  (void)c;
  const int *p = (const int *)A->p;
  const int *ri = (const int *)A->i;
  size_t bw = 0;
  for (size_t j = 0; j < A->ncol; j++)
    for (int q = p[j]; q < p[j + 1]; q++) {
      const long i = ri[q];
      if (i <= (long)j && (size_t)((long)j - i) > bw) bw = (size_t)((long)j - i);
    }
  cholmod_factor *L = calloc(1, sizeof(cholmod_factor));
  L->n = A->ncol;
  L->bw = bw;
  L->band = calloc(L->n * (bw + 1), sizeof(double));
  return L;
}

int cholmod_factorize(cholmod_sparse *A, cholmod_factor *L, cholmod_common *c) {
  const size_t n = L->n, w = L->bw + 1;
  double *B = L->band;
  memset(B, 0, n * w * sizeof(double));
  const int *p = (const int *)A->p;
  const int *ri = (const int *)A->i;
  const double *ax = (const double *)A->x;
  /* upper entry (i,j), i<=j, becomes lower entry (j,i) of the band */
  for (size_t j = 0; j < A->ncol; j++)
    for (int q = p[j]; q < p[j + 1]; q++) {
      const size_t i = (size_t)ri[q];
      if (i <= j) B[i * w + (j - i)] = ax[q];
    }
  c->status = 0;
  /* right-looking band factorisation */
  for (size_t j = 0; j < n; j++) {
    double d = B[j * w];
    if (!(d > 0.0)) {
      c->status = 1; /* not positive definite */
      d = 1.0;
    }
    d = sqrt(d);
    B[j * w] = d;
    const size_t last = (j + L->bw < n - 1) ? j + L->bw : n - 1;
    for (size_t i = j + 1; i <= last; i++) B[j * w + (i - j)] /= d;
#pragma omp parallel for schedule(static)
    for (long cc = (long)j + 1; cc <= (long)last; cc++) {
      const double ljc = B[j * w + ((size_t)cc - j)];
      for (size_t r = (size_t)cc; r <= last; r++)
        B[(size_t)cc * w + (r - (size_t)cc)] -= B[j * w + (r - j)] * ljc;
    }
  }
  return c->status == 0;
}

int cholmod_free_factor(cholmod_factor **L, cholmod_common *c) {
  (void)c;
  if (L && *L) {
    free((*L)->band);
    free(*L);
    *L = NULL;
  }
  return 1;
}

int cholmod_solve2(int sys, cholmod_factor *L, cholmod_dense *B, void *Bset,
                   cholmod_dense **X_Handle, void *Xset_Handle,
                   cholmod_dense **Y_Handle, cholmod_dense **E_Handle,
                   cholmod_common *c) {
  (void)sys; (void)Bset; (void)Xset_Handle; (void)Y_Handle; (void)E_Handle;
  const size_t n = L->n, w = L->bw + 1;
  if (*X_Handle == NULL) *X_Handle = cholmod_allocate_dense(n, 1, n, CHOLMOD_REAL, c);
  double *x = (double *)(*X_Handle)->x;
  const double *b = (const double *)B->x;
  const double *Lb = L->band;
  memcpy(x, b, n * sizeof(double));
  /* L y = b */
  for (size_t j = 0; j < n; j++) {
    x[j] /= Lb[j * w];
    const size_t last = (j + L->bw < n - 1) ? j + L->bw : n - 1;
    for (size_t i = j + 1; i <= last; i++) x[i] -= Lb[j * w + (i - j)] * x[j];
  }
  /* L^T x = y */
  for (size_t jj = n; jj-- > 0;) {
    const size_t last = (jj + L->bw < n - 1) ? jj + L->bw : n - 1;
    double s = x[jj];
    for (size_t i = jj + 1; i <= last; i++) s -= Lb[jj * w + (i - jj)] * x[i];
    x[jj] = s / Lb[jj * w];
  }
  return 1;
}
