/*
 * CHOLMOD-subset stand-in used ONLY to compile the reference's own C as a CPU
 * oracle (test infrastructure, never shipped in the product library).
 *
 * The reference calls SuiteSparse CHOLMOD 5.1.2 for its coarsest-level solve
 * (stencil_assembly.c:366-503). SuiteSparse is not in the image, so this
 * header declares the handful of types and calls that file uses, and
 * cholmod_shim.c implements them with a dense banded Cholesky factorisation
 * (natural ordering). Only the fields the reference touches exist here.
 * Any exact direct factorisation gives the same solution up to rounding.
 */
#ifndef ORACLE_CHOLMOD_SHIM_H
#define ORACLE_CHOLMOD_SHIM_H

#include <stddef.h>

#define CHOLMOD_REAL 1
#define CHOLMOD_A 0

typedef struct cholmod_common_struct {
  int nmethods;
  int status;
} cholmod_common;

typedef struct cholmod_sparse_struct {
  size_t nrow, ncol, nzmax;
  void *p; /* int column pointers, length ncol+1 */
  void *i; /* int row indices */
  void *x; /* double values */
  int stype;
} cholmod_sparse;

typedef struct cholmod_dense_struct {
  size_t nrow, ncol, d;
  void *x;
} cholmod_dense;

typedef struct cholmod_factor_struct {
  size_t n;
  size_t bw;   /* half bandwidth */
  double *band; /* lower band, band[j*(bw+1) + (i-j)] = L(i,j), i>=j */
} cholmod_factor;

int cholmod_start(cholmod_common *c);
int cholmod_finish(cholmod_common *c);
int cholmod_print_common(const char *name, cholmod_common *c);
cholmod_sparse *cholmod_allocate_sparse(size_t nrow, size_t ncol, size_t nzmax,
                                        int sorted, int packed, int stype,
                                        int xtype, cholmod_common *c);
int cholmod_free_sparse(cholmod_sparse **A, cholmod_common *c);
cholmod_dense *cholmod_allocate_dense(size_t nrow, size_t ncol, size_t d,
                                      int xtype, cholmod_common *c);
int cholmod_free_dense(cholmod_dense **X, cholmod_common *c);
cholmod_factor *cholmod_analyze(cholmod_sparse *A, cholmod_common *c);
int cholmod_factorize(cholmod_sparse *A, cholmod_factor *L, cholmod_common *c);
int cholmod_free_factor(cholmod_factor **L, cholmod_common *c);
int cholmod_solve2(int sys, cholmod_factor *L, cholmod_dense *B, void *Bset,
                   cholmod_dense **X_Handle, void *Xset_Handle,
                   cholmod_dense **Y_Handle, cholmod_dense **E_Handle,
                   cholmod_common *c);

#endif
