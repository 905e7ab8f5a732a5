/*
 * Minimal CBLAS stand-in used ONLY to compile the reference's own C as a CPU
 * oracle (test infrastructure, never shipped in the product library).
 *
 * The reference links OpenBLAS 0.2.20 for two call shapes in its element
 * stiffness set-up (local_matrix.c:242-246, :304-310): row-major dgemm with
 * A not transposed or transposed, B never transposed. This header declares
 * just that entry point; cblas_shim.c implements it as a plain triple loop.
 * OpenBLAS itself is not in the image; its blocked summation order differs
 * from the triple loop only by rounding (about 1e-16 relative on KE).
 */
#ifndef ORACLE_CBLAS_SHIM_H
#define ORACLE_CBLAS_SHIM_H

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };

void cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE transA,
                 enum CBLAS_TRANSPOSE transB, int M, int N, int K,
                 double alpha, const double *A, int lda, const double *B,
                 int ldb, double beta, double *C, int ldc);

#endif
