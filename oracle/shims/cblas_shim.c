/*
 * Row-major dgemm by a plain triple loop: C = alpha*op(A)*B + beta*C.
 * Test infrastructure for the CPU oracle only (see cblas.h).
 * The summation order (k innermost, ascending) is the one the oracle's own
 * element-matrix restatement uses, so both give identical KE bits.
 */
#include "cblas.h"

void cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE transA,
                 enum CBLAS_TRANSPOSE transB, int M, int N, int K,
                 double alpha, const double *A, int lda, const double *B,
                 int ldb, double beta, double *C, int ldc) {
  (void)order; /* only row-major is used by the reference */
  (void)transB;
  for (int m = 0; m < M; m++)
    for (int n = 0; n < N; n++) {
      double acc = 0.0;
      for (int k = 0; k < K; k++) {
        const double a = (transA == CblasNoTrans) ? A[m * lda + k] : A[k * lda + m];
        acc += a * B[k * ldb + n];
      }
      C[m * ldc + n] = alpha * acc + (beta == 0.0 ? 0.0 : beta * C[m * ldc + n]);
    }
}
