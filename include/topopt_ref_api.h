/*
 * Drop-in entry points with the reference's own names, signatures and data
 * layouts (topopt/TopOpt-in-OpenMP-GPU), backed by libtopopt_gb300.
 *
 * A caller written against the reference's headers links
 * libtopopt_ref32.so (CTYPE/DTYPE float, the reference as shipped) or
 * libtopopt_ref64.so (CTYPE/DTYPE double, the FP64 oracle form) instead of
 * the reference's objects. Arrays are HOST arrays in the reference's padded
 * layout: halo of one node/element on every face, y padded so that
 * (nely+1+pad) is a multiple of STENCIL_SIZE_Y (gpu_definitions.c:67-92);
 * node (i,j,k) at 3*(i*wrapy*wrapz + k*wrapy + j), element at
 * i*(wrapy-1)*(wrapz-1) + k*(wrapy-1) + j, 1-based inside the halo.
 * Each call copies its inputs to the GPU, runs the CUDA kernels, and copies
 * its outputs back; the GPU state per grid is cached between calls. All
 * arithmetic is FP64 on the GPU regardless of the flavour.
 *
 * The structs below reproduce the reference's field order so that a caller
 * compiled against either header sees the same layout (definitions.h:31-53,
 * gpu_definitions.h:7-37, stencil_assembly.h:8-27). CoarseSolverData keeps the
 * reference's seven pointer slots; the first holds this library's handle.
 */
#ifndef TOPOPT_REF_API_H
#define TOPOPT_REF_API_H

#include <stdint.h>

#ifndef TP_REF_FLOAT
#define TP_REF_FLOAT 1
#endif

#define STENCIL_SIZE_Y 128
#define STENCIL_SIZE_X 1
#define STENCIL_SIZE_Z 1
#define number_of_matrix_free_levels 2

typedef double MTYPE;
typedef double STYPE;
#if TP_REF_FLOAT
typedef float CTYPE;
typedef float DTYPE;
#else
typedef double CTYPE;
typedef double DTYPE;
#endif

#ifdef __cplusplus
extern "C" {
#endif

struct FixedDofs {
  uint_fast32_t n;
  uint_fast32_t *idx;
};

struct gridContext {
  double E0;
  double Emin;
  double nu;
  double elementSizeX;
  double elementSizeY;
  double elementSizeZ;
  uint_fast32_t nelx;
  uint_fast32_t nely;
  uint_fast32_t nelz;
  uint_fast32_t wrapx;
  uint_fast32_t wrapy;
  uint_fast32_t wrapz;
  double penal;
  MTYPE **precomputedKE;
  struct FixedDofs *fixedDofs;
};

struct CSRMatrix {
  uint64_t nnz;
  int32_t nrows;
  int *rowOffsets;
  int *colIndex;
  MTYPE *vals;
};

struct CoarseSolverData {
  void *handle; /* the reference's cholmod_common* slot */
  void *reserved[6];
};

struct SolverDataBuffer {
  CTYPE *r;
  CTYPE *p;
  CTYPE *q;
  CTYPE *z;
  MTYPE **invD;
  CTYPE **dmg;
  CTYPE **rmg;
  CTYPE **zmg;
  struct CSRMatrix *coarseMatrices;
  struct CoarseSolverData bottomSolver;
};

struct gpuNode {
  int id;
  struct gpuNode *prev;
  struct gpuNode *next;
  struct gridContext *gc;
  int offset_x;
  int x_global;
};

struct gpuGrid {
  int num_targets;
  struct gpuNode *target;
};

/* stencil_optimization.h:5-21 */
void top3dmgcg(const uint_fast32_t nelx, const uint_fast32_t nely, const uint_fast32_t nelz,
               const DTYPE volfrac, const DTYPE rmin, const uint_fast32_t nl, const float cgtol,
               const uint_fast32_t cgmax, const int verbose, const int write_result,
               const int max_iterations);
void applyDensityFilter(const struct gridContext gc, const DTYPE rmin, const DTYPE *rho, DTYPE *out);
void applyDensityFilterGradient(const struct gridContext gc, const DTYPE rmin, DTYPE *v);
void writeDensityVtkFile(const int nelx, const int nely, const int nelz, const DTYPE *densityArray,
                         const char *filename);
void writeDensityVtkFileWithHalo(const int nelx, const int nely, const int nelz,
                                 const DTYPE *densityArray, const char *filename);

/* stencil_methods.h:6-28 */
void applyStateOperator_stencil(const struct gpuNode *gpu_node, const DTYPE *x, const CTYPE *in, CTYPE *out);
void applyStateOperatorSubspace_halo(const struct gpuNode *gpu_node, const int l, const DTYPE *x, CTYPE *in,
                                     CTYPE *out);
void getComplianceAndSensetivity_halo(const struct gpuNode *gpu_node, const DTYPE *x, STYPE *u, DTYPE *c,
                                      DTYPE *dcdx);
void projectToFinerGrid_halo(const struct gpuNode *gpu_node, const int l, const CTYPE *ucoarse, CTYPE *ufine);
void projectToCoarserGrid_halo(const struct gpuNode *gpu_node, const int l, const CTYPE *ufine, CTYPE *ucoarse);
void assembleInvertedMatrixDiagonalSubspace_halo(const struct gpuNode *gpu_node, const DTYPE *x, const int l,
                                                 MTYPE *diag);

/* stencil_solvers.h:8-32 */
void smoothDampedJacobi_halo(const struct gpuNode *gpu_node, const DTYPE *x, const uint_fast32_t nswp,
                             const CTYPE omega, const MTYPE *invD, CTYPE *u, const CTYPE *b, CTYPE *tmp);
void smoothDampedJacobiSubspaceMatrix_halo(const struct gridContext *gc, const struct CSRMatrix M, const int l,
                                           const uint_fast32_t nswp, const CTYPE omega, const MTYPE *invD,
                                           CTYPE *u, const CTYPE *b, CTYPE *tmp);
void smoothDampedJacobiSubspace_halo(const struct gpuNode *gpu_node, const DTYPE *x, const int l,
                                     const uint_fast32_t nswp, const CTYPE omega, const MTYPE *invD, CTYPE *u,
                                     const CTYPE *b, CTYPE *tmp);
void solveStateMG_halo(const struct gpuGrid *gpu_gc, DTYPE *x, const int nswp, const int nl, const CTYPE tol,
                       struct SolverDataBuffer *data, int *finalIter, float *finalRes, CTYPE *b, STYPE *u);
void allocateSolverData(const struct gridContext gc, const int nl, struct SolverDataBuffer *data);
void freeSolverData(struct SolverDataBuffer *data, const int nl);

/* stencil_assembly.h:29-55 (CSR of the assembled levels, host arrays) */
void allocateSubspaceMatrix(const struct gridContext gc, const int l, struct CSRMatrix *M);
void freeSubspaceMatrix(struct CSRMatrix *M);
void assembleSubspaceMatrix(const struct gridContext gc, const int l, const DTYPE *x, struct CSRMatrix M,
                            MTYPE *tmp);
void applyStateOperatorSubspaceMatrix(const struct gridContext gc, const int l, const struct CSRMatrix M,
                                      const CTYPE *in, CTYPE *out);
void initializeCholmod(const struct gridContext gc, const int l, struct CoarseSolverData *solverData,
                       const struct CSRMatrix M);
void finishCholmod(const struct gridContext gc, const int l, struct CoarseSolverData *solverData,
                   const struct CSRMatrix M, const int verbose);
void factorizeSubspaceMatrix(const struct gridContext gc, const int l, struct CoarseSolverData solverData,
                             const struct CSRMatrix M);
void solveSubspaceMatrix(const struct gridContext gc, const int l, struct CoarseSolverData solverData,
                         const CTYPE *in, CTYPE *out);

/* gpu_definitions.h:39-86 */
void gridContextToGPUGrid(struct gridContext *gc, struct gpuGrid *gpu_gc, const int nl, const int verbose);
void freeGPUGrid(struct gpuGrid *gpu_gc, const int nl);
void computePadding(const struct gridContext *gc, const int l, int *ncell, int *wrapx, int *wrapy, int *wrapz,
                    uint_fast32_t *ndof);
DTYPE compute_volume(const struct gridContext gc, DTYPE *xPhys);
float compute_change(DTYPE *x, DTYPE *xnew, const int nelem);
void update_solution(const DTYPE *x, DTYPE *xnew, const DTYPE *dv, const DTYPE *dc, const int nelem,
                     const DTYPE g);
void enter_data(const struct gridContext gridContext, const struct SolverDataBuffer solverData,
                const struct gpuGrid gpu_gc, const DTYPE *xPhys, const DTYPE *x, const DTYPE *xnew, const STYPE *U,
                const CTYPE *F, const DTYPE *dc, const int nelem, const int nl);

/* stencil_grid_utility.h:5-17 */
void setFixedDof_halo(struct gridContext *gc, const int l);
void setupGC(struct gridContext *gc, const int nl, const int nelx, const int nely, const int nelz);
void freeGC(struct gridContext *gc, const int nl);
void allocateZeroPaddedStateField(const struct gridContext gc, const int l, CTYPE **v);
void allocateZeroPaddedStateField_MTYPE(const struct gridContext gc, const int l, MTYPE **v);
void allocateZeroPaddedStateField_STYPE(const struct gridContext gc, const int l, STYPE **v);

/* local_matrix.h:7-21 */
void getC(MTYPE C[6][6], const MTYPE nu);
void getB(MTYPE B[6][24], MTYPE *jdet, const MTYPE iso[3], const MTYPE xe[24]);
void getKEsubspace(MTYPE *KEarray, const MTYPE nu, const int l);

/* No counterpart in the reference: bytes the entry points above have copied
 * host -> device (*h2d) and device -> host (*d2h) since the library was
 * loaded or last reset (reset != 0 clears the counts after reading them).
 * Every GPU-backed entry point copies its host arrays in and out at each
 * call; TOPOPT_PRECISION=mixed in the environment selects the mixed form
 * (FP32 V-cycle, FP64 CG) for all of them, the default being FP64. */
void topopt_ref_transfer_bytes(long *h2d, long *d2h, int reset);

#ifdef __cplusplus
}
#endif
#endif
