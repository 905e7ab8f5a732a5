/*
 * libtopopt_gb300 -- GB300-native SIMP compliance minimisation with a
 * matrix-free, multigrid-preconditioned CG state solve.
 *
 * Handle API (this header). The reference-signature drop-in entry points
 * (top3dmgcg, applyStateOperator_stencil, ...) are declared in
 * topopt_ref_api.h and are thin wrappers over this API.
 *
 * Conventions
 *  - Every entry point returns tp_status (0 = TP_OK) except the plain getters.
 *  - Arrays are double unless the name ends in _f32, and use the canonical
 *    unpadded layout: level l has (nelx>>l)+1 x (nely>>l)+1 x (nelz>>l)+1
 *    nodes, node (i,k,j) at n = (i*nz + k)*ny + j with DOFs 3n+0..2 (x,y,z);
 *    fine element (i,k,j) at (i*nelz + k)*nely + j. This is the reference's
 *    ordering (stencil_utility.h:19-52) without its halo and y-padding.
 *  - "_dev" arguments are device pointers on the context's device; other
 *    array arguments are host pointers. Work is stream-ordered on the
 *    context's stream; tp_sync() waits for it.
 *  - A context is used by one host thread at a time.
 */
#ifndef TOPOPT_GB300_H
#define TOPOPT_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TP_OK = 0,
  TP_ERR_ARG = 1,           /* invalid argument or size */
  TP_ERR_CUDA = 2,          /* a CUDA call or launch failed */
  TP_ERR_ALLOC = 3,         /* device or host allocation failed */
  TP_ERR_NOT_SPD = 4,       /* coarse Cholesky met a non-positive pivot */
  TP_ERR_NOT_CONVERGED = 5, /* CG reached cgmax without relres < cgtol */
  TP_ERR_NONFINITE = 6,     /* NaN/Inf in a residual or reduction */
  TP_ERR_TIMEOUT = 7,       /* a bounded device wait gave up */
  TP_ERR_STATE = 8          /* call out of order (e.g. operators not assembled) */
} tp_status;

typedef enum {
  TP_FP64 = 0, /* everything FP64: the drop-in form of the reference's path */
  TP_MIXED = 1 /* FP32 V-cycle and smoother; FP64 CG vectors, dots, updates and coarse sweeps;
                  double-single CG matvec and coarse factor (tp_set_fine_arith,
                  tp_set_coarse_arith switch those to FP64) */
} tp_precision;

typedef struct tp_ctx tp_ctx;

typedef struct {
  int nelx, nely, nelz; /* fine elements; each divisible by 2^(nl-1) */
  int nl;               /* multigrid levels, >= 3 (stencil_optimization.c:13) */
  double volfrac;       /* volume fraction (the reference's main() holds it as float) */
  double rmin;          /* density-filter radius in elements */
  double cgtol;         /* relative residual tolerance (top3d.c:82) */
  int cgmax;            /* CG iteration cap; the reference hard-codes 1000 (stencil_solvers.c:334) */
  int nswp;             /* Jacobi sweeps per smoothing (stencil_optimization.c:154) */
  double omega;         /* Jacobi damping (stencil_solvers.c:332) */
  int precision;        /* tp_precision */
  int nrhs;             /* load cases solved together (1 = the reference's single load) */
  int device;           /* CUDA device ordinal */
} tp_params;

typedef struct {
  int loop;        /* 1-based design iteration */
  double c;        /* compliance (summed over load cases) */
  double vol;      /* volume fraction of xPhys */
  double change;   /* max |x - xnew|, rounded through float as the reference does */
  int cgiters;     /* last CG iteration index, as the reference reports it */
  double relres;   /* final relative residual, rounded through float */
  double ms;       /* device milliseconds of this design iteration */
} tp_iter_info;

typedef enum {
  TP_FIELD_X = 0,     /* design variables x (fine elements) */
  TP_FIELD_XPHYS = 1, /* filtered densities xPhys */
  TP_FIELD_XNEW = 2,
  TP_FIELD_DC = 3,    /* compliance sensitivity (after the filter adjoint in the loop) */
  TP_FIELD_DV = 4,    /* volume sensitivity, filter adjoint of ones */
  TP_FIELD_F = 5,     /* load vectors, nrhs * ndof(0) */
  TP_FIELD_U = 6      /* displacements, nrhs * ndof(0) */
} tp_field;

/* Reference defaults: 12x6x6 coarse elements at nl=4 (top3d.c:16-24),
 * volfrac (float)0.2, rmin 1.5, cgtol (float)1e-5, cgmax 1000, nswp 4,
 * omega 0.6, FP64, one load case, device 0. */
void tp_default_params(tp_params* p);

tp_status tp_create(const tp_params* p, tp_ctx** out);
void tp_destroy(tp_ctx* c);
const char* tp_status_string(tp_status s);
const char* tp_error_message(const tp_ctx* c);
tp_status tp_sync(tp_ctx* c);

long tp_ndof(const tp_ctx* c, int level);   /* 3 * nodes of level */
long tp_nelem(const tp_ctx* c);             /* fine elements */
long tp_device_bytes(const tp_ctx* c);      /* device memory the context holds */
double* tp_field_ptr(tp_ctx* c, tp_field f); /* device pointer to a context field */
/* The caller has written field f through tp_field_ptr (with its own copies,
 * finished before this call): what tp_upload would do after its copy. For
 * TP_FIELD_XPHYS the assembled operators are marked stale. */
tp_status tp_field_written(tp_ctx* c, tp_field f);

/* Host <-> device copies of context fields (count = elements of the field). */
tp_status tp_upload(tp_ctx* c, tp_field f, const double* host, long count);
tp_status tp_download(tp_ctx* c, tp_field f, double* host, long count);

/* Set-up data, for checks: element stiffness tables of level l
 * (576 * 8^l doubles, local_matrix.c:251-319) and the fixed DOFs of level l
 * (stencil_grid_utility.c:7-65). *count receives the number written. */
tp_status tp_element_matrices(const tp_ctx* c, int level, double* out_host);
/* The same tables without a context (host only): nu = Poisson's ratio. */
tp_status tp_element_matrix_tables(int level, double nu, double* out_host);
/* The reference's cantilever load for a fine grid, host only
 * (stencil_optimization.c:37-95): 3*(nelx+1)*(nely+1)*(nelz+1) doubles. */
tp_status tp_reference_load(int nelx, int nely, int nelz, double* F_host);
tp_status tp_fixed_dofs(const tp_ctx* c, int level, long* out_host, long* count);

/* Builds every level's operator for the current xPhys: E(xPhys), inverse
 * Jacobi diagonals, assembled stencils of levels >= 1, and the band Cholesky
 * factor of the coarsest level on FP64 storage (stencil_solvers.c:283-302). */
tp_status tp_assemble(tp_ctx* c);
/* The same assembly enqueued on the context's stream without waiting, so that
 * host work (copies on streams of the caller's own) overlaps it; the next
 * tp_assemble completes it and reports its status. A change of xPhys or of
 * the solver's set-up in between discards it (tp_assemble then assembles
 * again). */
tp_status tp_assemble_async(tp_ctx* c);

/* Operators on device vectors of level `level`.
 * level 0: the matrix-free hex8 stencil (stencil_methods.c:7-428);
 * level 1: the subspace operator (stencil_methods.c:436-519);
 * level >= 2: the assembled operator with fixed rows and columns zeroed
 * (stencil_assembly.c:126-364). Fixed rows return the input. */
tp_status tp_apply(tp_ctx* c, int level, const double* in_dev, double* out_dev);
tp_status tp_apply_f32(tp_ctx* c, int level, const float* in_dev, float* out_dev);
tp_status tp_inv_diag(tp_ctx* c, int level, double* out_dev);            /* stencil_methods.c:693-773 */
tp_status tp_restrict(tp_ctx* c, int level, const double* fine_dev, double* coarse_dev);  /* :595-688 */
tp_status tp_prolong(tp_ctx* c, int level, const double* coarse_dev, double* fine_dev);   /* :521-590 */
tp_status tp_smooth(tp_ctx* c, int level, int nswp, double omega, const double* b_dev,
                    double* u_dev);                                       /* stencil_solvers.c:11-122 */
tp_status tp_coarse_solve(tp_ctx* c, const double* rhs_dev, double* x_dev); /* stencil_assembly.c:439-503 */
tp_status tp_vcycle(tp_ctx* c, const double* r_dev, double* z_dev);       /* stencil_solvers.c:129-252 */

/* PCG solve of K(xPhys) U = F, warm-started from U (stencil_solvers.c:259-397).
 * Assembles the operators first. */
tp_status tp_solve(tp_ctx* c, int* iters, double* relres);
/* The same solve for an arbitrary right-hand side (an adjoint solve). */
tp_status tp_solve_rhs(tp_ctx* c, const double* rhs_dev, double* sol_dev, int* iters, double* relres);

/* Compliance c = sum E(xPhys_e) u_e^T KE u_e and dc/dxPhys
 * (stencil_methods.c:808-862) for the context's U, into TP_FIELD_DC. */
tp_status tp_compliance(tp_ctx* c, double* c_out);
/* General adjoint sensitivity: out_e = -3 (E0-Emin) xPhys_e^2 w_e^T KE u_e. */
tp_status tp_element_sensitivity(tp_ctx* c, const double* u_dev, const double* w_dev, double* out_dev);

/* Density filter xPhys = (H x)/Hs and its adjoint v <- H (v/Hs)
 * (stencil_optimization.c:228-395). */
tp_status tp_filter(tp_ctx* c, const double* in_dev, double* out_dev);
tp_status tp_filter_T(tp_ctx* c, double* v_dev);
tp_status tp_volume(tp_ctx* c, double* vol);   /* sum of xPhys / nelem (gpu_definitions.c:94-108) */
/* OC bisection update from x, dc, dv with constraint value g
 * (gpu_definitions.c:127-157), then change = max|x - xnew| and x <- xnew
 * (:110-125). */
tp_status tp_oc_update(tp_ctx* c, double g, double* change);

/* One design iteration of the loop at stencil_optimization.c:148-189, and the
 * whole loop from x = xPhys = volfrac (:97-189). The loop stops when
 * change <= 1e-2 or after max_iterations. hist may be NULL. */
tp_status tp_init_design(tp_ctx* c);
tp_status tp_design_iteration(tp_ctx* c, tp_iter_info* info);
tp_status tp_run(tp_ctx* c, int max_iterations, tp_iter_info* hist, int* loops);

/* ---- entry points behind the reference-signature layer (topopt_ref_api.h) ---- */
/* Changes the filter radius (recomputes the filter row sums). */
tp_status tp_set_rmin(tp_ctx* c, double rmin);
/* Changes the CG tolerance and cap and the smoother's sweeps and damping. */
tp_status tp_set_cg(tp_ctx* c, double cgtol, int cgmax, int nswp, double omega);
/* Level-0 kernel selection (no counterpart in the reference): variant 0 =
 * the element-centric, sum-factorised kernel wherever its launch plan
 * applies (nely <= 256, 16-byte aligned vectors), else the node-centric
 * stencil; variant 1 = the node-centric stencil everywhere; variant 2 =
 * variant 0 with the FP32 product, sweep and residual on the packed kernel
 * (two z groups per thread in f32x2 arithmetic). Variants 0 and 2 reset the
 * FP32 launch plans to that kernel's defaults (tp_autotune re-tunes them). */
tp_status tp_set_fine_variant(tp_ctx* c, int variant);
/* Arithmetic of the element-centric level-0 kernel on double vectors (no
 * counterpart in the reference): 0 = FP64; 1 = double-single, pairs of FP32
 * numbers with about 48 significant bits, each addition's error bounded by
 * ~2^-45 (|a| + |b|) instead of 2^-53 (|a| + |b|). The vectors stay FP64 in
 * memory. The default is 1 for TP_MIXED (its CG matvec and residual, and the
 * element energies of the compliance pass) and 0 for TP_FP64. Double-single has FP32's exponent range: vector entries of
 * magnitude below 2^-126 (1.2e-38) count as zero, above 2^128 as infinity
 * (which the solve then reports as TP_ERR_NONFINITE); select 0 for
 * right-hand sides scaled outside that range. */
tp_status tp_set_fine_arith(tp_ctx* c, int arith);
/* Coarsest-level direct solver selection (no counterpart in the reference,
 * whose coarse factor and solve are CHOLMOD's, stencil_assembly.c:435-484):
 * variant 0 = the band Cholesky as one cooperative launch (a chain CTA
 * factoring the diagonal tiles, the other CTAs solving panel tiles and
 * updating the trailing band, handing work over through flags) and both
 * triangular sweeps as one cooperative launch with grid barriers between the
 * block steps, wherever their launch plans apply; variant 1 = launches per
 * 32-column factor step and two launches per solve block step. The factor is
 * redone at the next solve. Each variant sums in a fixed order, so repeated
 * runs agree bit for bit; the two variants agree to rounding. */
tp_status tp_set_coarse_solve_variant(tp_ctx* c, int variant);
/* Arithmetic of the coarsest-level band Cholesky (its single-launch factor
 * and the diagonal-block inverses; no counterpart in the reference): 0 =
 * FP64; 1 = double-single (pairs of FP32 numbers, about 48 significant bits)
 * on the same FP64 storage. The triangular sweeps are FP64 either way. The
 * default is 1 for TP_MIXED, whose V-cycle is FP32, and 0 for TP_FP64. The
 * factor is redone at the next solve. */
tp_status tp_set_coarse_arith(tp_ctx* c, int arith);
/* Elimination order of the coarsest-level factor (CHOLMOD, which the
 * reference calls at stencil_assembly.c:394-396, picks its own fill-reducing
 * order): 0 = the natural node order, one band; 1 (the default) = one level
 * of nested dissection, the middle x node plane as the separator: the two
 * halves are banded factors eliminated at the same time (half the natural
 * chain of 32-column steps each), then the separator's Schur complement, and
 * the solve sweeps both halves in the same phases. Order 1 applies with the
 * single-launch variant where the coarsest grid is large enough (otherwise
 * the natural band is used); where a solve phase of both halves does not fit
 * the shared memory (wide bands), the halves are swept one after the other,
 * and order 2 asks for that form everywhere. The orders agree to rounding;
 * the factor is redone at the next solve. */
tp_status tp_set_coarse_order(tp_ctx* c, int order);
/* Failure detection of the single-launch coarse factor and solve (host-side
 * fault injection, for tests): each of their waits in global memory gives up
 * after spin polls (0 = the default, about a second) and, with missing = 1,
 * each grid barrier of the solve waits for one arrival that never comes, so
 * every such wait runs out. The factor or solve then reports TP_ERR_TIMEOUT
 * and the context stays usable; (0, 0) restores the defaults. */
tp_status tp_fault_coarse_barrier(tp_ctx* c, long spin, int missing);
/* Launch plan of the element-centric level-0 kernel for one vector type and
 * fused mode (no counterpart in the reference): the one tp_autotune chose, or
 * one set by the caller -- to keep a tuning between runs, or to pick one by
 * hand. vec = 0 FP32 vectors (the mixed form's V-cycle), 1 double vectors (in
 * the arithmetic tp_set_fine_arith selected); mode = 0 product, 1 product
 * with the dot product, 2 damped-Jacobi sweep, 3 residual. plan[0..6] =
 * {z groups of node rows per CTA, x chunks, staging of b and invD (0 read
 * from global memory, 1 staged per CTA in shared memory, 2 copied ahead by
 * each thread, FP32 only), register cap (FP32: 1 = capped for more CTAs per
 * SM), packed (FP32 modes 0, 2, 3: two z groups per thread in f32x2
 * arithmetic; groups even), moduli staged in shared memory one layer ahead
 * (1; 0 = loaded into registers per layer, FP32 one-group kernel only),
 * threads along y (read only)} -- tp_get_fine_plan fills plan[0..6],
 * tp_set_fine_plan reads plan[0..5] and returns TP_ERR_ARG for a plan the
 * grid or the shared memory does not allow. */
tp_status tp_get_fine_plan(tp_ctx* c, int vec, int mode, int* plan);
tp_status tp_set_fine_plan(tp_ctx* c, int vec, int mode, const int* plan);
/* Failure detection of the set-up (host-side fault injection, for tests; no
 * counterpart in the reference, which checks no allocation): with k > 0, the
 * k-th device or pinned-host allocation the library makes from now on fails
 * as if cudaMalloc had returned cudaErrorMemoryAllocation, without calling it;
 * k = 0 switches the injection off. tp_create then returns TP_ERR_ALLOC with
 * the context's message set, and tp_destroy of that context frees what was
 * allocated. Returns the number of the library's allocations currently live
 * (every context's), so a test can check that nothing is left behind. */
long tp_fault_alloc(long k);
/* Times the element-centric kernel's launch shapes (z groups per CTA, x
 * chunks) for each precision and fused mode on the context's grid and keeps
 * the fastest. It overwrites the solver work vectors (not F, U, x, xPhys):
 * call it before a solve, not inside one. ms_out (optional, 8 entries)
 * receives the best time per (precision, mode): FP32 modes 0-3, then the
 * double-vector modes 4-7 in the arithmetic tp_set_fine_arith selected. */
tp_status tp_autotune(tp_ctx* c, double* ms_out);
/* Multi-load problem generator (no counterpart in the reference, whose one
 * load is built at stencil_optimization.c:41-95): fills F_host (ncase columns
 * of 3*(nelx+1)*(nely+1)*(nelz+1) doubles) with ncase load cases of nload unit
 * nodal forces each, on distinct nodes of the free end face x = nelx drawn
 * uniformly, directions uniform on the unit sphere; SplitMix64 from seed.
 * Upload it as TP_FIELD_F of a context created with nrhs = ncase; the design
 * loop then minimises the summed compliance of the cases. */
tp_status tp_multiload(int nelx, int nely, int nelz, int ncase, int nload, unsigned long long seed,
                       double* F_host);
/* How tp_solve drives the CG loop (no counterpart in the reference):
 * on = 0 (default) one CUDA graph launch (a conditional while node over the
 * captured iteration) for contexts with nrhs > 1, the host-driven loop of the
 * reference for one load; 1 = the graph launch always; 2 = the host-driven
 * loop always (every kernel then shows in the tp_profile_* timings). */
tp_status tp_set_graph_solve(tp_ctx* c, int on);

/* How tp_design_iteration drives one iteration (no counterpart in the
 * reference, whose loop waits on the device ~55 times per iteration:
 * stencil_optimization.c:148-189, gpu_definitions.c:94-157):
 * on = 1 (default) with a single host wait, at the iteration's end -- the CG
 * loop is one graph launch (a conditional while node, also for one load), the
 * volume and the constraint value stay on the device, the OC bisection is one
 * graph launch (a conditional while node over batches of 8 steps, capped at
 * 240 steps), and the coarse factor's status word comes back with the
 * scalars; on = 0 host-driven as the reference (one residual read per CG
 * iteration for one load, the volume read before the OC update, the
 * bisection checked every 24 steps). Both give the same bits. With
 * tp_profile_enable on, iterations run host-driven so that every kernel is
 * timed. */
tp_status tp_set_device_loop(tp_ctx* c, int on);

/* Checkpoint/restart of the loop state (no counterpart in the reference):
 * x, xPhys, U and F (all load cases) with the grid, level count, load-case
 * count, precision, volfrac, rmin and the caller's design-iteration number,
 * in one binary file with an FNV-1a checksum (layout in tp_checkpoint.cpp),
 * written to <path>.tmp and renamed. Load requires the same grid and nrhs;
 * it rejects a missing, truncated or corrupt file with TP_ERR_ARG.
 * tp_checkpoint_info reads and checks a file without a context: info[7] =
 * {nelx, nely, nelz, nl, nrhs, precision, loop}. */
tp_status tp_checkpoint_save(tp_ctx* c, const char* path, int loop);
tp_status tp_checkpoint_load(tp_ctx* c, const char* path, int* loop);
tp_status tp_checkpoint_info(const char* path, int* info);
/* Per load case of the last tp_solve: iters[r] = index of the CG iteration at
 * which case r met the tolerance (-1 if it did not), relres[r] its relative
 * residual then (nrhs entries each). */
tp_status tp_solve_columns(tp_ctx* c, int* iters, double* relres);
/* The reference's matrix-free subspace operator of any level >= 1
 * (stencil_methods.c:436-519): unlike tp_apply at levels >= 2, fixed columns
 * keep their coupling; fixed rows return the input. Level 0 = tp_apply. */
tp_status tp_apply_subspace(tp_ctx* c, int level, const double* in_dev, double* out_dev);
/* nswp damped-Jacobi sweeps with a caller-supplied inverse diagonal (NULL =
 * the assembled one); subspace != 0 selects the subspace operator at levels
 * >= 2 (stencil_solvers.c:11-49), else the V-cycle's operator of that level. */
tp_status tp_smooth_ex(tp_ctx* c, int level, int subspace, int nswp, double omega, const double* invD_dev,
                       const double* b_dev, double* u_dev);
/* Copies the assembled block stencil of a level >= 1 to the host:
 * 243*nodes doubles, A[(m*9 + 3*a + b)*nodes + n] couples DOF a of node n with
 * DOF b of neighbour m = (dx+1)*9 + (dz+1)*3 + (dy+1). */
tp_status tp_download_stencil(tp_ctx* c, int level, int subspace, double* host);
/* Band-Cholesky factor of a caller's coarsest-level CSR (host arrays, n rows,
 * entries with column <= row are read) and solves with that factor
 * (stencil_assembly.c:428-503). */
tp_status tp_coarse_factor_csr(tp_ctx* c, long n, const int* rowptr, const int* col, const double* val);
tp_status tp_coarse_solve_factored(tp_ctx* c, const double* rhs_dev, double* x_dev);
/* Reductions and the OC bisection over arbitrary device arrays of length n
 * (gpu_definitions.c:94-157): sum, max|x - xnew| with x <- xnew, and xnew
 * from x, dv, dc and the constraint value g. */
tp_status tp_vec_sum(tp_ctx* c, long n, const double* v_dev, double* out);
tp_status tp_vec_change(tp_ctx* c, long n, double* x_dev, const double* xnew_dev, double* change);
tp_status tp_oc_bisect(tp_ctx* c, long n, const double* x_dev, const double* dv_dev, const double* dc_dev,
                       double g, double* xnew_dev);

/* Density-filter adjoint v <- H (v / Hs) without any device allocation and
 * without a context; it has no counterpart in the reference. It is for callers
 * that cannot call cudaMalloc: applications that reserve the GPU's memory as
 * their own arena or pool and forbid linked libraries to allocate or free
 * device memory (an outside allocation can exhaust or fragment the arena, and
 * cudaFree waits for the whole device), and loops with a fixed time budget
 * that cannot absorb an allocation's latency. The caller passes v (device,
 * nelx*nely*nelz doubles, overwritten in place) and a cudaStream_t (NULL = the
 * default stream); the work is queued on that stream and the call returns
 * without waiting. The intermediate v/Hs lives in a fixed 16 MiB device array
 * compiled into the library, so grids above
 * tp_filter_T_noalloc_max_elements() elements (2^21) are rejected with
 * TP_ERR_ARG, as are a non-positive or non-finite rmin. The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress) and
 * should come before any stream capture. All calls share the array, which
 * keeps the last call's contents: calls that overlap on the GPU race. A launch
 * failure returns TP_ERR_CUDA; an error left pending by the caller's own
 * earlier work is neither reported nor cleared. */
tp_status tp_filter_T_noalloc(int nelx, int nely, int nelz, double rmin, double* v_dev, void* stream);
long tp_filter_T_noalloc_max_elements(void);

/* Optional timing of kernel classes with CUDA events on the context's
 * stream (fine_apply_f64, fine_jacobi_f32, stencil, coarse_solve, ...).
 * tp_profile_get folds finished events into per-class launch counts and
 * milliseconds; name receives a static string. */
tp_status tp_profile_enable(tp_ctx* c, int on);
tp_status tp_profile_reset(tp_ctx* c);
int tp_profile_classes(void);
tp_status tp_profile_get(tp_ctx* c, int idx, const char** name, long* launches, double* ms);

#ifdef __cplusplus
}
#endif
#endif
