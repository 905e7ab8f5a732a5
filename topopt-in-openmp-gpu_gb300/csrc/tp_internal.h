// Internal declarations of libtopopt_gb300 (not part of the public C ABI).
//
// Device layout (every vector, every level): canonical, unpadded, AoS.
//   level l: ex = nelx >> l elements in x (ey, ez likewise), nx = ex + 1 nodes;
//   node (i, k, j) -> n = (i*nz + k)*ny + j, DOFs 3n + {0,1,2} (x, y, z);
//   fine element (i, k, j) -> (i*nelz + k)*nely + j.
// This is the reference's ordering (stencil_utility.h:19-52) with its halo
// and its y-padding to multiples of 128 (gpu_definitions.c:67-92) removed;
// the reference-layout entry points convert at the boundary.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <utility>
#include <vector>

#include "topopt_gb300.h"

#define TP_MAXL 8

namespace tp {

// Every device and pinned-host allocation of the library goes through these
// (tp_api.cu). They count the live allocations and honour the host-side
// fault injection of tp_fault_alloc: the chosen allocation fails as if
// cudaMalloc had returned cudaErrorMemoryAllocation, without calling it.
cudaError_t dev_malloc(void** p, size_t bytes);
void dev_free(void* p);
cudaError_t host_malloc_pinned(void** p, size_t bytes);
void host_free_pinned(void* p);
template <typename T>
inline cudaError_t dev_malloc(T** p, size_t bytes) {
  return dev_malloc(reinterpret_cast<void**>(p), bytes);
}

struct Level {
  int ex, ey, ez;     // elements
  int nx, ny, nz;     // nodes
  long nnodes, ndof;
  int lim;            // fixed strip width: nodes j < lim or j >= ny - lim on the x=0 face
  long nfixed;        // fixed DOFs
};

Level make_level(int nelx, int nely, int nelz, int l);

// Host set-up (tp_setup.cpp)
void element_matrix_tables(double nu, int l, double* KE);   // 576 * ncell^3
void cantilever_load(const Level& L0, double* F);            // 3*nnodes
bool moment_tables(const double* ke0, const double* ke_l, int l, std::vector<int>& off, std::vector<int>& pidx,
                   std::vector<double>& coef);               // level-l element matrices from 27 moments

// Reduction scratch: partial sums of one pass, one slot per block.
constexpr int kRedSlots = 4096;

// Scalars the CG keeps on the device (indices into ctx->d_scal).
enum Scalar {
  S_RHO = 0, S_RHOOLD, S_ALPHA, S_BETA, S_DPR, S_RNORM2, S_BNORM2, S_RELRES,
  S_C, S_VOL, S_CHANGE, S_L1, S_L2, S_LMID, S_GT, S_OCDONE, S_TMP0, S_TMP1,
  S_CONV,   // column converged (1) in the current solve
  S_ITER,   // iteration at which it converged
  S_MAXRR,  // (column 0) largest relres over the columns
  S_IT,     // (column 0) iteration counter of the captured CG loop
  S_G,      // (column 0) constraint value g = vol - volfrac of the OC bisection
  S_RL,     // (column 0) 1/sqrt(lmid) of the next bisection step, formed once per step
  S_BLO,    // (column 0) the bisection's first phase, searched: steps below BLO keep gt <= 0,
  S_BHI,    //            step BHI has gt > 0 (or BHI = cap + 1); S_TMP1 the step probed
  S_DVBAD,  // (column 0) nonzero when some dv is not positive: the first phase runs step by step
  S_COUNT
};

// The coarsest-level direct solver: band Cholesky on FP64 storage, FP64 or
// double-single arithmetic (tp_cholesky.cu).
// Its status word (Coarse::info) holds the first non-positive pivot's column
// + 1, or'ed with kCoarseWaitGaveUp if a bounded wait inside the factor gave up.
constexpr int kCoarseWaitGaveUp = 1 << 30;
struct Coarse {
  long n = 0, bw = 0;           // order, half bandwidth
  double* band = nullptr;       // L(r,c) at c*bw + r, 0 <= r - c <= bw (column-major, ld = bw)
  size_t band_elems = 0;
  int nbs = 0, nblk = 0;        // solve block size and count
  double* dinv = nullptr;       // inverse D_k of each diagonal block of L, row-major nbs*nbs per block
  double* dinvT = nullptr;      // D_k^T, row-major
  double* lrow = nullptr;       // row-major band rows left of each block: nbs x bw per block
  double* vec = nullptr;        // work columns: y (8), t (8), rhs, sol (n each)
  double* rhs = nullptr;
  double* sol = nullptr;
  int* info = nullptr;          // device status: first non-positive pivot + 1, 0 if none
  double* linv = nullptr;       // current 32x32 diagonal block of L (row-major) and its 32 reciprocal pivots
  cudaGraphExec_t graph_exec = nullptr;   // the captured block-solve sequence
  cudaGraphExec_t factor_exec = nullptr;  // the captured factorisation sequence
  cudaStream_t s2 = nullptr;    // second stream of the factorisation's lookahead
  cudaEvent_t ev_panel = nullptr, ev_rest = nullptr;
  int prio_high = 0;            // highest stream priority of the device (the lookahead chain)
  int nsm = 0;                  // SMs of the device
  // single-launch solve (one cooperative kernel for all block steps)
  unsigned* bar = nullptr;      // its grid-barrier counter, then the status word (serr) and the exit counter; zero between launches
  int* serr = nullptr;          // its device status: 1 = a barrier wait gave up (until the host reads it)
  int ps_grid = 0, ps_R = 0, ps_P = 0, ps_seg = 0;  // CTAs, rows per CTA, warps per row, staged doubles per warp
  size_t ps_smem = 0;
  long ps_spin = 0;             // polls before a barrier wait gives up (0: the default, about a second)
  int ps_missing = 0;           // arrivals each barrier waits for beyond the grid (failure-detection test only)
  int solve_variant = 0;        // 0: single launches (factor and solve) where their plans apply; 1: launches per step
  bool alloc_failed = false;    // an allocation of the set-up failed (tp_create reports TP_ERR_ALLOC)
  int ds = 0;                   // single-launch factor and block inverses in double-single arithmetic
  // single-launch factor (one cooperative kernel for all 32-column steps)
  bool pf_ok = false;
  int pf_grid = 0;              // its CTAs (one per SM)
  int pf_NT = 0, pf_TS = 0;     // diagonal tiles; row stride of its flag arrays
  int* pf_flags = nullptr;      // fdone [NT], sdone [NT][TS], tver [NT][TS], abort [1]
  size_t pf_flag_bytes = 0;
  double* pf_rpk = nullptr;     // [NT][32] reciprocal pivots per diagonal tile
  long* pf_off = nullptr;       // [NT+1] work items of the other CTAs before each step
  // One level of nested dissection (x planes): the node plane xs is the
  // separator S; part A (planes < xs, natural order) and part B (planes > xs,
  // in mirrored plane order) are each a band with S as a trailing block,
  // factored at the same time by halves of the grid up to S; S's Schur
  // complement (the sum of the two trailing blocks) is then factored alone.
  // Composite rows: view A [pad_a, A, S tail], view B [pad_b, B, S tail],
  // view S; the band, block inverses and block rows share the arrays above.
  int order = 1;                // requested: 0 natural band, 1 dissected where its plan applies,
                                //   2 dissected with the halves' sweeps one after the other
  bool nd_ok = false;           // the dissected plan applies (sizes, launch plans)
  bool nd_use = false;          // the current factor is the dissected one
  int nd_xs = 0;                // separator plane
  long nd_ns = 0;               // separator rows
  long nd_own[3] = {0, 0, 0};   // rows in solve blocks per view (pad + part; S: ns)
  long nd_org[3] = {0, 0, 0};   // first composite row of each view
  long nd_pad[2] = {0, 0};      // identity rows ahead of A and B (own rows a multiple of 32)
  int nd_nblk[3] = {0, 0, 0};   // solve blocks per view
  int nd_blk0[3] = {0, 0, 0};   // first block of each view in dinv / lrow
  long nd_ntot = 0;             // composite rows
  int* nd_map = nullptr;        // [ntot] composite row -> natural row, -1 for pads and tails
  double* nd_vec = nullptr;     // composite work columns: rhs, y, t, x, 8 columns each
  double* nd_tail = nullptr;    // [2][ns][bw] rows of the A and B tails left of S, row-major
  int nd_NT[3] = {0, 0, 0}, nd_TS[3] = {0, 0, 0};  // factor steps and flag row stride per view
  int* nd_flags = nullptr;      // per view: fdone, sdone, tver; then the shared abort flag
  size_t nd_flag_bytes = 0;
  long nd_fo[3] = {0, 0, 0};    // offsets of each view's flags in nd_flags
  double* nd_rpk = nullptr;     // per view [NT][32]
  long* nd_off = nullptr;       // per view [NT+1] work items
  long nd_ro[3] = {0, 0, 0}, nd_io[3] = {0, 0, 0};  // offsets into nd_rpk (tiles) and nd_off
  int nd_grid[2] = {0, 0};      // CTAs of the dissected factor's launches, FP64 and double-single
  int nd_split[2] = {0, 0};     // CTAs of the A group in the concurrent factor
  int ps2_grid = 0, ps2_R = 0, ps2_P = 0, ps2_seg = 0;  // solve plan of two views per phase
  size_t ps2_smem = 0;
  cudaGraphExec_t nd_graph_exec = nullptr, nd_factor_exec = nullptr;
};

// Launch plan of the element-centric level-0 kernel (tp_kernels_fine_ec.cu):
// z groups of node rows (ngz groups of zbase or zbase + 1 rows), nzg groups
// per CTA, ncx chunks of cx node planes along x, nyt threads along y.
struct EcPlan {
  bool ok = false;
  int nyt = 0, nzg = 1, ngz = 0, zbase = 0, zextra = 0, ncx = 1, cx = 0;
  int own = 0;  // sweep/residual: 1 stage b and invD in shared memory per CTA; 2 (packed
                //   kernel) each thread copies its own entries ahead into shared memory
  int occ3 = 0;  // FP32: the form with registers capped for more CTAs per SM
  int pk = 0;    // FP32: the packed kernel (two z groups per thread, f32x2 arithmetic)
  int estage = 1;  // the moduli E staged in shared memory one layer ahead (FP32 one-group
                   //   kernel: 0 loads them into registers when a layer starts)
};
struct EcGeom {
  int nx, ny, nz, ex, ey, ez, lim;
  int ngz, zbase, zextra, cx;
  long vstride;               // distance between right-hand sides
  int slab_bytes, own_bytes;  // shared memory per stage
  int e_bytes;                // shared memory per stage of the moduli E
  int pt_bytes;               // packed kernel: per-thread slots of b and invD (0: not used)
};
// fused consumers of the level-0 operator
enum { FM_APPLY = 0, FM_APPLY_DOT = 1, FM_JACOBI = 2, FM_RESID = 3 };

// Kernel classes the optional CUDA-event profiler times (tp_profile_*).
enum ProfId {
  P_FINE_APPLY_F64 = 0, P_FINE_JACOBI_F64, P_FINE_RESID_F64,
  P_FINE_APPLY_F32, P_FINE_JACOBI_F32, P_FINE_RESID_F32,
  P_STENCIL, P_TRANSFER, P_COARSE_SOLVE, P_COARSE_FACTOR, P_ASSEMBLE,
  P_VECTOR, P_DESIGN, P_COUNT
};

}  // namespace tp

struct tp_ctx {
  tp_params p;
  int nl;
  tp::Level L[TP_MAXL];
  cudaStream_t s = nullptr;
  int device = 0;
  std::string err;   // sticky: a CUDA error; every later call fails
  std::string note;  // the last failure that leaves the context usable (a non-positive pivot, a
                     // non-finite residual, a bounded wait that gave up, a checkpoint file refused)

  // element stiffness tables per level (576 * ncell^3), FP64 and FP32 copies
  double* d_ke[TP_MAXL] = {};
  // levels >= 2: element matrices from moments (tp_setup.cpp moment_tables):
  // coefficients [nnz], then moment indices [nnz] and block offsets [577] as ints
  double* d_mgc[TP_MAXL] = {};
  int* d_mgi[TP_MAXL] = {};
  int mg_nnz[TP_MAXL] = {};   // 0: that level assembles from the sub-cell tables
  double* d_mom = nullptr;    // 27 moments per coarse element (the largest such level)
  float* d_kef[TP_MAXL] = {};

  // design fields (fine elements), FP64
  double *d_x = nullptr, *d_xphys = nullptr, *d_xnew = nullptr, *d_dc = nullptr,
         *d_dv = nullptr, *d_hs = nullptr;
  double* d_E = nullptr;  // E(xPhys) per fine element
  double* d_fw = nullptr; // nonzero filter weights, then their packed offsets (x, z, y loop order)
  int fw_n = 0;           // their count
  double* d_ocb = nullptr;  // OC scratch, 3 x ocb_n: x sqrt(-dc/dv), max(0, x-0.2), min(1, x+0.2) per element
  long ocb_n = 0;
  float* d_Ef = nullptr;

  // state: load and displacement (FP64), nrhs columns, column-contiguous
  double *d_F = nullptr, *d_U = nullptr;

  // CG vectors (FP64)
  double *d_r = nullptr, *d_z = nullptr, *d_p = nullptr, *d_q = nullptr;

  // multigrid vectors per level, in the V-cycle precision
  // (FP64 form: the double set; mixed form: the float set)
  double *mg_r[TP_MAXL] = {}, *mg_z[TP_MAXL] = {}, *mg_d[TP_MAXL] = {}, *mg_t[TP_MAXL] = {};
  float *mgf_r[TP_MAXL] = {}, *mgf_z[TP_MAXL] = {}, *mgf_d[TP_MAXL] = {}, *mgf_t[TP_MAXL] = {};
  double* invD[TP_MAXL] = {};
  float* invDf[TP_MAXL] = {};

  // assembled block stencils of levels 1 .. nl-1, half stored (kStencilCoef
  // coefficients per node, coefficient-major: A[((m-13)*9 + c*3 + d)*nnodes + n]
  // for the neighbours m = 13..26), without boundary conditions
  double* st[TP_MAXL] = {};
  float* stf[TP_MAXL] = {};
  // on demand: an FP64 copy of a level that only has an FP32 stencil (the
  // mixed form), for the reference-signature entry points
  double* st_sub[TP_MAXL] = {};
  bool st_sub_valid[TP_MAXL] = {};
  double* scratch_invD = nullptr;

  tp::Coarse coarse;

  // reductions
  double* d_red = nullptr;   // kRedSlots partials
  double* d_scal = nullptr;  // S_COUNT scalars
  double* h_scal = nullptr;  // pinned mirror
  int* d_flag = nullptr;     // device error flag (bounded waits)

  // level-0 kernel selection: 0 element-centric where it applies, 1 the
  // node-centric stencil everywhere; plans per precision and fused mode
  int fine_variant = 0;
  // element-centric operator on double vectors evaluated in double-single
  // (pairs of floats) instead of FP64; plans of its own
  int fine_ds = 0;
  bool ec_ok = false;        // KZ built and its sparsity pattern verified
  tp::EcPlan ec_f32[4], ec_f64[4], ec_ds[4];

  bool assembled = false;    // operators built for the current xPhys
  bool assemble_pending = false;  // tp_assemble_async enqueued an assembly that tp_assemble completes
  long mem_bytes = 0;

  // the multi-load solve: one CUDA graph per context, a while-node looping
  // over the captured CG iteration (tp_api_batch.cu)
  bool capturing = false;    // launches are being recorded into a graph
  cudaGraphExec_t cg_exec = nullptr;
  int cg_exec_nr = 0;        // columns the captured graph solves
  int graph_solve = 0;       // 1: tp_solve runs the captured graph also for one load
  // the design iteration without host round trips before its end
  // (tp_set_device_loop): CG loop and OC bisection as graph launches
  int device_loop = 1;
  cudaGraphExec_t oc_exec = nullptr;  // the OC bisection steps under a conditional while node
  int* h_info = nullptr;     // pinned: the coarse factor's status word, read at the iteration's end
  cudaEvent_t it_ev[2] = {nullptr, nullptr};  // brackets of tp_design_iteration's device time

  // optional per-kernel-class timing with CUDA events on c->s
  bool prof = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
  size_t ev_next = 0;
  long prof_launches[tp::P_COUNT] = {};
  double prof_ms[tp::P_COUNT] = {};
};

namespace tp {
// brackets one launch (or a short sequence) of class `id` when profiling is on
struct ProfScope {
  tp_ctx* c;
  int id;
  cudaEvent_t e1 = nullptr;
  ProfScope(tp_ctx* ctx, int i);
  ~ProfScope();
};
void prof_collect(tp_ctx* c);  // folds finished event pairs into the totals
void prof_destroy(tp_ctx* c);
}  // namespace tp

namespace tp {

// kernels (tp_kernels_*.cu); every launcher enqueues on ctx->s
void set_fine_ke(const double* ke0_host);  // __constant__ copies (FP64 + FP32)

void compute_E(tp_ctx* c);  // d_E, d_Ef from d_xphys
int fine_blocks(const tp_ctx* c);

// level 0 (matrix-free hex8 stencil)
// nr: right-hand sides stored as consecutive columns of ndof(0) (E and invD are shared)
template <typename T> void fine_apply(tp_ctx* c, const T* E, const T* in, T* out, int nr = 1);
template <typename T> int fine_apply_dot(tp_ctx* c, const T* E, const T* in, T* out, int nr = 1);  // + <in,out> partials per column; returns their count per column
template <typename T> void fine_jacobi(tp_ctx* c, const T* E, const T* invD, const T* b, const T* u, T* unew, T omega, int nr = 1);
template <typename T> void fine_resid(tp_ctx* c, const T* E, const T* b, const T* u, T* d, int nr = 1);
void fine_inv_diag(tp_ctx* c, double* invD);
// element-centric form (tp_kernels_fine_ec.cu): returns the number of CTAs
// launched, or -1 when the plan or the pointers rule it out
bool set_fine_kz(const double* ke0, double* kz_out);
// The 45 non-zeros (index, row, column) of KZ = T KE T^T / 64 (T the per-axis
// sum/difference transform of an element's 8 nodes, b = bx*4 + by*2 + bz,
// row = 3b + c), listed once for every kernel that unrolls over them.
#define TP_KZ_PATTERN(X)                                                                                     \
  X(0, 3, 3) X(1, 3, 14) X(2, 4, 4) X(3, 4, 8) X(4, 5, 5) X(5, 5, 7) X(6, 5, 12) X(7, 6, 6) X(8, 6, 13)     \
  X(9, 9, 9) X(10, 9, 16) X(11, 9, 20) X(12, 7, 5) X(13, 7, 7) X(14, 7, 12) X(15, 10, 10) X(16, 10, 15)   \
  X(17, 8, 4) X(18, 8, 8) X(19, 11, 11) X(20, 11, 18) X(21, 12, 5) X(22, 12, 7) X(23, 12, 12)             \
  X(24, 15, 10) X(25, 15, 15) X(26, 13, 6) X(27, 13, 13) X(28, 16, 9) X(29, 16, 16) X(30, 16, 20)          \
  X(31, 14, 3) X(32, 14, 14) X(33, 17, 17) X(34, 17, 19) X(35, 18, 11) X(36, 18, 18) X(37, 21, 21)         \
  X(38, 19, 17) X(39, 19, 19) X(40, 22, 22) X(41, 20, 9) X(42, 20, 16) X(43, 20, 20) X(44, 23, 23)
void set_design_kz(const double* kz45);  // the KZ values for the element energies (tp_kernels_design.cu)
bool ec_plan(tp_ctx* c, int nzg, int ncx, EcPlan* p);
void ec_default_plans(tp_ctx* c);
void ec_select_packed(tp_ctx* c, bool on);  // FP32 plans: packed kernel defaults or one-group defaults
template <typename T> int fine_ec(tp_ctx* c, int mode, const T* E, const T* in, T* out, const T* b, const T* invD, T omega, int nr = 1);

// levels >= 1 (assembled block stencils)
// Level >= 1 stencils: the symmetric operator without boundary conditions,
// half stored (kStencilCoef coefficients per node); masked < 0 applies the
// level's own conditions (fixed rows identity; columns of fixed DOFs dropped
// from level 2 on), 0 or 1 forces the column masking off or on.
constexpr int kStencilCoef = 14 * 9;
template <typename T> void assemble_stencil(tp_ctx* c, int l, const T* E, const T* ke, T* st, double* invD);
template <typename T> void stencil_apply(tp_ctx* c, int l, const T* st, const T* in, T* out, int nr = 1, int masked = -1);
template <typename T> void stencil_jacobi(tp_ctx* c, int l, const T* st, const T* invD, const T* b, const T* u, T* unew, T omega, int nr = 1, int masked = -1);
template <typename T> void stencil_resid(tp_ctx* c, int l, const T* st, const T* b, const T* u, T* d, int nr = 1, int masked = -1);
void stencil_expand(tp_ctx* c, int l, const double* st, double* out, int masked);  // full 243-coefficient form with BCs

// grid transfer
template <typename T> void restrict_fw(tp_ctx* c, int l, const T* fine, T* coarse, int nr = 1);
template <typename T> void prolong_add(tp_ctx* c, int l, const T* coarse, T* fine, int nr = 1);
template <typename T> void prolong_set(tp_ctx* c, int l, const T* coarse, T* fine, int nr = 1);

// vectors
template <typename T> void vscale(tp_ctx* c, long n, const T* a, const T* b, T* out, T omega, int nr = 1);  // out = omega*a*b
template <typename TB>
void dot_partials(tp_ctx* c, long n, const double* a, const TB* b, int* nblocks, int nr = 1);
#ifdef __CUDACC__
// The 256 values of a block (one per thread) folded in a fixed tree --
// pairs (i, i + 128), then (i, i + 64), (i, i + 32), then a warp's shuffles
// -- so that the result is the same at every run; the value is thread 0's.
// On this part an FP64 add holds its unit for ~67 cycles, so the serial fold
// of 256 values by one thread took ~8 us.
__device__ __forceinline__ double fold256(double v, bool is_max, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = 128; w >= 32; w >>= 1) {
    if (threadIdx.x < w) {
      const double a = sh[threadIdx.x], b = sh[threadIdx.x + w];
      sh[threadIdx.x] = is_max ? fmax(a, b) : a + b;
    }
    __syncthreads();
  }
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = sh[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) {
      const double b = __shfl_down_sync(0xffffffffu, r, o);
      r = is_max ? fmax(r, b) : r + b;
    }
  }
  return r;
}

// (sh: 256 doubles of shared memory; every thread of the block calls it)
#endif
void finish_sum(tp_ctx* c, int nblocks, int slot, int op, int nr = 1);  // column r: partials -> d_scal[r*S_COUNT + slot]
void cast_d2f(tp_ctx* c, long n, const double* a, float* b);
void cast_f2d(tp_ctx* c, long n, const float* a, double* b);
template <typename TZ>
void cg_pupdate(tp_ctx* c, long n, const TZ* z, double* p, int first, int nr = 1);
void cg_xr_update(tp_ctx* c, long n, double* u, double* r, const double* p, const double* q, int* nblocks, int nr = 1,
                  float* rf = nullptr);
void cg_scalars(tp_ctx* c, int what, int nr = 1, double tol = 0.0, int iter = 0);
void cg_reset(tp_ctx* c, int nr);

// coarsest level (tp_cholesky.cu)
void coarse_alloc(tp_ctx* c);
void coarse_free(tp_ctx* c);
void coarse_assemble(tp_ctx* c);  // from the FP64 stencil of level nl-1
void coarse_factor(tp_ctx* c);
void coarse_use_natural(tp_ctx* c);  // a caller's natural-order factor follows (tp_coarse_factor_csr)
void coarse_graphs_free(tp_ctx* c);  // the captured factor and solve sequences
void coarse_solve(tp_ctx* c, const double* rhs, double* x, int nr = 1);  // nr columns of ndof(nl-1)
// TP_ERR_TIMEOUT (with the message set) if a single-launch solve gave up at a
// grid barrier; synchronises the context's stream
tp_status coarse_status(tp_ctx* c);

// design-variable ops (tp_kernels_design.cu)
void compliance(tp_ctx* c, const double* u, double* dc, int* nblocks, int nr = 1);  // sums over the nr load cases
void filter_hs(tp_ctx* c, double* hs);
void filter_fwd(tp_ctx* c, const double* x, double* out);
void filter_adj(tp_ctx* c, double* v, double* tmp);
void volume_partials(tp_ctx* c, const double* xphys, int* nblocks);
int oc_update(tp_ctx* c, double g);   // bisection; leaves xnew, change and x <- xnew
// the same bisection as one graph launch, g read from d_scal[S_G]: enqueues
// only (no host wait); S_OCDONE = 0 afterwards means it hit its step cap
bool oc_update_graph(tp_ctx* c);
void oc_graph_free(tp_ctx* c);
void constraint_from_volume(tp_ctx* c);  // d_scal[S_G] = d_scal[S_VOL] / nelem - volfrac
int oc_bisect(tp_ctx* c, long n, double* x, double* xnew, const double* dc, const double* dv, double g,
              bool commit);
void vec_change(tp_ctx* c, long n, double* x, const double* xnew);  // S_CHANGE, x <- xnew
void vec_sum(tp_ctx* c, long n, const double* v, int slot);
void element_sens(tp_ctx* c, const double* u, const double* w, double* out);
int filter_fwd_blocks(const tp_ctx* c);
void set_design_ke(const double* ke0_host);

// PCG pieces (tp_api.cu) and the graph-captured solve (tp_api_batch.cu)
void pcg_prologue(tp_ctx* c, const double* b, const double* u, int nr);
void pcg_iteration(tp_ctx* c, double* u, int iter, int nr);
tp_status pcg_graph(tp_ctx* c, int* iters, double* relres);
tp_status pcg_graph_enqueue(tp_ctx* c);  // set-up and the graph launch, no host wait
tp_status pcg_graph_status(tp_ctx* c, int* iters, double* relres);  // after h_scal is copied back
void graph_free(tp_ctx* c);

// error helpers
bool cuda_ok(tp_ctx* c, cudaError_t e, const char* what);
int grid_for(long n, int threads);

}  // namespace tp

#define TP_CHECK_LAUNCH(c, what)                                   \
  do {                                                             \
    cudaError_t _e = cudaGetLastError();                           \
    if (_e != cudaSuccess) {                                       \
      (c)->err = std::string(what) + ": " + cudaGetErrorString(_e); \
    }                                                              \
  } while (0)
