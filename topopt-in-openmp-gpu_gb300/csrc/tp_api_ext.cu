// Handle-API entry points that serve the reference-signature layer
// (topopt_ref_api.h): the unmasked "subspace" operator at any level, a
// smoother with a caller-supplied diagonal, stencil export, a coarse factor
// from a caller's CSR, and reductions / OC over arbitrary device arrays.
#include <algorithm>
#include <cmath>
#include <vector>

#include "tp_internal.h"

using namespace tp;

namespace {

tp_status sync_status(tp_ctx* c) {
  cudaError_t e = cudaStreamSynchronize(c->s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    c->err = cudaGetErrorString(e);
    return TP_ERR_CUDA;
  }
  return c->err.empty() ? TP_OK : TP_ERR_CUDA;
}

// FP64 stencil of level l >= 1 (half stored, no boundary conditions: the
// caller picks the semantics when it applies it -- the reference's subspace
// operator, stencil_methods.c:436-519, keeps the fixed columns; its CSR
// levels, stencil_assembly.c:226-259, drop them): the context's own where it
// is FP64, else an FP64 copy assembled on demand
const double* api_stencil(tp_ctx* c, int l) {
  if (c->assembled && c->st[l]) return c->st[l];
  if (!c->st_sub[l]) {
    if (dev_malloc(&c->st_sub[l], sizeof(double) * kStencilCoef * c->L[l].nnodes) != cudaSuccess) return nullptr;
    c->mem_bytes += 8L * kStencilCoef * c->L[l].nnodes;
  }
  if (!c->st_sub_valid[l]) {
    if (!c->scratch_invD) dev_malloc(&c->scratch_invD, sizeof(double) * c->L[0].ndof);
    compute_E(c);
    assemble_stencil<double>(c, l, c->d_E, c->d_ke[l], c->st_sub[l], c->scratch_invD);
    c->st_sub_valid[l] = true;
  }
  return c->st_sub[l];
}

}  // namespace

extern "C" {

tp_status tp_set_rmin(tp_ctx* c, double rmin) {
  if (!c || !(rmin > 0)) return TP_ERR_ARG;
  if (rmin != c->p.rmin) {
    c->p.rmin = rmin;
    filter_hs(c, c->d_hs);
  }
  return sync_status(c);
}

tp_status tp_set_cg(tp_ctx* c, double cgtol, int cgmax, int nswp, double omega) {
  if (!c || !(cgtol > 0) || cgmax < 1 || nswp < 0) return TP_ERR_ARG;
  if (c->p.cgtol == cgtol && c->p.cgmax == cgmax && c->p.nswp == nswp && c->p.omega == omega) return TP_OK;
  c->p.cgtol = cgtol;
  c->p.cgmax = cgmax;
  c->p.nswp = nswp;
  c->p.omega = omega;
  graph_free(c);  // the captured CG loop holds the old values
  return TP_OK;
}

tp_status tp_set_fine_variant(tp_ctx* c, int variant) {
  if (!c || variant < 0 || variant > 2) return TP_ERR_ARG;
  // 2 is the element-centric kernel with the packed FP32 plans; choosing 0 or
  // 2 resets the FP32 plans to that kernel's defaults
  if (variant != 1) ec_select_packed(c, variant == 2);
  c->fine_variant = variant == 1 ? 1 : 0;
  graph_free(c);
  return TP_OK;
}

tp_status tp_set_fine_arith(tp_ctx* c, int arith) {
  if (!c || arith < 0 || arith > 1) return TP_ERR_ARG;
  c->fine_ds = arith;
  graph_free(c);
  return TP_OK;
}

// the factorisation is redone with the chosen launches or arithmetic at the next solve
static void coarse_reset(tp_ctx* c) {
  coarse_graphs_free(c);
  c->assembled = false;
  c->assemble_pending = false;
  graph_free(c);
}

tp_status tp_set_coarse_solve_variant(tp_ctx* c, int variant) {
  if (!c || variant < 0 || variant > 1) return TP_ERR_ARG;
  c->coarse.solve_variant = variant;
  coarse_reset(c);
  return TP_OK;
}

tp_status tp_set_coarse_order(tp_ctx* c, int order) {
  if (!c || order < 0 || order > 2) return TP_ERR_ARG;
  c->coarse.order = order;
  coarse_reset(c);
  return TP_OK;
}

tp_status tp_set_coarse_arith(tp_ctx* c, int arith) {
  if (!c || arith < 0 || arith > 1) return TP_ERR_ARG;
  c->coarse.ds = arith;
  coarse_reset(c);
  return TP_OK;
}

tp_status tp_fault_coarse_barrier(tp_ctx* c, long spin, int missing) {
  if (!c || spin < 0 || missing < 0 || missing > 1) return TP_ERR_ARG;
  Coarse& C = c->coarse;
  C.ps_spin = spin;
  C.ps_missing = missing;
  coarse_graphs_free(c);  // the captured solve and factorisation hold the old values
  graph_free(c);
  return TP_OK;
}

tp_status tp_apply_subspace(tp_ctx* c, int level, const double* in, double* out) {
  if (!c || level < 0 || level >= c->nl || !in || !out) return TP_ERR_ARG;
  if (level == 0) return tp_apply(c, 0, in, out);
  const double* st = api_stencil(c, level);
  if (!st) return TP_ERR_ALLOC;
  stencil_apply<double>(c, level, st, in, out, 1, 0);  // fixed columns kept
  return sync_status(c);
}

tp_status tp_smooth_ex(tp_ctx* c, int level, int subspace, int nswp, double omega, const double* invD,
                       const double* b, double* u) {
  if (!c || level < 0 || level >= c->nl || !b || !u || nswp < 0) return TP_ERR_ARG;
  if (!c->assembled) {
    tp_status st = tp_assemble(c);
    if (st != TP_OK) return st;
  }
  const double* A = nullptr;
  if (level >= 1) {
    A = api_stencil(c, level);
    if (!A) return TP_ERR_STATE;
  }
  const int masked = (level >= 2 && !subspace) ? 1 : 0;
  const double* D = invD ? invD : c->invD[level];
  const long nd = c->L[level].ndof;
  double* cur = u;
  double* nxt = c->d_q;  // level-0 sized scratch
  for (int s = 0; s < nswp; s++) {
    if (level == 0)
      fine_jacobi<double>(c, c->d_E, D, b, cur, nxt, omega);
    else
      stencil_jacobi<double>(c, level, A, D, b, cur, nxt, omega, 1, masked);
    std::swap(cur, nxt);
  }
  if (cur != u) cudaMemcpyAsync(u, cur, sizeof(double) * nd, cudaMemcpyDeviceToDevice, c->s);
  return sync_status(c);
}

tp_status tp_download_stencil(tp_ctx* c, int level, int subspace, double* host) {
  if (!c || level < 1 || level >= c->nl || !host) return TP_ERR_ARG;
  if (!c->assembled) {
    tp_status st = tp_assemble(c);
    if (st != TP_OK) return st;
  }
  const double* A = api_stencil(c, level);
  if (!A) return TP_ERR_STATE;
  const long nc = 243L * c->L[level].nnodes;
  double* full = nullptr;
  if (dev_malloc(&full, sizeof(double) * nc) != cudaSuccess) return TP_ERR_ALLOC;
  stencil_expand(c, level, A, full, (level >= 2 && !subspace) ? 1 : 0);
  cudaMemcpyAsync(host, full, sizeof(double) * nc, cudaMemcpyDeviceToHost, c->s);
  tp_status st = sync_status(c);
  dev_free(full);
  return st;
}

// Factor the coarsest operator given as CSR on the host (row-major, the
// reference's coarse CSR layout); as CHOLMOD with stype = 1 does for that
// matrix, only entries with column <= row are read.
tp_status tp_coarse_factor_csr(tp_ctx* c, long n, const int* rowptr, const int* col, const double* val) {
  if (!c || !rowptr || !col || !val || n != c->coarse.n) return TP_ERR_ARG;
  Coarse& C = c->coarse;
  coarse_use_natural(c);
  std::vector<double> band(C.band_elems, 0.0);
  for (long r = 0; r < n; r++)
    for (int q = rowptr[r]; q < rowptr[r + 1]; q++) {
      const long cc = col[q];
      if (cc > r) continue;
      if (r - cc > C.bw) return TP_ERR_ARG;
      band[cc * C.bw + r] = val[q];
    }
  cudaMemcpyAsync(C.band, band.data(), sizeof(double) * C.band_elems, cudaMemcpyHostToDevice, c->s);
  coarse_factor(c);
  int info = 0;
  cudaMemcpyAsync(&info, C.info, sizeof(int), cudaMemcpyDeviceToHost, c->s);
  tp_status st = sync_status(c);
  if (st != TP_OK) return st;
  if (info & kCoarseWaitGaveUp) {
    c->note = "coarse Cholesky: a bounded wait gave up";
    return TP_ERR_TIMEOUT;
  }
  if (info != 0) {
    c->note = "coarse Cholesky: non-positive pivot at column " + std::to_string(info - 1);
    return TP_ERR_NOT_SPD;
  }
  return TP_OK;
}

// coarse solve with the current factor, without re-assembling it
tp_status tp_coarse_solve_factored(tp_ctx* c, const double* rhs, double* x) {
  if (!c || !rhs || !x) return TP_ERR_ARG;
  coarse_solve(c, rhs, x);
  tp_status st = sync_status(c);
  return st != TP_OK ? st : coarse_status(c);
}

tp_status tp_vec_sum(tp_ctx* c, long n, const double* v, double* out) {
  if (!c || n < 0 || !v || !out) return TP_ERR_ARG;
  vec_sum(c, n, v, S_TMP1);
  cudaMemcpyAsync(c->h_scal + S_TMP1, c->d_scal + S_TMP1, sizeof(double), cudaMemcpyDeviceToHost, c->s);
  tp_status st = sync_status(c);
  *out = c->h_scal[S_TMP1];
  return st;
}

tp_status tp_vec_change(tp_ctx* c, long n, double* x, const double* xnew, double* change) {
  if (!c || n < 0 || !x || !xnew || !change) return TP_ERR_ARG;
  vec_change(c, n, x, xnew);
  cudaMemcpyAsync(c->h_scal + S_CHANGE, c->d_scal + S_CHANGE, sizeof(double), cudaMemcpyDeviceToHost, c->s);
  tp_status st = sync_status(c);
  *change = c->h_scal[S_CHANGE];
  return st;
}

tp_status tp_oc_bisect(tp_ctx* c, long n, const double* x, const double* dv, const double* dc, double g,
                       double* xnew) {
  if (!c || n < 0 || !x || !dv || !dc || !xnew) return TP_ERR_ARG;
  if (oc_bisect(c, n, const_cast<double*>(x), xnew, dc, dv, g, false) != 0) {
    c->note = "OC bisection did not terminate";
    return TP_ERR_TIMEOUT;
  }
  return sync_status(c);
}

}  // extern "C"
