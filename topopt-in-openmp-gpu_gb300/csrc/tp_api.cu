// The handle API (include/topopt_gb300.h): context, operator assembly,
// V-cycle, PCG and the design loop, all stream-ordered on one CUDA stream
// of one GPU.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "tp_internal.h"

using namespace tp;

namespace tp {

namespace {
std::atomic<long> g_live_allocs{0};
std::atomic<long> g_fault_countdown{0};  // > 0: allocations left before the one that fails
bool fault_now() {
  long k = g_fault_countdown.load();
  while (k > 0) {
    if (g_fault_countdown.compare_exchange_weak(k, k - 1)) return k == 1;
  }
  return false;
}
}  // namespace

cudaError_t dev_malloc(void** p, size_t bytes) {
  *p = nullptr;
  if (fault_now()) return cudaErrorMemoryAllocation;
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess) g_live_allocs++;
  else *p = nullptr;
  return e;
}
void dev_free(void* p) {
  if (!p) return;
  cudaFree(p);
  g_live_allocs--;
}
cudaError_t host_malloc_pinned(void** p, size_t bytes) {
  *p = nullptr;
  if (fault_now()) return cudaErrorMemoryAllocation;
  const cudaError_t e = cudaMallocHost(p, bytes);
  if (e == cudaSuccess) g_live_allocs++;
  else *p = nullptr;
  return e;
}
void host_free_pinned(void* p) {
  if (!p) return;
  cudaFreeHost(p);
  g_live_allocs--;
}

bool cuda_ok(tp_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  c->err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

template <typename T>
static T* dalloc(tp_ctx* c, long n) {
  if (n <= 0) n = 1;
  T* p = nullptr;
  if (dev_malloc(&p, sizeof(T) * (size_t)n) != cudaSuccess) {
    c->err = "cudaMalloc of " + std::to_string(sizeof(T) * n) + " bytes failed";
    return nullptr;
  }
  c->mem_bytes += (long)sizeof(T) * n;
  return p;
}


static tp_status check(tp_ctx* c) {
  if (!c->err.empty()) return TP_ERR_CUDA;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    c->err = cudaGetErrorString(e);
    return TP_ERR_CUDA;
  }
  return TP_OK;
}

static tp_status sync_check(tp_ctx* c) {
  cudaError_t e = cudaStreamSynchronize(c->s);
  if (e != cudaSuccess) {
    c->err = std::string("stream: ") + cudaGetErrorString(e);
    return TP_ERR_CUDA;
  }
  return check(c);
}

static double read_scalar(tp_ctx* c, int slot) {
  cudaMemcpyAsync(c->h_scal + slot, c->d_scal + slot, sizeof(double), cudaMemcpyDeviceToHost, c->s);
  cudaStreamSynchronize(c->s);
  return c->h_scal[slot];
}

static bool mixed(const tp_ctx* c) { return c->p.precision == TP_MIXED; }

// ---------------------------------------------------------------------------
// multigrid operator dispatch in precision T
template <typename T>
struct MG {
  T *r[TP_MAXL], *z[TP_MAXL], *d[TP_MAXL], *t[TP_MAXL], *invD[TP_MAXL], *st[TP_MAXL];
  const T* E;
};

template <typename T>
static void op_jacobi(tp_ctx* c, MG<T>& m, int l, const T* u, T* unew, int nr) {
  const T om = (T)c->p.omega;
  if (l == 0)
    fine_jacobi<T>(c, m.E, m.invD[0], m.r[0], u, unew, om, nr);
  else
    stencil_jacobi<T>(c, l, m.st[l], m.invD[l], m.r[l], u, unew, om, nr);
}
template <typename T>
static void op_resid(tp_ctx* c, MG<T>& m, int l, const T* u, T* d, int nr) {
  if (l == 0)
    fine_resid<T>(c, m.E, m.r[0], u, d, nr);
  else
    stencil_resid<T>(c, l, m.st[l], m.r[l], u, d, nr);
}

// coarsest correction in FP64 (rhs and solution through the double buffers
// of the coarsest level)
static void coarse_correct(tp_ctx* c, MG<double>& m, int lc, int nr) { coarse_solve(c, m.r[lc], m.z[lc], nr); }
static void coarse_correct(tp_ctx* c, MG<float>& m, int lc, int nr) {
  const long n = c->L[lc].ndof;
  cast_f2d(c, n * nr, m.r[lc], c->mg_r[lc]);
  coarse_solve(c, c->mg_r[lc], c->mg_z[lc], nr);
  cast_d2f(c, n * nr, c->mg_z[lc], m.z[lc]);
}

// One V(nswp, nswp) cycle from m.r[l] (stencil_solvers.c:129-252); the
// result lands in m.z[l]. The pre-smoothing starts from z = 0, whose first
// sweep needs no operator application (K*0 = 0, also at fixed DOFs). nr
// load cases go through together, each level's vectors holding nr columns.
template <typename T>
static void vcycle(tp_ctx* c, MG<T>& m, int l, int nr) {
  const long nd = c->L[l].ndof;
  const int nswp = c->p.nswp;
  // the sweeps alternate buffers 2*nswp - 1 times: start in t so z ends in z
  T* za = (nswp > 0) ? m.t[l] : m.z[l];
  T* zb = (nswp > 0) ? m.z[l] : m.t[l];
  if (nswp > 0) {
    vscale<T>(c, nd, m.invD[l], m.r[l], za, (T)c->p.omega, nr);
    for (int s = 1; s < nswp; s++) {
      op_jacobi<T>(c, m, l, za, zb, nr);
      std::swap(za, zb);
    }
  } else {
    cudaMemsetAsync(za, 0, sizeof(T) * nd * nr, c->s);
  }
  op_resid<T>(c, m, l, za, m.d[l], nr);
  restrict_fw<T>(c, l, m.d[l], m.r[l + 1], nr);
  if (l + 2 == c->nl)
    coarse_correct(c, m, l + 1, nr);
  else
    vcycle<T>(c, m, l + 1, nr);
  prolong_add<T>(c, l, m.z[l + 1], za, nr);
  for (int s = 0; s < nswp; s++) {
    op_jacobi<T>(c, m, l, za, zb, nr);
    std::swap(za, zb);
  }
}

static MG<double> mg_double(tp_ctx* c) {
  MG<double> m;
  for (int l = 0; l < c->nl; l++) {
    m.r[l] = c->mg_r[l];
    m.z[l] = c->mg_z[l];
    m.d[l] = c->mg_d[l];
    m.t[l] = c->mg_t[l];
    m.invD[l] = c->invD[l];
    m.st[l] = c->st[l];
  }
  m.E = c->d_E;
  return m;
}
static MG<float> mg_float(tp_ctx* c) {
  MG<float> m;
  for (int l = 0; l < c->nl; l++) {
    m.r[l] = c->mgf_r[l];
    m.z[l] = c->mgf_z[l];
    m.d[l] = c->mgf_d[l];
    m.t[l] = c->mgf_t[l];
    m.invD[l] = c->invDf[l];
    m.st[l] = c->stf[l];
  }
  m.E = c->d_Ef;
  return m;
}

// z = M^{-1} r on level 0 (FP64 in and out), nr columns
static void precondition(tp_ctx* c, const double* r, double* z, int nr = 1) {
  const long n = c->L[0].ndof;
  if (!mixed(c)) {
    MG<double> m = mg_double(c);
    m.r[0] = const_cast<double*>(r);  // read only on level 0
    m.z[0] = z;
    vcycle<double>(c, m, 0, nr);
  } else {
    MG<float> m = mg_float(c);
    cast_d2f(c, n * nr, r, m.r[0]);
    vcycle<float>(c, m, 0, nr);
    cast_f2d(c, n * nr, m.z[0], z);
  }
}

// ---------------------------------------------------------------------------
// Enqueues the assembly of every level and the coarse factorisation; the
// factor's status word is checked by assemble_status (or, in the design
// iteration without host round trips, read once at the iteration's end).
static void assemble_enqueue(tp_ctx* c) {
  compute_E(c);
  fine_inv_diag(c, c->invD[0]);
  if (mixed(c)) cast_d2f(c, c->L[0].ndof, c->invD[0], c->invDf[0]);
  for (int l = 1; l < c->nl; l++) {
    const bool coarsest = (l == c->nl - 1);
    if (!mixed(c) || coarsest) {
      assemble_stencil<double>(c, l, c->d_E, c->d_ke[l], c->st[l], c->invD[l]);
    }
    if (mixed(c) && !coarsest) {
      assemble_stencil<float>(c, l, c->d_Ef, c->d_kef[l], c->stf[l], c->invD[l]);
      cast_d2f(c, c->L[l].ndof, c->invD[l], c->invDf[l]);
    }
    if (mixed(c) && coarsest) cast_d2f(c, c->L[l].ndof, c->invD[l], c->invDf[l]);
  }
  coarse_assemble(c);
  coarse_factor(c);
  for (int l = 0; l < TP_MAXL; l++) c->st_sub_valid[l] = false;
}

// the coarse factor's status word `info` -> the assembly's status
static tp_status assemble_status(tp_ctx* c, int info) {
  // the operators count as assembled only with a usable coarse factor: after
  // a timeout or a non-positive pivot every later call assembles again (and
  // reports the same status) instead of solving with the failed factor
  c->assembled = false;
  if (info & kCoarseWaitGaveUp) {
    c->note = "coarse Cholesky: a bounded wait gave up";
    return TP_ERR_TIMEOUT;
  }
  if (info != 0) {
    c->note = "coarse Cholesky: non-positive pivot at column " + std::to_string(info - 1);
    return TP_ERR_NOT_SPD;
  }
  c->assembled = true;
  return TP_OK;
}

static tp_status assemble(tp_ctx* c) {
  if (!c->assemble_pending) assemble_enqueue(c);
  c->assemble_pending = false;
  tp_status st = check(c);
  if (st != TP_OK) return st;
  cudaMemcpyAsync(c->h_info, c->coarse.info, sizeof(int), cudaMemcpyDeviceToHost, c->s);
  st = sync_check(c);
  if (st != TP_OK) return st;
  return assemble_status(c, *c->h_info);
}

// PCG set-up: r = b - K u, |b|^2 per column, converged marks cleared; the
// mixed form's first V-cycle input (float) r
void pcg_prologue(tp_ctx* c, const double* b, const double* u, int nr) {
  const long n = c->L[0].ndof;
  int nb = 0;
  fine_resid<double>(c, c->d_E, b, u, c->d_r, nr);
  if (mixed(c)) cast_d2f(c, n * nr, c->d_r, c->mgf_r[0]);
  dot_partials(c, n, b, b, &nb, nr);
  finish_sum(c, nb, S_BNORM2, 0, nr);
  cg_reset(c, nr);
}

// One PCG iteration over nr columns. iter >= 0 is the host's iteration
// index; iter = -1 takes it from the device counter (the captured loop).
// The mixed form's V-cycle reads r as the float copy that the prologue and
// the last r update wrote, and the dot and the p update read its float
// output directly (widened exactly), so neither cast pass runs here.
void pcg_iteration(tp_ctx* c, double* u, int iter, int nr) {
  const long n = c->L[0].ndof;
  double *r = c->d_r, *z = c->d_z, *p = c->d_p, *q = c->d_q;
  int nb = 0;
  const int first = iter < 0 ? -1 : (iter == 0);
  if (mixed(c)) {
    MG<float> m = mg_float(c);
    vcycle<float>(c, m, 0, nr);
    dot_partials(c, n, r, (const float*)m.z[0], &nb, nr);
    finish_sum(c, nb, S_RHO, 0, nr);
    if (iter != 0) cg_scalars(c, 0, nr);
    cg_pupdate(c, n, (const float*)m.z[0], p, first, nr);
  } else {
    precondition(c, r, z, nr);
    dot_partials(c, n, r, (const double*)z, &nb, nr);
    finish_sum(c, nb, S_RHO, 0, nr);
    if (iter != 0) cg_scalars(c, 0, nr);
    cg_pupdate(c, n, (const double*)z, p, first, nr);
  }
  finish_sum(c, fine_apply_dot<double>(c, c->d_E, p, q, nr), S_DPR, 0, nr);
  cg_scalars(c, 1, nr);
  cg_xr_update(c, n, u, r, p, q, &nb, nr, mixed(c) ? c->mgf_r[0] : nullptr);
  finish_sum(c, nb, S_RNORM2, 0, nr);
  cg_scalars(c, 2, nr, c->p.cgtol, iter);
}

// PCG (stencil_solvers.c:259-397) in FP64 for K u = b, warm start from u,
// host-driven: the largest relres of the nr columns is read back once per
// iteration, as the reference reads its residual norm.
static tp_status pcg(tp_ctx* c, const double* b, double* u, int* iters, double* relres, int nr = 1) {
  pcg_prologue(c, b, u, nr);
  const double tol = c->p.cgtol;
  int it = 0;
  double rr = 0.0;
  bool converged = false;
  for (int iter = 0; iter < c->p.cgmax; iter++) {
    pcg_iteration(c, u, iter, nr);
    tp_status st = check(c);
    if (st != TP_OK) return st;
    rr = read_scalar(c, S_MAXRR);
    it = iter;
    if (!std::isfinite(rr)) {
      *iters = it;
      *relres = rr;
      if (coarse_status(c) != TP_OK) return TP_ERR_TIMEOUT;
      c->note = "CG: non-finite residual";
      return TP_ERR_NONFINITE;
    }
    if (rr < tol) {
      converged = true;
      break;
    }
  }
  *iters = it;
  *relres = (double)(float)rr;  // the reference reports it through a float
  tp_status st = check(c);
  if (st != TP_OK) return st;
  st = coarse_status(c);
  if (st != TP_OK) return st;
  return converged ? TP_OK : TP_ERR_NOT_CONVERGED;
}

}  // namespace tp

// ===========================================================================
extern "C" {

void tp_default_params(tp_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->nelx = 12 * 4;
  p->nely = 6 * 4;
  p->nelz = 6 * 4;
  p->nl = 4;
  p->volfrac = (double)0.2f;
  p->rmin = 1.5;
  p->cgtol = (double)1e-5f;
  p->cgmax = 1000;
  p->nswp = 4;
  p->omega = 0.6;
  p->precision = TP_FP64;
  p->nrhs = 1;
  p->device = 0;
}

const char* tp_status_string(tp_status s) {
  switch (s) {
    case TP_OK: return "ok";
    case TP_ERR_ARG: return "invalid argument";
    case TP_ERR_CUDA: return "CUDA error";
    case TP_ERR_ALLOC: return "allocation failed";
    case TP_ERR_NOT_SPD: return "coarse matrix not positive definite";
    case TP_ERR_NOT_CONVERGED: return "CG did not converge";
    case TP_ERR_NONFINITE: return "non-finite value";
    case TP_ERR_TIMEOUT: return "device wait timed out";
    case TP_ERR_STATE: return "call out of order";
  }
  return "unknown status";
}

const char* tp_error_message(const tp_ctx* c) {
  if (!c) return "null context";
  return c->err.empty() ? c->note.c_str() : c->err.c_str();
}

long tp_ndof(const tp_ctx* c, int level) {
  if (!c || level < 0 || level >= c->nl) return -1;
  return c->L[level].ndof;
}
long tp_nelem(const tp_ctx* c) { return c ? (long)c->L[0].ex * c->L[0].ey * c->L[0].ez : -1; }
long tp_device_bytes(const tp_ctx* c) { return c ? c->mem_bytes : -1; }

long tp_fault_alloc(long k) {
  tp::g_fault_countdown.store(k > 0 ? k : 0);
  return tp::g_live_allocs.load();
}

tp_status tp_sync(tp_ctx* c) {
  if (!c) return TP_ERR_ARG;
  return sync_check(c);
}

// frees everything the context holds and clears the pointers, so that a
// second call (tp_destroy of a context whose tp_create failed) frees nothing
static void destroy_buffers(tp_ctx* c) {
  auto F = [](auto*& p) {
    dev_free(p);
    p = nullptr;
  };
  for (int l = 0; l < TP_MAXL; l++) {
    F(c->d_ke[l]); F(c->d_kef[l]); F(c->d_mgc[l]); F(c->d_mgi[l]);
    F(c->mg_r[l]); F(c->mg_z[l]); F(c->mg_d[l]); F(c->mg_t[l]);
    F(c->mgf_r[l]); F(c->mgf_z[l]); F(c->mgf_d[l]); F(c->mgf_t[l]);
    F(c->invD[l]); F(c->invDf[l]); F(c->st[l]); F(c->stf[l]); F(c->st_sub[l]);
  }
  F(c->d_x); F(c->d_xphys); F(c->d_xnew); F(c->d_dc); F(c->d_dv); F(c->d_hs); F(c->d_ocb);
  F(c->d_E); F(c->d_Ef); F(c->d_F); F(c->d_U);
  F(c->d_r); F(c->d_z); F(c->d_p); F(c->d_q);
  F(c->d_red); F(c->d_scal); F(c->d_flag); F(c->scratch_invD); F(c->d_fw); F(c->d_mom);
  host_free_pinned(c->h_scal);
  host_free_pinned(c->h_info);
  c->h_scal = nullptr;
  c->h_info = nullptr;
  for (auto& e : c->it_ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  graph_free(c);
  oc_graph_free(c);
  coarse_free(c);
  prof_destroy(c);
}

tp_status tp_create(const tp_params* p, tp_ctx** out) {
  if (!p || !out) return TP_ERR_ARG;
  *out = nullptr;
  if (p->nl < 2 || p->nl > TP_MAXL || p->nelx < 1 || p->nely < 1 || p->nelz < 1) return TP_ERR_ARG;
  const int q = 1 << (p->nl - 1);
  if (p->nelx % q || p->nely % q || p->nelz % q) return TP_ERR_ARG;
  if (p->nrhs < 1 || p->nrhs > 16 || p->cgmax < 1 || p->nswp < 0 || !(p->rmin > 0)) return TP_ERR_ARG;
  if (p->precision != TP_FP64 && p->precision != TP_MIXED) return TP_ERR_ARG;

  tp_ctx* c = new tp_ctx();
  c->p = *p;
  c->nl = p->nl;
  c->device = p->device;
  if (!cuda_ok(c, cudaSetDevice(p->device), "cudaSetDevice") ||
      !cuda_ok(c, cudaStreamCreateWithFlags(&c->s, cudaStreamDefault), "stream")) {
    *out = c;
    return TP_ERR_CUDA;
  }
  for (int l = 0; l < c->nl; l++) c->L[l] = make_level(p->nelx, p->nely, p->nelz, l);
  const Level& L0 = c->L[0];
  const long ne = (long)L0.ex * L0.ey * L0.ez;

  bool ok = true;
  // element stiffness tables
  std::vector<double> ke0;
  long mom_n = 0;
  for (int l = 0; l < c->nl && ok; l++) {
    const long nk = 576L << (3 * l);
    std::vector<double> ke(nk);
    element_matrix_tables(0.3, l, ke.data());
    std::vector<float> kf(ke.begin(), ke.end());
    ok = (c->d_ke[l] = dalloc<double>(c, nk)) && (c->d_kef[l] = dalloc<float>(c, nk));
    if (ok) {
      cudaMemcpy(c->d_ke[l], ke.data(), sizeof(double) * nk, cudaMemcpyHostToDevice);
      cudaMemcpy(c->d_kef[l], kf.data(), sizeof(float) * nk, cudaMemcpyHostToDevice);
    }
    if (l >= 2 && ok) {  // element matrices from moments where they reproduce the tables
      std::vector<int> off, pidx;
      std::vector<double> coef;
      if (moment_tables(ke0.data(), ke.data(), l, off, pidx, coef)) {
        const int nnz = (int)coef.size();
        std::vector<int> ints(pidx);
        ints.insert(ints.end(), off.begin(), off.end());
        ok = (c->d_mgc[l] = dalloc<double>(c, nnz)) && (c->d_mgi[l] = dalloc<int>(c, (long)ints.size()));
        if (ok) {
          cudaMemcpy(c->d_mgc[l], coef.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice);
          cudaMemcpy(c->d_mgi[l], ints.data(), sizeof(int) * ints.size(), cudaMemcpyHostToDevice);
          c->mg_nnz[l] = nnz;
          mom_n = std::max(mom_n, 27L * c->L[l].ex * c->L[l].ey * c->L[l].ez);
        }
      }
    }
    if (l == 0) {
      ke0 = ke;
      set_fine_ke(ke.data());
      set_design_ke(ke.data());
      double kz45[45];
      c->ec_ok = set_fine_kz(ke.data(), kz45);
      if (c->ec_ok) set_design_kz(kz45);
    }
  }
  const bool mx = p->precision == TP_MIXED;
  const long nv = L0.ndof * p->nrhs;
  ok = ok && (c->d_x = dalloc<double>(c, ne)) && (c->d_xphys = dalloc<double>(c, ne)) &&
       (c->d_xnew = dalloc<double>(c, ne)) && (c->d_dc = dalloc<double>(c, ne)) &&
       (c->d_dv = dalloc<double>(c, ne)) && (c->d_hs = dalloc<double>(c, ne)) &&
       (c->d_ocb = dalloc<double>(c, 3 * ne)) && ((c->ocb_n = ne) > 0) &&
       (c->d_E = dalloc<double>(c, ne)) && (c->d_Ef = dalloc<float>(c, ne)) &&
       (c->d_F = dalloc<double>(c, nv)) && (c->d_U = dalloc<double>(c, nv)) &&
       (c->d_r = dalloc<double>(c, nv)) && (c->d_z = dalloc<double>(c, nv)) &&
       (c->d_p = dalloc<double>(c, nv)) && (c->d_q = dalloc<double>(c, nv));
  if (ok && mom_n > 0) ok = (c->d_mom = dalloc<double>(c, mom_n)) != nullptr;
  // every solver vector holds one column per load case
  for (int l = 0; l < c->nl && ok; l++) {
    const long nd = c->L[l].ndof, ndr = nd * p->nrhs;
    const bool coarsest = l == c->nl - 1;
    ok = (c->invD[l] = dalloc<double>(c, nd)) != nullptr;
    if (ok && (!mx || coarsest))
      ok = (c->mg_r[l] = dalloc<double>(c, ndr)) && (c->mg_z[l] = dalloc<double>(c, ndr)) &&
           (c->mg_d[l] = dalloc<double>(c, ndr)) && (c->mg_t[l] = dalloc<double>(c, ndr));
    if (ok && mx)
      ok = (c->mgf_r[l] = dalloc<float>(c, ndr)) && (c->mgf_z[l] = dalloc<float>(c, ndr)) &&
           (c->mgf_d[l] = dalloc<float>(c, ndr)) && (c->mgf_t[l] = dalloc<float>(c, ndr)) &&
           (c->invDf[l] = dalloc<float>(c, nd));
    if (ok && l >= 1 && (!mx || coarsest))
      ok = (c->st[l] = dalloc<double>(c, kStencilCoef * c->L[l].nnodes)) != nullptr;
    if (ok && l >= 1 && mx && !coarsest)
      ok = (c->stf[l] = dalloc<float>(c, kStencilCoef * c->L[l].nnodes)) != nullptr;
  }
  const long red = std::max<long>(1 << 16, (long)fine_blocks(c) * p->nrhs);
  const long nscal = (long)S_COUNT * p->nrhs;
  ok = ok && (c->d_red = dalloc<double>(c, red)) && (c->d_scal = dalloc<double>(c, nscal)) &&
       (c->d_flag = dalloc<int>(c, 4));
  if (ok) ok = cuda_ok(c, host_malloc_pinned((void**)&c->h_scal, sizeof(double) * nscal), "cudaMallocHost");
  if (ok) ok = cuda_ok(c, host_malloc_pinned((void**)&c->h_info, sizeof(int) * 4), "cudaMallocHost");
  if (ok) ok = cuda_ok(c, cudaEventCreate(&c->it_ev[0]), "cudaEventCreate") &&
               cuda_ok(c, cudaEventCreate(&c->it_ev[1]), "cudaEventCreate");
  if (ok) {
    coarse_alloc(c);
    ok = c->coarse.band && c->coarse.dinv && c->coarse.dinvT && c->coarse.lrow && c->coarse.vec && c->coarse.info &&
         c->coarse.linv && !c->coarse.alloc_failed;
    if (!ok) c->err = "coarse solver allocation failed";
  }
  if (!ok) {
    destroy_buffers(c);
    *out = c;
    return TP_ERR_ALLOC;
  }
  cudaMemsetAsync(c->d_scal, 0, sizeof(double) * nscal, c->s);
  cudaMemsetAsync(c->d_U, 0, sizeof(double) * nv, c->s);
  cudaMemsetAsync(c->d_F, 0, sizeof(double) * nv, c->s);
  for (int l = 0; l < c->nl; l++) {
    if (c->mg_z[l]) cudaMemsetAsync(c->mg_z[l], 0, sizeof(double) * c->L[l].ndof * p->nrhs, c->s);
    if (c->mgf_z[l]) cudaMemsetAsync(c->mgf_z[l], 0, sizeof(float) * c->L[l].ndof * p->nrhs, c->s);
  }
  {
    std::vector<double> F(L0.ndof);
    cantilever_load(L0, F.data());
    cudaMemcpyAsync(c->d_F, F.data(), sizeof(double) * L0.ndof, cudaMemcpyHostToDevice, c->s);
    cudaStreamSynchronize(c->s);
  }
  filter_hs(c, c->d_hs);
  if (!c->d_fw) {
    destroy_buffers(c);
    *out = c;
    return TP_ERR_ALLOC;
  }
  ec_default_plans(c);
  c->fine_ds = c->coarse.ds = mixed(c) ? 1 : 0;
  tp_status st = sync_check(c);
  *out = c;
  if (st != TP_OK) return st;
  return tp_init_design(c);
}

void tp_destroy(tp_ctx* c) {
  if (!c) return;
  if (c->s) cudaStreamSynchronize(c->s);
  destroy_buffers(c);
  if (c->s) cudaStreamDestroy(c->s);
  delete c;
}

double* tp_field_ptr(tp_ctx* c, tp_field f) {
  if (!c) return nullptr;
  switch (f) {
    case TP_FIELD_X: return c->d_x;
    case TP_FIELD_XPHYS: return c->d_xphys;
    case TP_FIELD_XNEW: return c->d_xnew;
    case TP_FIELD_DC: return c->d_dc;
    case TP_FIELD_DV: return c->d_dv;
    case TP_FIELD_F: return c->d_F;
    case TP_FIELD_U: return c->d_U;
  }
  return nullptr;
}

static long field_count(const tp_ctx* c, tp_field f) {
  if (f == TP_FIELD_F || f == TP_FIELD_U) return c->L[0].ndof * c->p.nrhs;
  return tp_nelem(c);
}

tp_status tp_field_written(tp_ctx* c, tp_field f) {
  if (!c || !tp_field_ptr(c, f)) return TP_ERR_ARG;
  if (f == TP_FIELD_XPHYS) {
    c->assembled = false;
    c->assemble_pending = false;
    for (int l = 0; l < TP_MAXL; l++) c->st_sub_valid[l] = false;
  }
  return TP_OK;
}

tp_status tp_upload(tp_ctx* c, tp_field f, const double* host, long count) {
  if (!c || !host || count != field_count(c, f)) return TP_ERR_ARG;
  double* d = tp_field_ptr(c, f);
  if (!d) return TP_ERR_ARG;
  if (!cuda_ok(c, cudaMemcpyAsync(d, host, sizeof(double) * count, cudaMemcpyHostToDevice, c->s), "upload"))
    return TP_ERR_CUDA;
  tp_field_written(c, f);
  return sync_check(c);
}

tp_status tp_download(tp_ctx* c, tp_field f, double* host, long count) {
  if (!c || !host || count != field_count(c, f)) return TP_ERR_ARG;
  double* d = tp_field_ptr(c, f);
  if (!d) return TP_ERR_ARG;
  if (!cuda_ok(c, cudaMemcpyAsync(host, d, sizeof(double) * count, cudaMemcpyDeviceToHost, c->s), "download"))
    return TP_ERR_CUDA;
  return sync_check(c);
}

tp_status tp_element_matrices(const tp_ctx* c, int level, double* out_host) {
  if (!c || level < 0 || level >= c->nl || !out_host) return TP_ERR_ARG;
  element_matrix_tables(0.3, level, out_host);
  return TP_OK;
}

tp_status tp_element_matrix_tables(int level, double nu, double* out_host) {
  if (level < 0 || level >= TP_MAXL || !out_host) return TP_ERR_ARG;
  element_matrix_tables(nu, level, out_host);
  return TP_OK;
}

tp_status tp_reference_load(int nelx, int nely, int nelz, double* F_host) {
  if (nelx < 1 || nely < 1 || nelz < 1 || !F_host) return TP_ERR_ARG;
  cantilever_load(make_level(nelx, nely, nelz, 0), F_host);
  return TP_OK;
}

tp_status tp_fixed_dofs(const tp_ctx* c, int level, long* out_host, long* count) {
  if (!c || level < 0 || level >= c->nl) return TP_ERR_ARG;
  const Level& L = c->L[level];
  long q = 0;
  for (int k = 0; k < L.nz; k++) {
    for (int j = 0; j < L.lim; j++)
      for (int d = 0; d < 3; d++, q++)
        if (out_host) out_host[q] = 3L * ((long)k * L.ny + j) + d;
    for (int j = L.ny - L.lim; j < L.ny; j++)
      for (int d = 0; d < 3; d++, q++)
        if (out_host) out_host[q] = 3L * ((long)k * L.ny + j) + d;
  }
  if (count) *count = q;
  return TP_OK;
}

tp_status tp_assemble(tp_ctx* c) {
  if (!c) return TP_ERR_ARG;
  return assemble(c);
}

// The assembly enqueued without a wait: the caller's host work (copies on
// streams of its own) overlaps it; the next tp_assemble completes it (one
// synchronisation, the factor's status) unless xPhys or the solver's set-up
// changed in between, which discards it.
tp_status tp_assemble_async(tp_ctx* c) {
  if (!c) return TP_ERR_ARG;
  if (!c->assemble_pending) assemble_enqueue(c);
  c->assemble_pending = true;
  return check(c);
}

tp_status tp_apply(tp_ctx* c, int level, const double* in, double* out) {
  if (!c || level < 0 || level >= c->nl || !in || !out) return TP_ERR_ARG;
  if (level == 0) {
    compute_E(c);
    fine_apply<double>(c, c->d_E, in, out);
  } else {
    if (!c->assembled || !c->st[level]) return TP_ERR_STATE;
    stencil_apply<double>(c, level, c->st[level], in, out);
  }
  return sync_check(c);
}

tp_status tp_apply_f32(tp_ctx* c, int level, const float* in, float* out) {
  if (!c || level < 0 || level >= c->nl || !in || !out) return TP_ERR_ARG;
  if (level == 0) {
    compute_E(c);
    fine_apply<float>(c, c->d_Ef, in, out);
  } else {
    if (!c->assembled || !c->stf[level]) return TP_ERR_STATE;
    stencil_apply<float>(c, level, c->stf[level], in, out);
  }
  return sync_check(c);
}

tp_status tp_inv_diag(tp_ctx* c, int level, double* out) {
  if (!c || level < 0 || level >= c->nl || !out) return TP_ERR_ARG;
  if (!c->assembled) {
    tp_status st = assemble(c);
    if (st != TP_OK) return st;
  }
  cudaMemcpyAsync(out, c->invD[level], sizeof(double) * c->L[level].ndof, cudaMemcpyDeviceToDevice, c->s);
  return sync_check(c);
}

tp_status tp_restrict(tp_ctx* c, int level, const double* fine, double* coarse) {
  if (!c || level < 0 || level + 1 >= c->nl || !fine || !coarse) return TP_ERR_ARG;
  restrict_fw<double>(c, level, fine, coarse);
  return sync_check(c);
}

tp_status tp_prolong(tp_ctx* c, int level, const double* coarse, double* fine) {
  if (!c || level < 0 || level + 1 >= c->nl || !fine || !coarse) return TP_ERR_ARG;
  prolong_set<double>(c, level, coarse, fine);
  return sync_check(c);
}

tp_status tp_smooth(tp_ctx* c, int level, int nswp, double omega, const double* b, double* u) {
  if (!c || level < 0 || level >= c->nl || !b || !u || nswp < 0) return TP_ERR_ARG;
  if (!c->assembled) {
    tp_status st = assemble(c);
    if (st != TP_OK) return st;
  }
  if (level >= 1 && !c->st[level]) return TP_ERR_STATE;
  const long nd = c->L[level].ndof;
  double* t = c->d_q;  // level-0 sized scratch
  double* cur = u;
  double* nxt = t;
  for (int s = 0; s < nswp; s++) {
    if (level == 0)
      fine_jacobi<double>(c, c->d_E, c->invD[0], b, cur, nxt, omega);
    else
      stencil_jacobi<double>(c, level, c->st[level], c->invD[level], b, cur, nxt, omega);
    std::swap(cur, nxt);
  }
  if (cur != u) cudaMemcpyAsync(u, cur, sizeof(double) * nd, cudaMemcpyDeviceToDevice, c->s);
  tp_status st = sync_check(c);
  return st != TP_OK ? st : coarse_status(c);
}

tp_status tp_coarse_solve(tp_ctx* c, const double* rhs, double* x) {
  if (!c || !rhs || !x) return TP_ERR_ARG;
  if (!c->assembled) {
    tp_status st = assemble(c);
    if (st != TP_OK) return st;
  }
  coarse_solve(c, rhs, x);
  tp_status st = sync_check(c);
  return st != TP_OK ? st : coarse_status(c);
}

tp_status tp_vcycle(tp_ctx* c, const double* r, double* z) {
  if (!c || !r || !z) return TP_ERR_ARG;
  if (!c->assembled) {
    tp_status st = assemble(c);
    if (st != TP_OK) return st;
  }
  precondition(c, r, z);
  tp_status st = sync_check(c);
  return st != TP_OK ? st : coarse_status(c);
}

tp_status tp_solve(tp_ctx* c, int* iters, double* relres) {
  if (!c) return TP_ERR_ARG;
  tp_status st = assemble(c);
  if (st != TP_OK) return st;
  int it = 0;
  double rr = 0;
  // graph_solve: 0 the captured loop for several loads, host-driven for one;
  // 1 always the captured loop; 2 always host-driven
  const bool graph = c->graph_solve == 1 || (c->graph_solve == 0 && c->p.nrhs > 1);
  st = graph ? pcg_graph(c, &it, &rr) : pcg(c, c->d_F, c->d_U, &it, &rr, c->p.nrhs);
  if (iters) *iters = it;
  if (relres) *relres = rr;
  return st;
}

tp_status tp_solve_rhs(tp_ctx* c, const double* rhs, double* sol, int* iters, double* relres) {
  if (!c || !rhs || !sol) return TP_ERR_ARG;
  if (!c->assembled) {
    tp_status st = assemble(c);
    if (st != TP_OK) return st;
  }
  int it = 0;
  double rr = 0;
  // the context's own F and U (the drop-in layer's state solve): the captured
  // CG loop, one host wait per solve instead of one per iteration (the same
  // kernels and decisions); graph_solve 2 forces the host-driven loop
  const bool graph = rhs == c->d_F && sol == c->d_U && c->p.nrhs == 1 && c->graph_solve != 2;
  tp_status st = graph ? pcg_graph(c, &it, &rr) : pcg(c, rhs, sol, &it, &rr);
  if (iters) *iters = it;
  if (relres) *relres = rr;
  return st;
}

tp_status tp_compliance(tp_ctx* c, double* c_out) {
  if (!c) return TP_ERR_ARG;
  int nb = 0;
  compliance(c, c->d_U, c->d_dc, &nb, c->p.nrhs);
  finish_sum(c, nb, S_C, 0);
  tp_status st = check(c);
  if (st != TP_OK) return st;
  const double v = read_scalar(c, S_C);
  if (c_out) *c_out = v;
  return sync_check(c);
}

tp_status tp_element_sensitivity(tp_ctx* c, const double* u, const double* w, double* out) {
  if (!c || !u || !w || !out) return TP_ERR_ARG;
  element_sens(c, u, w, out);
  return sync_check(c);
}

tp_status tp_filter(tp_ctx* c, const double* in, double* out) {
  if (!c || !in || !out || in == out) return TP_ERR_ARG;
  filter_fwd(c, in, out);
  return sync_check(c);
}

tp_status tp_filter_T(tp_ctx* c, double* v) {
  if (!c || !v) return TP_ERR_ARG;
  filter_adj(c, v, c->d_xnew);
  return sync_check(c);
}

tp_status tp_volume(tp_ctx* c, double* vol) {
  if (!c || !vol) return TP_ERR_ARG;
  int nb = 0;
  volume_partials(c, c->d_xphys, &nb);
  finish_sum(c, nb, S_VOL, 0);
  tp_status st = check(c);
  if (st != TP_OK) return st;
  *vol = read_scalar(c, S_VOL) / (double)tp_nelem(c);
  return sync_check(c);
}

tp_status tp_oc_update(tp_ctx* c, double g, double* change) {
  if (!c) return TP_ERR_ARG;
  if (oc_update(c, g) != 0) {
    c->note = "OC bisection did not terminate";
    return TP_ERR_TIMEOUT;
  }
  tp_status st = check(c);
  if (st != TP_OK) return st;
  const double ch = read_scalar(c, S_CHANGE);
  if (change) *change = (double)(float)ch;
  return sync_check(c);
}

// x = xPhys = volfrac, dv = H^T(1/Hs), U = 0 (stencil_optimization.c:97-129)
__global__ void fill_kernel(long n, double* a, double v) {
  const long i = blockIdx.x * 256L + threadIdx.x;
  if (i < n) a[i] = v;
}

tp_status tp_init_design(tp_ctx* c) {
  if (!c) return TP_ERR_ARG;
  const long ne = tp_nelem(c);
  fill_kernel<<<grid_for(ne, 256), 256, 0, c->s>>>(ne, c->d_x, c->p.volfrac);
  fill_kernel<<<grid_for(ne, 256), 256, 0, c->s>>>(ne, c->d_xphys, c->p.volfrac);
  fill_kernel<<<grid_for(ne, 256), 256, 0, c->s>>>(ne, c->d_dv, 1.0);
  filter_adj(c, c->d_dv, c->d_xnew);
  cudaMemsetAsync(c->d_U, 0, sizeof(double) * c->L[0].ndof * c->p.nrhs, c->s);
  c->assembled = false;
  c->assemble_pending = false;
  return sync_check(c);
}

// One design iteration with the host in the loop, as the reference drives it:
// the CG loop reads the residual each iteration (for one load), the volume is
// read before the OC update and the bisection is checked every 24 steps.
static tp_status design_iteration_host(tp_ctx* c, tp_iter_info* info) {
  cudaEventRecord(c->it_ev[0], c->s);
  int it = 0;
  double rr = 0;
  tp_status st = tp_solve(c, &it, &rr);
  if (st != TP_OK && st != TP_ERR_NOT_CONVERGED) return st;
  double vol = 0;
  st = tp_volume(c, &vol);
  if (st != TP_OK) return st;
  int nb = 0;
  compliance(c, c->d_U, c->d_dc, &nb, c->p.nrhs);
  finish_sum(c, nb, S_C, 0);
  filter_adj(c, c->d_dc, c->d_xnew);
  const double g = vol - c->p.volfrac;
  if (oc_update(c, g) != 0) {
    c->note = "OC bisection did not terminate";
    return TP_ERR_TIMEOUT;
  }
  filter_fwd(c, c->d_x, c->d_xphys);
  c->assembled = false;
  c->assemble_pending = false;
  cudaEventRecord(c->it_ev[1], c->s);
  cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, c->s);
  st = sync_check(c);
  if (st != TP_OK) return st;
  float ms = 0;
  cudaEventElapsedTime(&ms, c->it_ev[0], c->it_ev[1]);
  if (info) {
    info->c = c->h_scal[S_C];
    info->vol = vol;
    info->change = (double)(float)c->h_scal[S_CHANGE];
    info->cgiters = it;
    info->relres = rr;
    info->ms = ms;
  }
  return TP_OK;
}

// The same iteration with one host wait, at its end: assembly and factor,
// the CG loop (one graph launch), volume, constraint value, compliance,
// filter adjoint, the OC bisection (one graph launch), change and filter are
// all enqueued first; the scalars and the coarse factor's status word come
// back together and are checked then. The arithmetic and its order are the
// host-driven form's, so both give the same bits.
static tp_status design_iteration_device(tp_ctx* c, tp_iter_info* info) {
  cudaEventRecord(c->it_ev[0], c->s);
  assemble_enqueue(c);
  tp_status st = pcg_graph_enqueue(c);
  if (st != TP_OK) return st;
  int nb = 0;
  volume_partials(c, c->d_xphys, &nb);
  finish_sum(c, nb, S_VOL, 0);
  constraint_from_volume(c);
  compliance(c, c->d_U, c->d_dc, &nb, c->p.nrhs);
  finish_sum(c, nb, S_C, 0);
  filter_adj(c, c->d_dc, c->d_xnew);
  if (!oc_update_graph(c)) {
    c->err = "OC bisection graph: capture or instantiation failed";
    return TP_ERR_CUDA;
  }
  filter_fwd(c, c->d_x, c->d_xphys);
  cudaEventRecord(c->it_ev[1], c->s);
  cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(double) * S_COUNT * c->p.nrhs, cudaMemcpyDeviceToHost, c->s);
  cudaMemcpyAsync(c->h_info, c->coarse.info, sizeof(int), cudaMemcpyDeviceToHost, c->s);
  st = sync_check(c);
  if (st != TP_OK) return st;
  // the factor's status first: a failed factor makes every later value moot
  st = assemble_status(c, *c->h_info);
  c->assembled = false;  // xPhys has changed
  c->assemble_pending = false;
  if (st != TP_OK) return st;
  int it = 0;
  double rr = 0;
  st = pcg_graph_status(c, &it, &rr);
  if (st != TP_OK && st != TP_ERR_NOT_CONVERGED) return st;
  if (c->h_scal[S_OCDONE] == 0.0) {
    c->note = "OC bisection did not terminate";
    return TP_ERR_TIMEOUT;
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, c->it_ev[0], c->it_ev[1]);
  if (info) {
    info->c = c->h_scal[S_C];
    info->vol = c->h_scal[S_VOL] / (double)tp_nelem(c);
    info->change = (double)(float)c->h_scal[S_CHANGE];
    info->cgiters = it;
    info->relres = rr;
    info->ms = ms;
  }
  return TP_OK;
}

tp_status tp_design_iteration(tp_ctx* c, tp_iter_info* info) {
  if (!c) return TP_ERR_ARG;
  // per-kernel timing needs every kernel launched from the host
  if (c->device_loop && !c->prof) return design_iteration_device(c, info);
  return design_iteration_host(c, info);
}

tp_status tp_set_device_loop(tp_ctx* c, int on) {
  if (!c || on < 0 || on > 1) return TP_ERR_ARG;
  c->device_loop = on;
  return TP_OK;
}

tp_status tp_run(tp_ctx* c, int max_iterations, tp_iter_info* hist, int* loops) {
  if (!c || max_iterations < 0) return TP_ERR_ARG;
  tp_status st = tp_init_design(c);
  if (st != TP_OK) return st;
  int loop = 0;
  float change = 1.0f;
  while (change > 1e-2 && loop < max_iterations) {
    loop++;
    tp_iter_info info;
    std::memset(&info, 0, sizeof info);
    st = tp_design_iteration(c, &info);
    if (st != TP_OK) {
      if (loops) *loops = loop;
      return st;
    }
    info.loop = loop;
    change = (float)info.change;
    if (hist) hist[loop - 1] = info;
  }
  if (loops) *loops = loop;
  return TP_OK;
}

}  // extern "C"
