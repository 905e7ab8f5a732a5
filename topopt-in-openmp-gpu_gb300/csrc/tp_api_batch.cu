// Several load cases sharing one stiffness operator: the multi-load problem
// generator, and the state solve of all cases as one multi-right-hand-side
// PCG whose iteration loop runs on the device.
//
// The solve: after the set-up (residuals and load norms of all columns), the
// whole CG loop is one CUDA graph launch. The graph holds a single
// conditional WHILE node whose body is one PCG iteration over the nr
// columns -- V-cycle, operator application and the vector updates, about a
// hundred kernels, captured once per context -- ending in a kernel that
// advances the iteration counter and clears the loop condition when every
// column's relative residual is below the tolerance, when a residual is not
// finite, or at the iteration cap. The host waits once per solve, not once
// per iteration. The reference solves one load case with host-driven
// iterations (stencil_solvers.c:259-397); each column here follows the same
// recurrence, so a single column reproduces its iterates exactly.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "tp_internal.h"

namespace tp {

// loop condition: continue while some column is above tol, all are finite
// and the cap is not reached; the counter counts executed iterations
__global__ void cg_cond_kernel(double* scal, cudaGraphConditionalHandle h, double tol, int cgmax) {
  const double it = scal[S_IT] + 1.0;
  scal[S_IT] = it;
  const double m = scal[S_MAXRR];
  const bool go = isfinite(m) && !(m < tol) && it < (double)cgmax;
  cudaGraphSetConditional(h, go ? 1u : 0u);
}

__global__ void cg_counter_reset_kernel(double* scal) { scal[S_IT] = 0.0; }

void graph_free(tp_ctx* c) {
  if (c->cg_exec) cudaGraphExecDestroy(c->cg_exec);
  c->cg_exec = nullptr;
  c->cg_exec_nr = 0;
}

static bool graph_build(tp_ctx* c, int nr) {
  graph_free(c);
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
  cudaGraphConditionalHandle h;
  bool ok = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  ok = ok && cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) == cudaSuccess;
  if (ok) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    ok = cudaStreamBeginCaptureToGraph(c->s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    if (ok) {
      c->capturing = true;
      pcg_iteration(c, c->d_U, -1, nr);
      cg_cond_kernel<<<1, 1, 0, c->s>>>(c->d_scal, h, c->p.cgtol, c->p.cgmax);
      c->capturing = false;
      cudaGraph_t out = nullptr;
      ok = cudaStreamEndCapture(c->s, &out) == cudaSuccess && c->err.empty();
    }
  }
  if (ok) ok = cudaGraphInstantiate(&c->cg_exec, g, 0) == cudaSuccess;
  cudaGraphDestroy(g);
  if (!ok) {
    c->cg_exec = nullptr;
    cudaGetLastError();
    if (c->err.empty()) c->err = "CG graph: capture or instantiation failed";
    return false;
  }
  c->cg_exec_nr = nr;
  return true;
}

// K U = F for the context's nrhs columns, warm start from U: set-up and the
// graph launch, enqueued only
tp_status pcg_graph_enqueue(tp_ctx* c) {
  const int nr = c->p.nrhs;
  if (!c->cg_exec || c->cg_exec_nr != nr) {
    if (!graph_build(c, nr)) return TP_ERR_CUDA;
  }
  pcg_prologue(c, c->d_F, c->d_U, nr);
  cg_counter_reset_kernel<<<1, 1, 0, c->s>>>(c->d_scal);
  cudaGraphLaunch(c->cg_exec, c->s);
  return TP_OK;
}

// the outcome of the enqueued solve, from the scalars already copied into
// h_scal (the caller has synchronised the stream)
tp_status pcg_graph_status(tp_ctx* c, int* iters, double* relres) {
  if (!c->err.empty()) return TP_ERR_CUDA;
  if (coarse_status(c) != TP_OK) return TP_ERR_TIMEOUT;
  const double* s = c->h_scal;
  const double rr = s[S_MAXRR];
  *iters = (int)s[S_IT] - 1;  // index of the last iteration, as the reference reports it
  *relres = (double)(float)rr;
  if (!std::isfinite(rr)) {
    c->note = "CG: non-finite residual";
    return TP_ERR_NONFINITE;
  }
  return rr < c->p.cgtol ? TP_OK : TP_ERR_NOT_CONVERGED;
}

tp_status pcg_graph(tp_ctx* c, int* iters, double* relres) {
  tp_status st = pcg_graph_enqueue(c);
  if (st != TP_OK) return st;
  cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(double) * S_COUNT * c->p.nrhs, cudaMemcpyDeviceToHost, c->s);
  cudaError_t e = cudaStreamSynchronize(c->s);
  if (e != cudaSuccess) {
    c->err = std::string("CG graph: ") + cudaGetErrorString(e);
    return TP_ERR_CUDA;
  }
  return pcg_graph_status(c, iters, relres);
}

}  // namespace tp

// ---------------------------------------------------------------------------
// Multi-load problem generator (no counterpart in the reference, whose
// single load is built at stencil_optimization.c:41-95): ncase load cases,
// each with nload unit nodal forces on distinct nodes of the free end face
// x = nelx, nodes drawn uniformly from that face and directions uniformly
// from the unit sphere (z = 2u - 1, phi = 2 pi v). The generator is a
// SplitMix64 stream from the seed, so every platform draws the same loads.
namespace {
struct SplitMix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
};
}  // namespace

extern "C" tp_status tp_multiload(int nelx, int nely, int nelz, int ncase, int nload, unsigned long long seed,
                                  double* F_host) {
  if (nelx < 1 || nely < 1 || nelz < 1 || ncase < 1 || nload < 1 || !F_host) return TP_ERR_ARG;
  const long ny = nely + 1, nz = nelz + 1, nx = nelx + 1;
  const long face = ny * nz;
  if (nload > face) return TP_ERR_ARG;
  const long ndof = 3 * nx * ny * nz;
  SplitMix64 rng{seed};
  std::vector<char> used(face);
  for (int r = 0; r < ncase; r++) {
    double* F = F_host + (long)r * ndof;
    for (long i = 0; i < ndof; i++) F[i] = 0.0;
    std::fill(used.begin(), used.end(), 0);
    for (int q = 0; q < nload; q++) {
      long f;
      do {
        f = (long)(rng.uniform() * (double)face);
        if (f >= face) f = face - 1;
      } while (used[f]);
      used[f] = 1;
      const long k = f / ny, j = f % ny;  // node (nelx, k, j) of the end face
      const double z = 2.0 * rng.uniform() - 1.0;
      const double phi = 2.0 * M_PI * rng.uniform();
      const double rxy = std::sqrt(std::fmax(0.0, 1.0 - z * z));
      const long n = ((long)nelx * nz + k) * ny + j;
      F[3 * n + 0] = rxy * std::cos(phi);
      F[3 * n + 1] = rxy * std::sin(phi);
      F[3 * n + 2] = z;
    }
  }
  return TP_OK;
}

// per load case of the last solve: the iteration index at which its relative
// residual fell below the tolerance (-1 if it did not) and that residual
extern "C" tp_status tp_solve_columns(tp_ctx* c, int* iters, double* relres) {
  if (!c || !iters || !relres) return TP_ERR_ARG;
  const int nr = c->p.nrhs;
  cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(double) * tp::S_COUNT * nr, cudaMemcpyDeviceToHost, c->s);
  if (cudaStreamSynchronize(c->s) != cudaSuccess) return TP_ERR_CUDA;
  for (int r = 0; r < nr; r++) {
    iters[r] = (int)c->h_scal[r * tp::S_COUNT + tp::S_ITER];
    relres[r] = c->h_scal[r * tp::S_COUNT + tp::S_RELRES];
  }
  return TP_OK;
}

extern "C" tp_status tp_set_graph_solve(tp_ctx* c, int on) {
  if (!c || on < 0 || on > 2) return TP_ERR_ARG;
  c->graph_solve = on;
  return TP_OK;
}
