// Optional per-kernel-class timing: CUDA events recorded on the context's
// stream around each instrumented launch, folded into per-class totals at
// collection points. Off by default; when on, it adds two event records per
// launch and no synchronisation except when the event pool runs out.
#include "tp_internal.h"

namespace tp {

static const char* kProfNames[P_COUNT] = {
    "fine_apply_f64", "fine_jacobi_f64", "fine_resid_f64", "fine_apply_f32", "fine_jacobi_f32",
    "fine_resid_f32", "stencil", "transfer", "coarse_solve", "coarse_factor", "assemble",
    "vector", "design"};

constexpr size_t kPool = 8192;

static cudaEvent_t take_event(tp_ctx* c) {
  if (c->ev_pool.empty()) {
    c->ev_pool.resize(kPool);
    for (auto& e : c->ev_pool) cudaEventCreate(&e);
  }
  if (c->ev_next >= c->ev_pool.size()) prof_collect(c);
  return c->ev_pool[c->ev_next++];
}

ProfScope::ProfScope(tp_ctx* ctx, int i) : c(ctx), id(i) {
  if (!c->prof || c->capturing) return;  // nothing is timed inside a graph capture
  e1 = take_event(c);
  cudaEventRecord(e1, c->s);
}

ProfScope::~ProfScope() {
  if (!c->prof || !e1) return;
  cudaEvent_t e2 = take_event(c);
  cudaEventRecord(e2, c->s);
  c->ev_pending.push_back({id, {e1, e2}});
}

void prof_collect(tp_ctx* c) {
  if (c->ev_pending.empty()) {
    c->ev_next = 0;
    return;
  }
  cudaStreamSynchronize(c->s);
  for (auto& p : c->ev_pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) {
      c->prof_ms[p.first] += ms;
      c->prof_launches[p.first] += 1;
    }
  }
  c->ev_pending.clear();
  c->ev_next = 0;
}

void prof_destroy(tp_ctx* c) {
  for (auto& e : c->ev_pool) cudaEventDestroy(e);
  c->ev_pool.clear();
  c->ev_pending.clear();
}

}  // namespace tp

using namespace tp;

extern "C" {

tp_status tp_profile_enable(tp_ctx* c, int on) {
  if (!c) return TP_ERR_ARG;
  prof_collect(c);
  c->prof = on != 0;
  return TP_OK;
}

tp_status tp_profile_reset(tp_ctx* c) {
  if (!c) return TP_ERR_ARG;
  prof_collect(c);
  for (int i = 0; i < P_COUNT; i++) {
    c->prof_ms[i] = 0.0;
    c->prof_launches[i] = 0;
  }
  return TP_OK;
}

int tp_profile_classes(void) { return P_COUNT; }

tp_status tp_profile_get(tp_ctx* c, int idx, const char** name, long* launches, double* ms) {
  if (!c || idx < 0 || idx >= P_COUNT) return TP_ERR_ARG;
  prof_collect(c);
  if (name) *name = kProfNames[idx];
  if (launches) *launches = c->prof_launches[idx];
  if (ms) *ms = c->prof_ms[idx];
  return TP_OK;
}

}  // extern "C"
