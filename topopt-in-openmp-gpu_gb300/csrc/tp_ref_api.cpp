// The reference's entry points (include/topopt_ref_api.h) over host arrays in
// its padded layout, backed by the GPU library. Built twice: TP_REF_FLOAT=1
// (CTYPE/DTYPE float, the reference as shipped) and TP_REF_FLOAT=0 (double).
//
// Each GPU-backed call converts its host inputs to the canonical device
// layout, runs the CUDA path through the handle API, and converts the
// outputs back, writing exactly the entries the reference's routine writes.
// One device context per grid (nelx, nely, nelz, levels) is cached.
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <mutex>
#include <utility>
#include <tuple>
#include <vector>

#include "topopt_gb300.h"
#include "topopt_ref_api.h"

namespace {

struct Dims {
  int ex, ey, ez, wx, wy, wz;
  long ndof_padded() const { return 3L * wx * wy * wz; }
};

Dims dims_of(int nelx, int nely, int nelz, int l) {
  Dims d;
  d.ex = nelx >> l;
  d.ey = nely >> l;
  d.ez = nelz >> l;
  const int py = (STENCIL_SIZE_Y - ((d.ey + 1) % STENCIL_SIZE_Y)) % STENCIL_SIZE_Y;
  d.wx = d.ex + 3;
  d.wy = d.ey + py + 3;
  d.wz = d.ez + 3;
  return d;
}

inline long pnode(const Dims& d, int i, int k, int j) { return (long)(i + 1) * d.wy * d.wz + (long)(k + 1) * d.wy + (j + 1); }
inline long cnode(const Dims& d, int i, int k, int j) { return ((long)i * (d.ez + 1) + k) * (d.ey + 1) + j; }

// TOPOPT_PRECISION=mixed selects the mixed form (FP32 V-cycle, FP64 CG) for
// every context of these entry points; the default is the FP64 form
int precision_from_env() {
  const char* prec = std::getenv("TOPOPT_PRECISION");
  return (prec && std::strcmp(prec, "mixed") == 0) ? TP_MIXED : TP_FP64;
}

// -- context cache -----------------------------------------------------------
std::map<std::tuple<int, int, int, int>, tp_ctx*> g_ctx;

tp_ctx* ctx_for(int nelx, int nely, int nelz, int nl) {
  const int q = 1 << (nl - 1);
  if (nl < 2 || nelx % q || nely % q || nelz % q) {
    std::fprintf(stderr, "topopt_gb300: grid %dx%dx%d cannot hold %d levels\n", nelx, nely, nelz, nl);
    std::abort();
  }
  auto key = std::make_tuple(nelx, nely, nelz, nl);
  auto it = g_ctx.find(key);
  if (it != g_ctx.end()) return it->second;
  tp_params p;
  tp_default_params(&p);
  p.nelx = nelx;
  p.nely = nely;
  p.nelz = nelz;
  p.nl = nl;
  p.precision = precision_from_env();
  tp_ctx* c = nullptr;
  const tp_status st = tp_create(&p, &c);
  if (st != TP_OK) {
    std::fprintf(stderr, "topopt_gb300: tp_create failed: %s (%s)\n", tp_status_string(st),
                 c ? tp_error_message(c) : "");
    std::abort();
  }
  // the level-0 kernels' launch plans tuned once for this grid (as a caller
  // of the handle API does with tp_autotune): every plan gives the same
  // results bit for bit; TOPOPT_AUTOTUNE=0 keeps the default plans
  const char* tune = std::getenv("TOPOPT_AUTOTUNE");
  if (!(tune && std::strcmp(tune, "0") == 0)) tp_autotune(c, nullptr);
  g_ctx[key] = c;
  return c;
}

// A context holding level `need` for the grid. A cached context of the grid
// with that many levels or more serves (the entry points that need no
// particular level count -- volume, compliance, filter -- then share the
// solver's context). Otherwise a new one gets the most levels the grid's
// divisibility allows while its coarsest level stays above ~5k DOFs, and at
// least `need`: with too few levels the coarsest level's band Cholesky would
// hold a band of the fine grid's size.
tp_ctx* ctx_levels(const gridContext& gc, int need) {
  const int nx = (int)gc.nelx, ny = (int)gc.nely, nz = (int)gc.nelz;
  if (need < 2) need = 2;
  tp_ctx* best = nullptr;
  int best_nl = 0;
  for (auto& kv : g_ctx) {
    const auto& k = kv.first;
    if (std::get<0>(k) == nx && std::get<1>(k) == ny && std::get<2>(k) == nz && std::get<3>(k) >= need &&
        std::get<3>(k) > best_nl) {
      best = kv.second;
      best_nl = std::get<3>(k);
    }
  }
  if (best) return best;
  int nl = need;
  for (;;) {
    const int q = 1 << nl;  // the next level count's coarsening factor
    if (nl + 1 > 8 || nx % q || ny % q || nz % q) break;
    const long coarse = 3L * (nx / q + 1) * (ny / q + 1) * (nz / q + 1);
    if (coarse < 5000) break;
    nl++;
  }
  return ctx_for(nx, ny, nz, nl);
}

void check(tp_ctx* c, tp_status st, const char* what) {
  if (st == TP_OK || st == TP_ERR_NOT_CONVERGED) return;
  std::fprintf(stderr, "topopt_gb300: %s failed: %s (%s)\n", what, tp_status_string(st), tp_error_message(c));
  std::abort();
}

// -- device scratch --------------------------------------------------------------
struct Scratch {
  double* p = nullptr;
  size_t n = 0;
  double* get(size_t want) {
    if (want > n) {
      if (p) cudaFree(p);
      if (cudaMalloc(&p, want * sizeof(double)) != cudaSuccess) {
        std::fprintf(stderr, "topopt_gb300: cudaMalloc of %zu doubles failed\n", want);
        std::abort();
      }
      n = want;
    }
    return p;
  }
};
Scratch g_s[4];

// -- host staging -------------------------------------------------------------
// The canonical host copies that cross to and from the device live in
// page-locked memory (cudaMallocHost), so every copy runs at the host link's
// full rate; blocks are cached by size and reused from call to call, and the
// vectors are left uninitialised on construction (the conversion that fills
// one writes every element). If page-locked memory is refused, plain memory
// stands in (slower copies, same results).
class PinnedCache {
 public:
  void* get(size_t bytes) {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = free_.lower_bound(bytes);
    if (it != free_.end() && it->first <= 2 * bytes + 4096) {
      void* p = it->second;
      free_.erase(it);
      return p;
    }
    void* p = nullptr;
    bool pinned = cudaMallocHost(&p, bytes) == cudaSuccess;
    if (!pinned) {
      cudaGetLastError();
      p = std::malloc(bytes ? bytes : 1);
      if (!p) throw std::bad_alloc();
    }
    info_[p] = std::make_pair(bytes, pinned);
    return p;
  }
  void put(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(mu_);
    free_.insert(std::make_pair(info_[p].first, p));
  }

 private:
  std::mutex mu_;
  std::multimap<size_t, void*> free_;
  std::map<void*, std::pair<size_t, bool>> info_;
};
PinnedCache& pinned_cache() {
  static PinnedCache* cache = new PinnedCache();  // kept until exit: blocks may outlive static destructors
  return *cache;
}

template <typename T>
struct StageAlloc {
  using value_type = T;
  StageAlloc() = default;
  template <typename U>
  StageAlloc(const StageAlloc<U>&) {}
  T* allocate(size_t n) { return static_cast<T*>(pinned_cache().get(n * sizeof(T))); }
  void deallocate(T* p, size_t) { pinned_cache().put(p); }
  template <typename U>
  void construct(U* p) noexcept {
    ::new (static_cast<void*>(p)) U;  // default-initialised: no zero fill
  }
  template <typename U, typename... A>
  void construct(U* p, A&&... a) {
    ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
  }
  template <typename U>
  bool operator==(const StageAlloc<U>&) const { return true; }
  template <typename U>
  bool operator!=(const StageAlloc<U>&) const { return false; }
};
using HVec = std::vector<double, StageAlloc<double>>;

// padded host vector of level l -> canonical double (host). A y line of
// nodes is contiguous in both layouts (3 (ey + 1) values), so each (x, z)
// line is one copy; the lines are shared out over all host threads.
template <typename T>
static inline void line_copy(double* dst, const T* src, long n) {
  if constexpr (sizeof(T) == sizeof(double)) {
    std::memcpy(dst, src, sizeof(double) * n);
  } else {
    for (long q = 0; q < n; q++) dst[q] = (double)src[q];
  }
}
template <typename T>
static inline void line_copy_out(T* dst, const double* src, long n) {
  if constexpr (sizeof(T) == sizeof(double)) {
    std::memcpy(dst, src, sizeof(double) * n);
  } else {
    for (long q = 0; q < n; q++) dst[q] = (T)src[q];
  }
}
template <typename T>
HVec to_canon(const Dims& d, const T* v) {
  HVec out(3L * (d.ex + 1) * (d.ey + 1) * (d.ez + 1));
  const long nl = 3L * (d.ey + 1);
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i <= d.ex; i++)
    for (int k = 0; k <= d.ez; k++) line_copy(&out[3 * cnode(d, i, k, 0)], v + 3 * pnode(d, i, k, 0), nl);
  return out;
}
template <typename T>
void from_canon(const Dims& d, const HVec& h, T* v) {
  const long nl = 3L * (d.ey + 1);
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i <= d.ex; i++)
    for (int k = 0; k <= d.ez; k++) line_copy_out(v + 3 * pnode(d, i, k, 0), &h[3 * cnode(d, i, k, 0)], nl);
}

// padded element array (fine level) <-> canonical, one y line per copy
HVec el_to_canon(const gridContext& gc, const DTYPE* x) {
  const int ex = gc.nelx, ey = gc.nely, ez = gc.nelz;
  const long wy = gc.wrapy - 1, wz = gc.wrapz - 1;
  HVec out((size_t)ex * ey * ez);
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < ex; i++)
    for (int k = 0; k < ez; k++)
      line_copy(&out[((size_t)i * ez + k) * ey], x + (i + 1) * wy * wz + (k + 1) * wy + 1, ey);
  return out;
}
void el_from_canon(const gridContext& gc, const HVec& h, DTYPE* x) {
  const int ex = gc.nelx, ey = gc.nely, ez = gc.nelz;
  const long wy = gc.wrapy - 1, wz = gc.wrapz - 1;
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < ex; i++)
    for (int k = 0; k < ez; k++)
      line_copy_out(x + (i + 1) * wy * wz + (k + 1) * wy + 1, &h[((size_t)i * ez + k) * ey], ey);
}

// an element array of n entries as a staged double copy
template <typename T>
HVec el_copy(const T* x, long n) {
  HVec out((size_t)n);
#pragma omp parallel for schedule(static)
  for (long e = 0; e < n; e++) out[e] = (double)x[e];
  return out;
}

// bytes copied host -> device and device -> host by the entry points
long g_h2d = 0, g_d2h = 0;

double* up(int slot, const HVec& h) {
  double* d = g_s[slot].get(h.size());
  cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
  g_h2d += (long)(h.size() * sizeof(double));
  return d;
}
HVec down(const double* d, size_t n) {
  HVec h(n);
  cudaMemcpy(h.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost);
  g_d2h += (long)(n * sizeof(double));
  return h;
}

// -- pipelined transfers -------------------------------------------------------
// A transfer of an array of lines (len doubles each, line l at l * len in the
// canonical layout) in chunks of whole lines through two page-locked buffers,
// on a stream of its own: the host converts chunk j + 1 (its lines shared out
// over the host threads) while chunk j is on the link, so conversion and copy
// overlap instead of adding up. Each call returns after its last chunk has
// landed (uploads) or been converted (downloads), so the device buffer is
// ready for the context's stream and the host array for the caller.
struct Pipe {
  static constexpr long kChunk = 1L << 20;  // doubles per buffer
  double* buf[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaStream_t st = nullptr;
  std::mutex mu;
  bool ready() {
    if (st) return true;
    for (int b = 0; b < 2; b++) {
      buf[b] = static_cast<double*>(pinned_cache().get(kChunk * sizeof(double)));
      if (cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming) != cudaSuccess) return false;
    }
    return cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
  }
};
Pipe& pipe() {
  static Pipe* p = new Pipe();  // kept until exit, like the staging cache
  return *p;
}
// the pipe's stream (created on first use), or null (then copies go on the
// legacy stream)
cudaStream_t transfer_stream() {
  Pipe& P = pipe();
  std::lock_guard<std::mutex> lock(P.mu);
  return P.ready() ? P.st : nullptr;
}

// fill(l, dst): canonical line l into dst[0 .. len); n: the array's doubles
// (the last line may be short)
template <typename Fill>
void up_lines(double* d, long n, long len, Fill fill) {
  Pipe& P = pipe();
  std::lock_guard<std::mutex> lock(P.mu);
  if (!P.ready()) throw std::runtime_error("pipelined transfer: no stream");
  const long nlines = (n + len - 1) / len, per = std::max(1L, Pipe::kChunk / len);
  long j = 0;
  for (long l0 = 0; l0 < nlines; l0 += per, j++) {
    const long l1 = std::min(nlines, l0 + per);
    const int b = (int)(j & 1);
    if (j >= 2) cudaEventSynchronize(P.ev[b]);  // the copy that last read this buffer
    double* dst = P.buf[b];
#pragma omp parallel for schedule(static)
    for (long l = l0; l < l1; l++) fill(l, dst + (l - l0) * len);
    const long lo = l0 * len, hi = std::min(n, l1 * len);
    cudaMemcpyAsync(d + lo, dst, (hi - lo) * sizeof(double), cudaMemcpyHostToDevice, P.st);
    cudaEventRecord(P.ev[b], P.st);
  }
  cudaStreamSynchronize(P.st);
  g_h2d += n * (long)sizeof(double);
}

// drain(l, src): canonical line l from src[0 .. len) into the caller's array
template <typename Drain>
void down_lines(const double* d, long n, long len, Drain drain) {
  Pipe& P = pipe();
  std::lock_guard<std::mutex> lock(P.mu);
  if (!P.ready()) throw std::runtime_error("pipelined transfer: no stream");
  const long nlines = (n + len - 1) / len, per = std::max(1L, Pipe::kChunk / len);
  auto issue = [&](long j) {
    const long l0 = j * per, l1 = std::min(nlines, l0 + per);
    const long lo = l0 * len, hi = std::min(n, l1 * len);
    cudaMemcpyAsync(P.buf[j & 1], d + lo, (hi - lo) * sizeof(double), cudaMemcpyDeviceToHost, P.st);
    cudaEventRecord(P.ev[j & 1], P.st);
  };
  const long nchunks = (nlines + per - 1) / per;
  if (nchunks > 0) issue(0);
  for (long j = 0; j < nchunks; j++) {
    if (j + 1 < nchunks) issue(j + 1);  // its buffer was drained at step j - 1
    cudaEventSynchronize(P.ev[j & 1]);
    const long l0 = j * per, l1 = std::min(nlines, l0 + per);
    const double* src = P.buf[j & 1];
#pragma omp parallel for schedule(static)
    for (long l = l0; l < l1; l++) drain(l, src + (l - l0) * len);
  }
  g_d2h += n * (long)sizeof(double);
}

// The padded host layouts hold the canonical lines (len values) as a regular
// box: line (i, k) at base + i si + k sk, si a multiple of sk. Double arrays
// cross in one strided copy between the caller's array and the device (the
// copy engines read pageable memory over the host link at ~85-185 GB/s on
// this part, several times a host-side conversion into staging; the halo is
// neither read nor written); float arrays (the float flavour) take the
// pipelined conversion above. With a stream s, the copy goes on s (a stream
// that does not wait for the context's) and returns once it has landed.
bool copy_box(double* dev, double* host, long len, long nk, long ni, long sk, long si, bool up,
              cudaStream_t s = nullptr) {
  cudaMemcpy3DParms p = {};
  const cudaPitchedPtr hp = make_cudaPitchedPtr(host, sk * sizeof(double), sk, si / sk);
  const cudaPitchedPtr dp = make_cudaPitchedPtr(dev, len * sizeof(double), len, nk);
  p.srcPtr = up ? hp : dp;
  p.dstPtr = up ? dp : hp;
  p.extent = make_cudaExtent(len * sizeof(double), nk, ni);
  p.kind = up ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  if (s ? (cudaMemcpy3DAsync(&p, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
        : cudaMemcpy3D(&p) != cudaSuccess)
    return false;
  (up ? g_h2d : g_d2h) += len * nk * ni * (long)sizeof(double);
  return true;
}

// the line shapes of the three layouts: a level's nodal vector (a y line of
// nodes, 3 (ey + 1) values, per (x, z)), the fine elements (a y line of ey per
// (x, z)), and a plain array of n values (lines of kPlain)
constexpr long kPlain = 4096;
template <typename T>
void up_nodes(double* d, const Dims& dm, const T* v, cudaStream_t s = nullptr) {
  const long len = 3L * (dm.ey + 1), nz = dm.ez + 1;
  if constexpr (sizeof(T) == sizeof(double)) {
    if (copy_box(d, (double*)(v + 3 * pnode(dm, 0, 0, 0)), len, nz, dm.ex + 1, 3L * dm.wy, 3L * dm.wy * dm.wz, true,
                 s))
      return;
    cudaGetLastError();
  }
  up_lines(d, len * (dm.ex + 1) * nz, len, [&](long l, double* dst) {
    line_copy(dst, v + 3 * pnode(dm, (int)(l / nz), (int)(l % nz), 0), len);
  });
}
template <typename T>
void down_nodes(const double* d, const Dims& dm, T* v) {
  const long len = 3L * (dm.ey + 1), nz = dm.ez + 1;
  if constexpr (sizeof(T) == sizeof(double)) {
    if (copy_box((double*)d, (double*)(v + 3 * pnode(dm, 0, 0, 0)), len, nz, dm.ex + 1, 3L * dm.wy,
                 3L * dm.wy * dm.wz, false))
      return;
    cudaGetLastError();
  }
  down_lines(d, len * (dm.ex + 1) * nz, len, [&](long l, const double* src) {
    line_copy_out(v + 3 * pnode(dm, (int)(l / nz), (int)(l % nz), 0), src, len);
  });
}
void up_elems(double* d, const gridContext& gc, const DTYPE* x) {
  const long ey = gc.nely, ez = gc.nelz, wy = gc.wrapy - 1, wz = gc.wrapz - 1;
  if constexpr (sizeof(DTYPE) == sizeof(double)) {
    if (copy_box(d, (double*)(x + wy * wz + wy + 1), ey, ez, gc.nelx, wy, wy * wz, true)) return;
    cudaGetLastError();
  }
  up_lines(d, (long)gc.nelx * ez * ey, ey, [&](long l, double* dst) {
    line_copy(dst, x + (l / ez + 1) * wy * wz + (l % ez + 1) * wy + 1, ey);
  });
}
void down_elems(const double* d, const gridContext& gc, DTYPE* x) {
  const long ey = gc.nely, ez = gc.nelz, wy = gc.wrapy - 1, wz = gc.wrapz - 1;
  if constexpr (sizeof(DTYPE) == sizeof(double)) {
    if (copy_box((double*)d, (double*)(x + wy * wz + wy + 1), ey, ez, gc.nelx, wy, wy * wz, false)) return;
    cudaGetLastError();
  }
  down_lines(d, (long)gc.nelx * ez * ey, ey, [&](long l, const double* src) {
    line_copy_out(x + (l / ez + 1) * wy * wz + (l % ez + 1) * wy + 1, src, ey);
  });
}
template <typename T>
void up_plain(double* d, const T* x, long n) {
  if constexpr (sizeof(T) == sizeof(double)) {
    if (cudaMemcpy(d, x, n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess) {
      g_h2d += n * (long)sizeof(double);
      return;
    }
    cudaGetLastError();
  }
  up_lines(d, n, kPlain, [&](long l, double* dst) { line_copy(dst, x + l * kPlain, std::min(kPlain, n - l * kPlain)); });
}
template <typename T>
void down_plain(const double* d, T* x, long n) {
  if constexpr (sizeof(T) == sizeof(double)) {
    if (cudaMemcpy(x, d, n * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess) {
      g_d2h += n * (long)sizeof(double);
      return;
    }
    cudaGetLastError();
  }
  down_lines(d, n, kPlain, [&](long l, const double* src) {
    line_copy_out(x + l * kPlain, src, std::min(kPlain, n - l * kPlain));
  });
}

void set_design(tp_ctx* c, const gridContext& gc, const DTYPE* x) {
  up_elems(tp_field_ptr(c, TP_FIELD_XPHYS), gc, x);
  check(c, tp_field_written(c, TP_FIELD_XPHYS), "upload xPhys");
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// local_matrix.h: the constitutive matrix, strain-displacement matrix and
// element stiffness tables (local_matrix.c:7-319)
void getC(MTYPE C[6][6], const MTYPE nu) {
  const MTYPE t1 = (1.0 - nu) / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const MTYPE t2 = nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const MTYPE t3 = 1.0 / (2.0 * (1.0 + nu));
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) C[i][j] = 0.0;
  C[0][0] = C[1][1] = C[2][2] = t1;
  C[3][3] = C[4][4] = C[5][5] = t3;
  C[0][1] = C[1][0] = C[0][2] = C[2][0] = C[1][2] = C[2][1] = t2;
}

// Strain-displacement matrix of the trilinear hexahedron at iso point
// (xi, eta, zeta) for nodal coordinates xe; strains ordered xx, yy, zz, xy,
// yz, zx with engineering shears. The Jacobian inverse is the adjugate over
// the determinant.
void getB(MTYPE B[6][24], MTYPE* jdet, const MTYPE iso[3], const MTYPE xe[24]) {
  static const int s[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                              {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  double dN[8][3];
  for (int q = 0; q < 8; q++) {
    const double a = 1 + s[q][0] * iso[0], b = 1 + s[q][1] * iso[1], c = 1 + s[q][2] * iso[2];
    dN[q][0] = 0.125 * s[q][0] * b * c;
    dN[q][1] = 0.125 * s[q][1] * a * c;
    dN[q][2] = 0.125 * s[q][2] * a * b;
  }
  double J[3][3] = {{0}};
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++)
      for (int q = 0; q < 8; q++) J[r][c] += dN[q][r] * xe[3 * q + c];
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  *jdet = det;
  double Ji[3][3];
  Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  for (int m = 0; m < 6; m++)
    for (int n = 0; n < 24; n++) B[m][n] = 0.0;
  for (int q = 0; q < 8; q++) {
    double g[3];
    for (int r = 0; r < 3; r++) g[r] = Ji[r][0] * dN[q][0] + Ji[r][1] * dN[q][1] + Ji[r][2] * dN[q][2];
    B[0][3 * q + 0] = g[0];
    B[1][3 * q + 1] = g[1];
    B[2][3 * q + 2] = g[2];
    B[3][3 * q + 0] = g[1];
    B[3][3 * q + 1] = g[0];
    B[4][3 * q + 1] = g[2];
    B[4][3 * q + 2] = g[1];
    B[5][3 * q + 0] = g[2];
    B[5][3 * q + 2] = g[0];
  }
}

void getKEsubspace(MTYPE* KEarray, const MTYPE nu, const int l) { tp_element_matrix_tables(l, nu, KEarray); }

// ---------------------------------------------------------------------------
// stencil_grid_utility.h / gpu_definitions.h: set-up on the host
void computePadding(const struct gridContext* gc, const int l, int* ncell, int* wrapx, int* wrapy, int* wrapz,
                    uint_fast32_t* ndof) {
  *ncell = 1 << l;
  const Dims d = dims_of((int)gc->nelx, (int)gc->nely, (int)gc->nelz, l);
  *wrapx = d.wx;
  *wrapy = d.wy;
  *wrapz = d.wz;
  *ndof = (uint_fast32_t)d.ndof_padded();
}

void setFixedDof_halo(struct gridContext* gc, const int l) {
  const Dims d = dims_of((int)gc->nelx, (int)gc->nely, (int)gc->nelz, l);
  const int nyc = d.ey + 1, nzc = d.ez + 1;
  const int lim = d.ey / 4 + 1;
  gc->fixedDofs[l].n = 3 * nzc * 2 * lim;
  gc->fixedDofs[l].idx = (uint_fast32_t*)std::malloc(sizeof(uint_fast32_t) * gc->fixedDofs[l].n);
  int o = 0;
  const long i = 1;
  for (long k = 1; k < nzc + 1; k++) {
    for (long j = 1; j < lim + 1; j++)
      for (int c = 0; c < 3; c++) gc->fixedDofs[l].idx[o++] = 3 * (i * d.wy * d.wz + d.wy * k + j) + c;
    for (long j = (nyc + 1) - lim; j < nyc + 1; j++)
      for (int c = 0; c < 3; c++) gc->fixedDofs[l].idx[o++] = 3 * (i * d.wy * d.wz + d.wy * k + j) + c;
  }
}

void setupGC(struct gridContext* gc, const int nl, const int nelx, const int nely, const int nelz) {
  gc->E0 = 1;
  gc->Emin = 1e-6;
  gc->nu = 0.3;
  gc->penal = 3;
  gc->elementSizeX = gc->elementSizeY = gc->elementSizeZ = 0.5;
  gc->nelx = nelx;
  gc->nely = nely;
  gc->nelz = nelz;
  const Dims d = dims_of(nelx, nely, nelz, 0);
  gc->wrapx = d.wx;
  gc->wrapy = d.wy;
  gc->wrapz = d.wz;
  gc->precomputedKE = (MTYPE**)std::malloc(sizeof(MTYPE*) * nl);
  gc->fixedDofs = (struct FixedDofs*)std::malloc(sizeof(struct FixedDofs) * nl);
  for (int l = 0; l < nl; l++) {
    const long n = 576L << (3 * l);
    gc->precomputedKE[l] = (MTYPE*)std::malloc(sizeof(MTYPE) * n);
    getKEsubspace(gc->precomputedKE[l], gc->nu, l);
    setFixedDof_halo(gc, l);
  }
}

void freeGC(struct gridContext* gc, const int nl) {
  for (int l = 0; l < nl; l++) {
    std::free(gc->precomputedKE[l]);
    std::free(gc->fixedDofs[l].idx);
  }
  std::free(gc->precomputedKE);
  std::free(gc->fixedDofs);
}

static void* zalloc(size_t n, size_t sz) { return std::calloc(n ? n : 1, sz); }

void allocateZeroPaddedStateField(const struct gridContext gc, const int l, CTYPE** v) {
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  *v = (CTYPE*)zalloc(d.ndof_padded(), sizeof(CTYPE));
}
void allocateZeroPaddedStateField_MTYPE(const struct gridContext gc, const int l, MTYPE** v) {
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  *v = (MTYPE*)zalloc(d.ndof_padded(), sizeof(MTYPE));
}
void allocateZeroPaddedStateField_STYPE(const struct gridContext gc, const int l, STYPE** v) {
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  *v = (STYPE*)zalloc(d.ndof_padded(), sizeof(STYPE));
}

// One device: the reference's x-slab split (gpu_definitions.c:3-53) is never
// exercised there (num_targets = 1); every target here sees the whole grid.
void gridContextToGPUGrid(struct gridContext* gc, struct gpuGrid* gpu_gc, const int nl, const int verbose) {
  const int n = gpu_gc->num_targets > 0 ? gpu_gc->num_targets : 1;
  gpu_gc->target = (struct gpuNode*)std::calloc(n, sizeof(struct gpuNode));
  for (int i = 0; i < n; i++) {
    struct gpuNode* node = &gpu_gc->target[i];
    node->id = i;
    node->prev = i > 0 ? &gpu_gc->target[i - 1] : nullptr;
    node->next = i < n - 1 ? &gpu_gc->target[i + 1] : nullptr;
    node->offset_x = i > 0 ? 1 : 0;
    node->x_global = 0;
    node->gc = (struct gridContext*)std::malloc(sizeof(struct gridContext));
    setupGC(node->gc, nl, (int)gc->nelx, (int)gc->nely, (int)gc->nelz);
    if (verbose == 1) std::printf("GPU %d: whole grid on one device\n", i);
  }
}

void freeGPUGrid(struct gpuGrid* gpu_gc, const int nl) {
  for (int i = 0; i < gpu_gc->num_targets; i++) {
    freeGC(gpu_gc->target[i].gc, nl);
    std::free(gpu_gc->target[i].gc);
  }
  std::free(gpu_gc->target);
}

// device residency is managed by the library: nothing to map
void enter_data(const struct gridContext, const struct SolverDataBuffer, const struct gpuGrid, const DTYPE*,
                const DTYPE*, const DTYPE*, const STYPE*, const CTYPE*, const DTYPE*, const int, const int) {}

// ---------------------------------------------------------------------------
// stencil_methods.h
void applyStateOperator_stencil(const struct gpuNode* node, const DTYPE* x, const CTYPE* in, CTYPE* out) {
  const gridContext& gc = *node->gc;
  tp_ctx* c = ctx_levels(gc, 2);
  set_design(c, gc, x);
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, 0);
  const HVec h = to_canon(d, in);
  double* din = up(0, h);
  double* dout = g_s[1].get(h.size());
  check(c, tp_apply(c, 0, din, dout), "applyStateOperator_stencil");
  from_canon(d, down(dout, h.size()), out);
  // y-padding of every x/z line is zeroed (stencil_methods.c:407-418)
  for (int i = 0; i < d.wx; i++)
    for (int k = 0; k < d.wz; k++)
      for (int j = d.ey + 2; j < d.wy; j++)
        for (int q = 0; q < 3; q++) out[3 * ((long)i * d.wy * d.wz + (long)k * d.wy + j) + q] = 0;
}

void applyStateOperatorSubspace_halo(const struct gpuNode* node, const int l, const DTYPE* x, CTYPE* in,
                                     CTYPE* out) {
  const gridContext& gc = *node->gc;
  tp_ctx* c = ctx_levels(gc, l + 1);
  set_design(c, gc, x);
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  const HVec h = to_canon(d, in);
  double* din = up(0, h);
  double* dout = g_s[1].get(h.size());
  if (l >= 1) check(c, tp_assemble(c), "assemble");
  check(c, tp_apply_subspace(c, l, din, dout), "applyStateOperatorSubspace_halo");
  std::memset(out, 0, sizeof(CTYPE) * d.ndof_padded());  // (stencil_methods.c:453-455)
  from_canon(d, down(dout, h.size()), out);
}

void getComplianceAndSensetivity_halo(const struct gpuNode* node, const DTYPE* x, STYPE* u, DTYPE* c_out,
                                      DTYPE* dcdx) {
  const gridContext& gc = *node->gc;
  tp_ctx* c = ctx_levels(gc, 2);
  set_design(c, gc, x);
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, 0);
  up_nodes(tp_field_ptr(c, TP_FIELD_U), d, u);
  double cc = 0;
  check(c, tp_compliance(c, &cc), "getComplianceAndSensetivity_halo");
  down_elems(tp_field_ptr(c, TP_FIELD_DC), gc, dcdx);
  *c_out = (DTYPE)cc;
}

void projectToFinerGrid_halo(const struct gpuNode* node, const int l, const CTYPE* ucoarse, CTYPE* ufine) {
  const gridContext& gc = *node->gc;
  tp_ctx* c = ctx_levels(gc, l + 2);
  const Dims dc = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l + 1);
  const Dims df = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  const HVec h = to_canon(dc, ucoarse);
  double* din = up(0, h);
  const size_t nf = 3L * (df.ex + 1) * (df.ey + 1) * (df.ez + 1);
  double* dout = g_s[1].get(nf);
  check(c, tp_prolong(c, l, din, dout), "projectToFinerGrid_halo");
  from_canon(df, down(dout, nf), ufine);
}

void projectToCoarserGrid_halo(const struct gpuNode* node, const int l, const CTYPE* ufine, CTYPE* ucoarse) {
  const gridContext& gc = *node->gc;
  tp_ctx* c = ctx_levels(gc, l + 2);
  const Dims dc = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l + 1);
  const Dims df = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  const HVec h = to_canon(df, ufine);
  double* din = up(0, h);
  const size_t nc = 3L * (dc.ex + 1) * (dc.ey + 1) * (dc.ez + 1);
  double* dout = g_s[1].get(nc);
  check(c, tp_restrict(c, l, din, dout), "projectToCoarserGrid_halo");
  from_canon(dc, down(dout, nc), ucoarse);
}

void assembleInvertedMatrixDiagonalSubspace_halo(const struct gpuNode* node, const DTYPE* x, const int l,
                                                 MTYPE* diag) {
  const gridContext& gc = *node->gc;
  tp_ctx* c = ctx_levels(gc, l + 1);
  set_design(c, gc, x);
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  const size_t n = 3L * (d.ex + 1) * (d.ey + 1) * (d.ez + 1);
  double* dout = g_s[1].get(n);
  check(c, tp_assemble(c), "assemble");
  check(c, tp_inv_diag(c, l, dout), "assembleInvertedMatrixDiagonalSubspace_halo");
  std::memset(diag, 0, sizeof(MTYPE) * d.ndof_padded());
  from_canon(d, down(dout, n), diag);
}

// ---------------------------------------------------------------------------
// stencil_solvers.h
static void smooth_common(const gridContext& gc, const DTYPE* x, int l, int subspace, int nswp, double omega,
                          const MTYPE* invD, CTYPE* u, const CTYPE* b) {
  tp_ctx* c = ctx_levels(gc, l + 1);
  set_design(c, gc, x);
  check(c, tp_assemble(c), "assemble");
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  const HVec hu = to_canon(d, u), hb = to_canon(d, b), hd = to_canon(d, invD);
  double* du = up(0, hu);
  double* db = up(1, hb);
  double* dd = up(2, hd);
  check(c, tp_smooth_ex(c, l, subspace, nswp, omega, dd, db, du), "smoothDampedJacobi");
  from_canon(d, down(du, hu.size()), u);
}

void smoothDampedJacobi_halo(const struct gpuNode* node, const DTYPE* x, const uint_fast32_t nswp,
                             const CTYPE omega, const MTYPE* invD, CTYPE* u, const CTYPE* b, CTYPE* tmp) {
  (void)tmp;
  smooth_common(*node->gc, x, 0, 0, (int)nswp, (double)omega, invD, u, b);
}

void smoothDampedJacobiSubspace_halo(const struct gpuNode* node, const DTYPE* x, const int l,
                                     const uint_fast32_t nswp, const CTYPE omega, const MTYPE* invD, CTYPE* u,
                                     const CTYPE* b, CTYPE* tmp) {
  (void)tmp;
  smooth_common(*node->gc, x, l, 1, (int)nswp, (double)omega, invD, u, b);
}

// CSR smoothing and SpMV run on the host, as the reference's own do
// (stencil_solvers.c:55-90, stencil_assembly.c:262-364); the GPU V-cycle
// does not use them.
void applyStateOperatorSubspaceMatrix(const struct gridContext gc, const int l, const struct CSRMatrix M,
                                      const CTYPE* in, CTYPE* out) {
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  std::memset(out, 0, sizeof(CTYPE) * d.ndof_padded());
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i <= d.ex; i++)
    for (int k = 0; k <= d.ez; k++)
      for (int j = 0; j <= d.ey; j++)
        for (int a = 0; a < 3; a++) {
          const long row = 3 * cnode(d, i, k, j) + a;
          double s = 0.0;
          for (int q = M.rowOffsets[row]; q < M.rowOffsets[row + 1]; q++) {
            const long col = M.colIndex[q];
            const long n = col / 3;
            const int jj = (int)(n % (d.ey + 1)), kk = (int)((n / (d.ey + 1)) % (d.ez + 1)),
                      ii = (int)(n / ((long)(d.ey + 1) * (d.ez + 1)));
            s += (double)in[3 * pnode(d, ii, kk, jj) + col % 3] * M.vals[q];
          }
          out[3 * pnode(d, i, k, j) + a] = (CTYPE)s;
        }
}

void smoothDampedJacobiSubspaceMatrix_halo(const struct gridContext* gc, const struct CSRMatrix M, const int l,
                                           const uint_fast32_t nswp, const CTYPE omega, const MTYPE* invD,
                                           CTYPE* u, const CTYPE* b, CTYPE* tmp) {
  const Dims d = dims_of((int)gc->nelx, (int)gc->nely, (int)gc->nelz, l);
  for (uint_fast32_t s = 0; s < nswp; s++) {
    applyStateOperatorSubspaceMatrix(*gc, l, M, u, tmp);
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i <= d.ex; i++)
      for (int k = 0; k <= d.ez; k++)
        for (int j = 0; j <= d.ey; j++)
          for (int a = 0; a < 3; a++) {
            const long p = 3 * pnode(d, i, k, j) + a;
            u[p] += omega * invD[p] * (b[p] - tmp[p]);
          }
  }
}

void solveStateMG_halo(const struct gpuGrid* gpu_gc, DTYPE* x, const int nswp, const int nl, const CTYPE tol,
                       struct SolverDataBuffer* data, int* finalIter, float* finalRes, CTYPE* b, STYPE* u) {
  (void)data;
  const gridContext& gc = *gpu_gc->target[0].gc;
  tp_ctx* c = ctx_for((int)gc.nelx, (int)gc.nely, (int)gc.nelz, nl);
  set_design(c, gc, x);
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, 0);
  double* F = tp_field_ptr(c, TP_FIELD_F);
  double* U = tp_field_ptr(c, TP_FIELD_U);
  // the reference's nswp and tol arrive per call; omega 0.6 and the cap of
  // 1000 iterations are fixed there (stencil_solvers.c:332-334)
  check(c, tp_set_cg(c, (double)tol, 1000, nswp, 0.6), "solver settings");
  // the operators (from xPhys alone) are assembled on the device while F and
  // U cross the host link on the transfer stream, which does not wait for
  // the context's
  check(c, tp_assemble_async(c), "assemble");
  const cudaStream_t s = transfer_stream();
  up_nodes(F, d, b, s);
  up_nodes(U, d, u, s);
  int it = 0;
  double rr = 0;
  check(c, tp_assemble(c), "assemble");
  const tp_status st = tp_solve_rhs(c, F, U, &it, &rr);
  check(c, st, "solveStateMG_halo");
  down_nodes(U, d, u);
  *finalIter = it;
  *finalRes = (float)rr;
}

void allocateSolverData(const struct gridContext gc, const int nl, struct SolverDataBuffer* data) {
  allocateZeroPaddedStateField(gc, 0, &data->r);
  allocateZeroPaddedStateField(gc, 0, &data->p);
  allocateZeroPaddedStateField(gc, 0, &data->q);
  allocateZeroPaddedStateField(gc, 0, &data->z);
  data->invD = (MTYPE**)std::malloc(sizeof(MTYPE*) * nl);
  data->dmg = (CTYPE**)std::malloc(sizeof(CTYPE*) * nl);
  data->rmg = (CTYPE**)std::malloc(sizeof(CTYPE*) * nl);
  data->zmg = (CTYPE**)std::malloc(sizeof(CTYPE*) * nl);
  allocateZeroPaddedStateField(gc, 0, &data->dmg[0]);
  allocateZeroPaddedStateField_MTYPE(gc, 0, &data->invD[0]);
  data->rmg[0] = data->r;
  data->zmg[0] = data->z;
  for (int l = 1; l < nl; l++) {
    allocateZeroPaddedStateField(gc, l, &data->dmg[l]);
    allocateZeroPaddedStateField(gc, l, &data->rmg[l]);
    allocateZeroPaddedStateField(gc, l, &data->zmg[l]);
    allocateZeroPaddedStateField_MTYPE(gc, l, &data->invD[l]);
  }
  data->coarseMatrices = (struct CSRMatrix*)std::calloc(nl, sizeof(struct CSRMatrix));
  for (int l = number_of_matrix_free_levels; l < nl; l++) allocateSubspaceMatrix(gc, l, &data->coarseMatrices[l]);
  std::memset(&data->bottomSolver, 0, sizeof(data->bottomSolver));
}

void freeSolverData(struct SolverDataBuffer* data, const int nl) {
  std::free(data->r);
  std::free(data->z);
  std::free(data->p);
  std::free(data->q);
  std::free(data->invD[0]);
  std::free(data->dmg[0]);
  for (int l = 1; l < nl; l++) {
    std::free(data->invD[l]);
    std::free(data->dmg[l]);
    std::free(data->rmg[l]);
    std::free(data->zmg[l]);
  }
  std::free(data->invD);
  std::free(data->dmg);
  std::free(data->zmg);
  std::free(data->rmg);
  for (int l = number_of_matrix_free_levels; l < nl; l++) freeSubspaceMatrix(&data->coarseMatrices[l]);
  std::free(data->coarseMatrices);
}

// ---------------------------------------------------------------------------
// stencil_assembly.h: the CSR of an assembled level. The pattern is the
// reference's (stencil_assembly.c:8-117): row 3n+a lists the in-range
// neighbours of node n in x, z, y order, three columns each; the values come
// from the GPU-assembled block stencil with fixed rows/columns zeroed and a
// unit diagonal.
void allocateSubspaceMatrix(const struct gridContext gc, const int l, struct CSRMatrix* M) {
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  const int nx = d.ex + 1, ny = d.ey + 1, nz = d.ez + 1;
  const int ndof = 3 * nx * ny * nz;
  M->nrows = ndof;
  M->rowOffsets = (int*)std::malloc(sizeof(int) * (ndof + 1));
  M->rowOffsets[0] = 0;
  for (int i = 0; i < nx; i++)
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++) {
        const int w = 3 * ((std::min(i + 1, nx - 1) - std::max(i - 1, 0) + 1) *
                           (std::min(j + 1, ny - 1) - std::max(j - 1, 0) + 1) *
                           (std::min(k + 1, nz - 1) - std::max(k - 1, 0) + 1));
        const int n = (i * nz + k) * ny + j;
        for (int a = 0; a < 3; a++) M->rowOffsets[3 * n + a + 1] = w;
      }
  for (int r = 1; r <= ndof; r++) M->rowOffsets[r] += M->rowOffsets[r - 1];
  M->nnz = (uint64_t)M->rowOffsets[ndof];
  M->colIndex = (int*)std::malloc(sizeof(int) * M->nnz);
  M->vals = (MTYPE*)std::calloc(M->nnz, sizeof(MTYPE));
  for (int i = 0; i < nx; i++)
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++) {
        const int n = (i * nz + k) * ny + j;
        int o[3] = {M->rowOffsets[3 * n], M->rowOffsets[3 * n + 1], M->rowOffsets[3 * n + 2]};
        for (int ii = std::max(i - 1, 0); ii < std::min(i + 2, nx); ii++)
          for (int kk = std::max(k - 1, 0); kk < std::min(k + 2, nz); kk++)
            for (int jj = std::max(j - 1, 0); jj < std::min(j + 2, ny); jj++) {
              const int m = (ii * nz + kk) * ny + jj;
              for (int a = 0; a < 3; a++)
                for (int b2 = 0; b2 < 3; b2++) M->colIndex[o[a] + b2] = 3 * m + b2;
              for (int a = 0; a < 3; a++) o[a] += 3;
            }
      }
}

void freeSubspaceMatrix(struct CSRMatrix* M) {
  std::free(M->rowOffsets);
  std::free(M->vals);
  std::free(M->colIndex);
}

void assembleSubspaceMatrix(const struct gridContext gc, const int l, const DTYPE* x, struct CSRMatrix M,
                            MTYPE* tmp) {
  tp_ctx* c = ctx_levels(gc, l + 1);
  set_design(c, gc, x);
  check(c, tp_assemble(c), "assemble");
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  const int nx = d.ex + 1, ny = d.ey + 1, nz = d.ez + 1;
  const long nn = (long)nx * ny * nz;
  std::vector<double> A(243 * nn);
  // the V-cycle's stencil of a level >= 2 already carries the CSR's BCs; at
  // level 1 the CSR is assembled from the same sums with them applied here
  check(c, tp_download_stencil(c, l, 0, A.data()), "download stencil");
  std::vector<char> fixed(3 * nn, 0);
  const int lim = d.ey / 4 + 1;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      if (j < lim || j >= ny - lim)
        for (int a = 0; a < 3; a++) fixed[3 * ((0L * nz + k) * ny + j) + a] = 1;
  for (int i = 0; i < nx; i++)
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++) {
        const long n = ((long)i * nz + k) * ny + j;
        for (int a = 0; a < 3; a++) {
          const long row = 3 * n + a;
          int q = M.rowOffsets[row];
          for (int ii = std::max(i - 1, 0); ii < std::min(i + 2, nx); ii++)
            for (int kk = std::max(k - 1, 0); kk < std::min(k + 2, nz); kk++)
              for (int jj = std::max(j - 1, 0); jj < std::min(j + 2, ny); jj++) {
                const int m = (ii - i + 1) * 9 + (kk - k + 1) * 3 + (jj - j + 1);
                const long nm = ((long)ii * nz + kk) * ny + jj;
                for (int b2 = 0; b2 < 3; b2++, q++) {
                  double v = A[(m * 9 + 3 * a + b2) * nn + n];
                  if (fixed[row] || fixed[3 * nm + b2]) v = (3 * nm + b2 == row) ? 1.0 : 0.0;
                  M.vals[q] = v;
                }
              }
        }
      }
  for (int r = 0; r < M.nrows; r++) tmp[r] = fixed[r] ? 0.0 : 1.0;
}

void initializeCholmod(const struct gridContext gc, const int l, struct CoarseSolverData* solverData,
                       const struct CSRMatrix M) {
  (void)M;
  std::memset(solverData, 0, sizeof(*solverData));
  solverData->handle = ctx_for((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l + 1);
}

void finishCholmod(const struct gridContext gc, const int l, struct CoarseSolverData* solverData,
                   const struct CSRMatrix M, const int verbose) {
  (void)gc; (void)l; (void)M;
  if (verbose == 1) std::printf("coarse solver: GPU band Cholesky (FP64)\n");
  solverData->handle = nullptr;
}

void factorizeSubspaceMatrix(const struct gridContext gc, const int l, struct CoarseSolverData solverData,
                             const struct CSRMatrix M) {
  tp_ctx* c = solverData.handle ? (tp_ctx*)solverData.handle : ctx_for((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l + 1);
  check(c, tp_coarse_factor_csr(c, M.nrows, M.rowOffsets, M.colIndex, M.vals), "factorizeSubspaceMatrix");
}

void solveSubspaceMatrix(const struct gridContext gc, const int l, struct CoarseSolverData solverData,
                         const CTYPE* in, CTYPE* out) {
  tp_ctx* c = solverData.handle ? (tp_ctx*)solverData.handle : ctx_for((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l + 1);
  const Dims d = dims_of((int)gc.nelx, (int)gc.nely, (int)gc.nelz, l);
  const HVec h = to_canon(d, in);
  double* din = up(0, h);
  double* dout = g_s[1].get(h.size());
  check(c, tp_coarse_solve_factored(c, din, dout), "solveSubspaceMatrix");
  from_canon(d, down(dout, h.size()), out);
}

// ---------------------------------------------------------------------------
// gpu_definitions.h: volume, change, OC update on the GPU
DTYPE compute_volume(const struct gridContext gc, DTYPE* xPhys) {
  tp_ctx* c = ctx_levels(gc, 2);
  const long n = (long)gc.nelx * gc.nely * gc.nelz;
  double* d = g_s[0].get(n);
  up_elems(d, gc, xPhys);
  double s = 0;
  check(c, tp_vec_sum(c, n, d, &s), "compute_volume");
  return (DTYPE)s;
}

// max |x - xnew| (exact in any order) and x <- xnew, on the host: the arrays
// are there already, and the copy back was the reference's host loop
float compute_change(DTYPE* x, DTYPE* xnew, const int nelem) {
  double ch = 0.0;
#pragma omp parallel for schedule(static) reduction(max : ch)
  for (int e = 0; e < nelem; e++) {
    const double dd = std::fabs((double)x[e] - (double)xnew[e]);
    ch = dd > ch ? dd : ch;
    x[e] = xnew[e];
  }
  return (float)ch;
}

void update_solution(const DTYPE* x, DTYPE* xnew, const DTYPE* dv, const DTYPE* dc, const int nelem,
                     const DTYPE g) {
  tp_ctx* c = g_ctx.empty() ? nullptr : g_ctx.begin()->second;
  if (!c) c = ctx_for(2, 2, 2, 2);
  double* dx = g_s[0].get(nelem);
  double* ddv = g_s[1].get(nelem);
  double* ddc = g_s[2].get(nelem);
  double* dn = g_s[3].get(nelem);
  up_plain(dx, x, nelem);
  up_plain(ddv, dv, nelem);
  up_plain(ddc, dc, nelem);
  check(c, tp_oc_bisect(c, nelem, dx, ddv, ddc, (double)g, dn), "update_solution");
  down_plain(dn, xnew, nelem);
}

// ---------------------------------------------------------------------------
// stencil_optimization.h
void applyDensityFilter(const struct gridContext gc, const DTYPE rmin, const DTYPE* rho, DTYPE* out) {
  tp_ctx* c = ctx_levels(gc, 2);
  check(c, tp_set_rmin(c, (double)rmin), "set rmin");
  const long n = (long)gc.nelx * gc.nely * gc.nelz;
  double* din = g_s[0].get(n);
  double* dout = g_s[1].get(n);
  up_elems(din, gc, rho);
  check(c, tp_filter(c, din, dout), "applyDensityFilter");
  down_elems(dout, gc, out);
}

void applyDensityFilterGradient(const struct gridContext gc, const DTYPE rmin, DTYPE* v) {
  tp_ctx* c = ctx_levels(gc, 2);
  check(c, tp_set_rmin(c, (double)rmin), "set rmin");
  const long n = (long)gc.nelx * gc.nely * gc.nelz;
  double* dv = g_s[0].get(n);
  up_elems(dv, gc, v);
  check(c, tp_filter_T(c, dv), "applyDensityFilterGradient");
  down_elems(dv, gc, v);
}

static void vtk_write(FILE* f, int wx, int wy, int wz, int ex, int ey, int ez, int e0, const DTYPE* dens,
                      int elwy, int elwz) {
  std::fprintf(f, "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
  std::fprintf(f, "<UnstructuredGrid>\n");
  std::fprintf(f, "<Piece NumberOfPoints=\"%i\" NumberOfCells=\"%i\">\n", wx * wy * wz, ex * ey * ez);
  std::fprintf(f, "<Points>\n");
  std::fprintf(f, "<DataArray type=\"Float32\" NumberOfComponents=\"%i\" format=\"ascii\">\n", 3);
  for (int i = 0; i < wx; i++)
    for (int k = 0; k < wz; k++)
      for (int j = 0; j < wy; j++) std::fprintf(f, "%e %e %e\n", (float)i, (float)j, (float)k);
  std::fprintf(f, "</DataArray>\n</Points>\n<Cells>\n");
  std::fprintf(f, "<DataArray type=\"Int32\" Name=\"connectivity\" format= \"ascii\">\n");
  for (int i = 0; i < ex; i++)
    for (int k = 0; k < ez; k++)
      for (int j = 0; j < ey; j++) {
        auto N = [&](int a, int c, int b) { return a * wy * wz + c * wy + b; };
        std::fprintf(f, "%d %d %d %d %d %d %d %d\n", N(i, k, j + 1), N(i + 1, k, j + 1), N(i + 1, k, j),
                     N(i, k, j), N(i, k + 1, j + 1), N(i + 1, k + 1, j + 1), N(i + 1, k + 1, j), N(i, k + 1, j));
      }
  std::fprintf(f, "</DataArray>\n");
  std::fprintf(f, "<DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n");
  for (int i = 1; i < ex * ey * ez + 1; i++) std::fprintf(f, "%d\n", i * 8);
  std::fprintf(f, "</DataArray>\n");
  std::fprintf(f, "<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n");
  for (int i = 0; i < ex * ey * ez; i++) std::fprintf(f, "%d\n", 12);
  std::fprintf(f, "</DataArray>\n</Cells>\n<CellData>\n");
  std::fprintf(f, "<DataArray type=\"Float32\" NumberOfComponents=\"1\" Name=\"density\" format=\"ascii\">\n");
  for (int i = e0; i < ex + e0; i++)
    for (int k = e0; k < ez + e0; k++)
      for (int j = e0; j < ey + e0; j++) std::fprintf(f, "%e\n", (double)dens[(long)i * elwy * elwz + (long)k * elwy + j]);
  std::fprintf(f, "</DataArray>\n</CellData>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n");
}

// ASCII .vtu of the density field without / with the halo
// (stencil_optimization.c:399-598)
void writeDensityVtkFile(const int nelx, const int nely, const int nelz, const DTYPE* densityArray,
                         const char* filename) {
  const Dims d = dims_of(nelx, nely, nelz, 0);
  FILE* f = std::fopen(filename, "w");
  if (!f) return;
  vtk_write(f, nelx + 1, nely + 1, nelz + 1, nelx, nely, nelz, 1, densityArray, d.wy - 1, d.wz - 1);
  std::fclose(f);
}

void writeDensityVtkFileWithHalo(const int nelx, const int nely, const int nelz, const DTYPE* densityArray,
                                 const char* filename) {
  const Dims d = dims_of(nelx, nely, nelz, 0);
  FILE* f = std::fopen(filename, "w");
  if (!f) return;
  vtk_write(f, d.wx, d.wy, d.wz, d.wx - 1, d.wy - 1, d.wz - 1, 0, densityArray, d.wy - 1, d.wz - 1);
  std::fclose(f);
}

// The design loop of stencil_optimization.c:13-223 on the GPU, with the
// reference's console output. cgmax is accepted and, as in the reference,
// not used (the CG cap is 1000, stencil_solvers.c:334).
void top3dmgcg(const uint_fast32_t nelx, const uint_fast32_t nely, const uint_fast32_t nelz, const DTYPE volfrac,
               const DTYPE rmin, const uint_fast32_t nl, const float cgtol, const uint_fast32_t cgmax,
               const int verbose, const int write_result, const int max_iterations) {
  (void)cgmax;
  tp_params p;
  tp_default_params(&p);
  p.nelx = (int)nelx;
  p.nely = (int)nely;
  p.nelz = (int)nelz;
  p.nl = (int)nl;
  p.volfrac = (double)volfrac;
  p.rmin = (double)rmin;
  p.cgtol = (double)cgtol;
  p.precision = precision_from_env();
  tp_ctx* c = nullptr;
  tp_status st = tp_create(&p, &c);
  if (st != TP_OK) {
    std::fprintf(stderr, "top3dmgcg: %s (%s)\n", tp_status_string(st), c ? tp_error_message(c) : "");
    if (c) tp_destroy(c);
    return;
  }
  if (verbose == 1) std::printf("GPU: libtopopt_gb300, %s form\n", p.precision == TP_MIXED ? "mixed" : "FP64");
  const double t0 = omp_get_wtime();
  int loop = 0;
  float change = 1.0f;
  double cval = 0, vol = 0;
  int cg_total = 0;
  while (change > 1e-2 && loop < max_iterations) {
    loop++;
    tp_iter_info info;
    st = tp_design_iteration(c, &info);
    check(c, st, "design iteration");
    change = (float)info.change;
    cval = info.c;
    vol = info.vol;
    cg_total += info.cgiters;
    if (verbose == 1) {
      std::printf("It.:%4i Obj.:%6.3e Vol.:%6.3f ch.:%4.2f relres: %4.2e iters: %4i ", loop, cval, vol, change,
                  info.relres, info.cgiters);
      std::printf("time: %6.3f \n", omp_get_wtime() - t0);
    }
  }
  std::printf("%4i %12.6f %6.3f %4.2f %9i %9i", loop, (DTYPE)cval, (DTYPE)vol, change, (int)(nelx * nely * nelz),
              cg_total);
  std::printf(" %6.3f \n", omp_get_wtime() - t0);
  if (verbose == 1) std::printf("End time: %6.3f \n", omp_get_wtime() - t0);
  if (write_result == 1) {
    const Dims d = dims_of((int)nelx, (int)nely, (int)nelz, 0);
    HVec xp(tp_nelem(c));
    check(c, tp_download(c, TP_FIELD_XPHYS, xp.data(), (long)xp.size()), "download xPhys");
  g_d2h += (long)(xp.size() * sizeof(double));
    std::vector<DTYPE> padded((size_t)(d.wx - 1) * (d.wy - 1) * (d.wz - 1), (DTYPE)0);
    gridContext gc;
    gc.nelx = nelx;
    gc.nely = nely;
    gc.nelz = nelz;
    gc.wrapx = d.wx;
    gc.wrapy = d.wy;
    gc.wrapz = d.wz;
    el_from_canon(gc, xp, padded.data());
    char n1[60], n2[60];
    std::snprintf(n1, 60, "out_%d_%d_%d.vtu", (int)nelx, (int)nely, (int)nelz);
    writeDensityVtkFile((int)nelx, (int)nely, (int)nelz, padded.data(), n1);
    std::snprintf(n2, 60, "out_%d_%d_%d_halo.vtu", (int)nelx, (int)nely, (int)nelz);
    writeDensityVtkFileWithHalo((int)nelx, (int)nely, (int)nelz, padded.data(), n2);
  }
  tp_destroy(c);
}

// bytes the entry points above have copied between host and device since the
// library was loaded (or last reset); no counterpart in the reference
void topopt_ref_transfer_bytes(long* h2d, long* d2h, int reset) {
  if (h2d) *h2d = g_h2d;
  if (d2h) *d2h = g_d2h;
  if (reset) g_h2d = g_d2h = 0;
}

}  // extern "C"
