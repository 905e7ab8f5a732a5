// Checkpoint and restart of the design loop's state (no counterpart in the
// reference, whose runs are short enough not to need it; long multi-load
// runs do).
//
// File layout, native little-endian, no padding between fields:
//   char     magic[8]   "TPCKPT1" and a zero byte
//   int32    version    1
//   int32    nelx, nely, nelz, nl, nrhs, precision, loop
//   int32    reserved   0
//   float64  volfrac, rmin
//   int64    nelem      nelx*nely*nelz
//   int64    ndof       3*(nelx+1)*(nely+1)*(nelz+1), per load case
//   uint64   checksum   FNV-1a (64-bit) over the payload bytes
// payload (float64): x[nelem], xPhys[nelem], U[nrhs*ndof], F[nrhs*ndof]
//
// The file is written to <path>.tmp and renamed over <path>, so an
// interrupted save leaves the previous checkpoint intact.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tp_internal.h"

namespace {

#pragma pack(push, 1)
struct CkptHeader {
  char magic[8];
  int32_t version;
  int32_t nelx, nely, nelz, nl, nrhs, precision, loop;
  int32_t reserved;
  double volfrac, rmin;
  int64_t nelem, ndof;
  uint64_t checksum;
};
#pragma pack(pop)
static_assert(sizeof(CkptHeader) == 8 + 4 * 9 + 8 * 2 + 8 * 2 + 8, "packed header");

const char kMagic[8] = {'T', 'P', 'C', 'K', 'P', 'T', '1', '\0'};

uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 0x100000001B3ull;
  }
  return h;
}
constexpr uint64_t kFnvBasis = 0xCBF29CE484222325ull;

// reads and checks a header and, with payload != nullptr, the payload too
tp_status read_file(const char* path, CkptHeader* h, std::vector<double>* payload) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return TP_ERR_ARG;
  tp_status st = TP_OK;
  // the payload's size follows from the header; it is checked against the
  // file's length before anything is allocated, so a corrupt header with
  // large, consistent dimensions is refused instead of sizing a huge buffer
  long file_bytes = -1;
  if (std::fseek(f, 0, SEEK_END) == 0) file_bytes = std::ftell(f);
  std::rewind(f);
  if (std::fread(h, sizeof(*h), 1, f) != 1 || std::memcmp(h->magic, kMagic, 8) != 0 || h->version != 1 ||
      h->nelx < 1 || h->nely < 1 || h->nelz < 1 || h->nrhs < 1 || h->nrhs > 16 ||
      h->nelem != (int64_t)h->nelx * h->nely * h->nelz ||
      h->ndof != 3LL * (h->nelx + 1) * (h->nely + 1) * (h->nelz + 1))
    st = TP_ERR_ARG;
  const int64_t n64 = st == TP_OK ? 2 * h->nelem + 2 * (int64_t)h->nrhs * h->ndof : 0;
  if (st == TP_OK && (file_bytes < 0 || n64 != ((int64_t)file_bytes - (int64_t)sizeof(*h)) / (int64_t)sizeof(double)))
    st = TP_ERR_ARG;
  if (st == TP_OK) {
    const size_t n = (size_t)n64;
    std::vector<double> buf(n);
    if (std::fread(buf.data(), sizeof(double), n, f) != n || std::fgetc(f) != EOF ||
        fnv1a(kFnvBasis, buf.data(), n * sizeof(double)) != h->checksum)
      st = TP_ERR_ARG;
    else if (payload)
      payload->swap(buf);
  }
  std::fclose(f);
  return st;
}

}  // namespace

extern "C" {

tp_status tp_checkpoint_save(tp_ctx* c, const char* path, int loop) {
  if (!c || !path) return TP_ERR_ARG;
  const long ne = tp_nelem(c), nd = tp_ndof(c, 0) * c->p.nrhs;
  std::vector<double> buf(2 * ne + 2 * nd);
  tp_status st = tp_download(c, TP_FIELD_X, buf.data(), ne);
  if (st == TP_OK) st = tp_download(c, TP_FIELD_XPHYS, buf.data() + ne, ne);
  if (st == TP_OK) st = tp_download(c, TP_FIELD_U, buf.data() + 2 * ne, nd);
  if (st == TP_OK) st = tp_download(c, TP_FIELD_F, buf.data() + 2 * ne + nd, nd);
  if (st != TP_OK) return st;
  CkptHeader h;
  std::memset(&h, 0, sizeof h);
  std::memcpy(h.magic, kMagic, 8);
  h.version = 1;
  h.nelx = c->p.nelx;
  h.nely = c->p.nely;
  h.nelz = c->p.nelz;
  h.nl = c->p.nl;
  h.nrhs = c->p.nrhs;
  h.precision = c->p.precision;
  h.loop = loop;
  h.volfrac = c->p.volfrac;
  h.rmin = c->p.rmin;
  h.nelem = ne;
  h.ndof = tp_ndof(c, 0);
  h.checksum = fnv1a(kFnvBasis, buf.data(), buf.size() * sizeof(double));
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) {
    c->note = "checkpoint: cannot open " + tmp;
    return TP_ERR_ARG;
  }
  const bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 &&
                  std::fwrite(buf.data(), sizeof(double), buf.size(), f) == buf.size();
  if (std::fclose(f) != 0 || !ok || std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    c->note = std::string("checkpoint: writing ") + path + " failed";
    return TP_ERR_ARG;
  }
  return TP_OK;
}

tp_status tp_checkpoint_load(tp_ctx* c, const char* path, int* loop) {
  if (!c || !path) return TP_ERR_ARG;
  CkptHeader h;
  std::vector<double> buf;
  if (read_file(path, &h, &buf) != TP_OK) {
    c->note = std::string("checkpoint: ") + path + " is missing, truncated or corrupt";
    return TP_ERR_ARG;
  }
  if (h.nelx != c->p.nelx || h.nely != c->p.nely || h.nelz != c->p.nelz || h.nrhs != c->p.nrhs) {
    c->note = "checkpoint: grid or load-case count differs from the context's";
    return TP_ERR_ARG;
  }
  const long ne = h.nelem, nd = (long)h.ndof * h.nrhs;
  tp_status st = tp_upload(c, TP_FIELD_X, buf.data(), ne);
  if (st == TP_OK) st = tp_upload(c, TP_FIELD_XPHYS, buf.data() + ne, ne);
  if (st == TP_OK) st = tp_upload(c, TP_FIELD_U, buf.data() + 2 * ne, nd);
  if (st == TP_OK) st = tp_upload(c, TP_FIELD_F, buf.data() + 2 * ne + nd, nd);
  if (st == TP_OK && loop) *loop = h.loop;
  return st;
}

tp_status tp_checkpoint_info(const char* path, int* info) {
  if (!path || !info) return TP_ERR_ARG;
  CkptHeader h;
  const tp_status st = read_file(path, &h, nullptr);
  if (st != TP_OK) return st;
  const int v[7] = {h.nelx, h.nely, h.nelz, h.nl, h.nrhs, h.precision, h.loop};
  std::memcpy(info, v, sizeof v);
  return TP_OK;
}

}  // extern "C"
