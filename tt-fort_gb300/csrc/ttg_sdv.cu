// The reference's binary TT file format (.sdv), host side: dtt_write /
// ztt_write and dtt_read / ztt_read (ttio.f90:29-399), so tensors move
// between this library and Fortran-side code without the dtt/ztt types.
//
// Layout (stream access, native byte order):
//   header, 128 bytes: 'TT' + 6 blanks, int32 version (1, 0), int32 info
//     (tt_size = 1023, 0, 0, 0), 64-byte comment (written as zeros), int32
//     i(8) with i(1) = l, i(2) = m (ttio.f90:10-17,71-72)
//   int32 l, m (first and last mode, 1-based)
//   int32 n(l:m), int32 r(l-1:m)
//   the cores back to back, each r(k-1) x n(k) x r(k) column-major, float64
//   (dtt) or complex128 (ztt); the file does not say which.
// The reader checks the 'TT' magic and version 1 as dtt_read does.
#include "ttg_common.cuh"
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

constexpr int kTTSize = 1023;   // tt_size of tt.f90:9, the largest d

struct FileGuard {
  FILE* f;
  ~FileGuard() { if (f) fclose(f); }
};

}  // namespace

extern "C" int ttg_sdv_write(const char* path, ttg_int d, const ttg_int* n, const ttg_int* r,
                             const double* cores, int is_complex) {
  if (!path || !n || !r || !cores || d < 1 || d > kTTSize) return TTG_ERR_ARG;
  for (ttg_int k = 0; k < d; ++k)
    if (n[k] < 1 || n[k] > INT32_MAX || r[k] < 1 || r[k] > INT32_MAX) return TTG_ERR_ARG;
  if (r[d] < 1 || r[d] > INT32_MAX) return TTG_ERR_ARG;
  unsigned char head[128];
  std::memset(head, 0, sizeof(head));
  std::memcpy(head, "TT      ", 8);
  const int32_t ver[2] = {1, 0}, inf[4] = {kTTSize, 0, 0, 0};
  std::memcpy(head + 8, ver, 8);
  std::memcpy(head + 16, inf, 16);
  int32_t hi[8] = {1, (int32_t)d, 0, 0, 0, 0, 0, 0};
  std::memcpy(head + 96, hi, 32);
  FileGuard g{fopen(path, "wb")};
  if (!g.f) return TTG_ERR_ARG;
  const int32_t lm[2] = {1, (int32_t)d};
  std::vector<int32_t> nr(2 * d + 1);
  for (ttg_int k = 0; k < d; ++k) nr[k] = (int32_t)n[k];
  for (ttg_int k = 0; k <= d; ++k) nr[d + k] = (int32_t)r[k];
  size_t elems = 0;
  for (ttg_int k = 0; k < d; ++k) elems += (size_t)r[k] * n[k] * r[k + 1];
  const size_t scalars = elems * (is_complex ? 2 : 1);
  if (fwrite(head, 1, 128, g.f) != 128 || fwrite(lm, 4, 2, g.f) != 2 ||
      fwrite(nr.data(), 4, nr.size(), g.f) != nr.size() ||
      fwrite(cores, sizeof(double), scalars, g.f) != scalars)
    return TTG_ERR_ARG;
  if (fclose(g.f) != 0) { g.f = nullptr; return TTG_ERR_ARG; }
  g.f = nullptr;
  return TTG_OK;
}

extern "C" int ttg_sdv_read(const char* path, int is_complex, ttg_int* d, ttg_int* n, ttg_int* r,
                            ttg_int nmax, double* cores, ttg_int* nelem) {
  if (!path || !d || !nelem) return TTG_ERR_ARG;
  FileGuard g{fopen(path, "rb")};
  if (!g.f) return TTG_ERR_ARG;
  unsigned char head[128];
  if (fread(head, 1, 128, g.f) != 128) return TTG_ERR_ARG;
  if (head[0] != 'T' || head[1] != 'T') return TTG_ERR_ARG;          // not a TT file
  int32_t ver[2];
  std::memcpy(ver, head + 8, 8);
  if (ver[0] != 1) return TTG_ERR_ARG;                                // wrong version
  int32_t lm[2];
  if (fread(lm, 4, 2, g.f) != 2) return TTG_ERR_ARG;
  const int64_t dd = (int64_t)lm[1] - lm[0] + 1;
  if (dd < 1 || dd > kTTSize) return TTG_ERR_ARG;
  std::vector<int32_t> nr(2 * dd + 1);
  if (fread(nr.data(), 4, nr.size(), g.f) != nr.size()) return TTG_ERR_ARG;
  *d = dd;
  size_t elems = 0;
  for (int64_t k = 0; k < dd; ++k) {
    if (nr[k] < 1 || nr[dd + k] < 1 || nr[dd + k + 1] < 1) return TTG_ERR_ARG;
    elems += (size_t)nr[dd + k] * nr[k] * nr[dd + k + 1];
  }
  *nelem = (ttg_int)elems;
  if (n || r) {
    if (!n || !r || nmax < dd) return TTG_ERR_ARG;
    for (int64_t k = 0; k < dd; ++k) n[k] = nr[k];
    for (int64_t k = 0; k <= dd; ++k) r[k] = nr[dd + k];
  }
  if (cores) {
    const size_t scalars = elems * (is_complex ? 2 : 1);
    if (fread(cores, sizeof(double), scalars, g.f) != scalars) return TTG_ERR_ARG;
  }
  return TTG_OK;
}
