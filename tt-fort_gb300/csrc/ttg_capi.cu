// extern "C" entry points of libttgpu: context, kernel-level calls on device
// pointers, result access.  Driver entry points (ttg_eigb, ttg_ksl_z,
// ttg_amen_solve) live beside their drivers.
#include "ttg_common.cuh"
#include <algorithm>
#include <cstring>
#include <cmath>

namespace ttg {

std::atomic<long long> g_launches{0};

bool pdl_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("TTG_PDL");
    return !(v && v[0] == '0');
  }();
  return on;
}

void Workspace::reserve(size_t bytes) {
  bytes = (bytes + 255) & ~size_t(255);
  if (bytes <= cap) return;
  if (base) {
    cudaFree(base);
    base = nullptr;
    cap = 0;
  }
  cudaError_t e = cudaMalloc(&base, bytes);
  if (e != cudaSuccess) {
    base = nullptr;
    throw Error{TTG_ERR_NOMEM, "workspace cudaMalloc failed"};
  }
  cap = bytes;
  top = 0;
}

void* Workspace::take(size_t bytes) {
  bytes = (bytes + 255) & ~size_t(255);
  if (top + bytes > cap) throw Error{TTG_ERR_NOMEM, "workspace exhausted"};
  void* p = base + top;
  top += bytes;
  return p;
}

void Workspace::release() {
  if (base) cudaFree(base);
  base = nullptr;
  cap = top = 0;
}

}  // namespace ttg

using namespace ttg;

#define TTG_API_BEGIN(ctx)                                \
  if (!(ctx)) return TTG_ERR_ARG;                         \
  try {                                                   \
    TTG_CUDA(cudaSetDevice((ctx)->device));
#define TTG_API_END(ctx)                                  \
  } catch (const ttg::Error& e) {                         \
    (ctx)->last_error = e.msg;                            \
    return e.code;                                        \
  } catch (const std::exception& e) {                     \
    (ctx)->last_error = e.what();                         \
    return TTG_ERR_ARG;                                   \
  }                                                       \
  return TTG_OK;

extern "C" {

int ttg_version(void) { return 10000; }

int ttg_create(int device, ttg_ctx** out) {
  if (!out) return TTG_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return TTG_ERR_CUDA;
  if (device < 0 || device >= n) return TTG_ERR_ARG;
  ttg_ctx* c = new ttg_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return TTG_ERR_CUDA;
  }
  c->own_stream = true;
  *out = c;
  return TTG_OK;
}

int ttg_destroy(ttg_ctx* c) {
  if (!c) return TTG_ERR_ARG;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->ws.release();
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return TTG_OK;
}

const char* ttg_last_error(const ttg_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

int ttg_set_stream(ttg_ctx* c, void* stream) {
  TTG_API_BEGIN(c)
  if ((cudaStream_t)stream == c->stream) return TTG_OK;
  if (c->own_stream && c->stream) {
    TTG_CUDA(cudaStreamSynchronize(c->stream));
    TTG_CUDA(cudaStreamDestroy(c->stream));
  }
  c->own_stream = false;
  c->stream = (cudaStream_t)stream;   // NULL: the legacy default stream
  TTG_API_END(c)
}

int ttg_synchronize(ttg_ctx* c) {
  TTG_API_BEGIN(c)
  TTG_CUDA(cudaStreamSynchronize(c->stream));
  TTG_API_END(c)
}

static void check_dims(ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n, ttg_int ry2,
                       ttg_int ra1, ttg_int ra2) {
  TTG_REQUIRE(rx1 > 0 && m > 0 && rx2 > 0 && ry1 > 0 && n > 0 && ry2 > 0 && ra1 > 0 && ra2 > 0,
              "all sizes must be positive");
  TTG_REQUIRE(rx1 * m * rx2 < (1ll << 31) && ry1 * n * ry2 < (1ll << 31),
              "local problem too large for 32-bit tile indexing");
}

int ttg_dbfun3(ttg_ctx* c, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
               ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1, const double* A,
               const double* phi2, const double* x, double* y, ttg_int nvec) {
  TTG_API_BEGIN(c)
  check_dims(rx1, m, rx2, ry1, n, ry2, ra1, ra2);
  TTG_REQUIRE(phi1 && A && phi2 && x && y && nvec > 0, "null pointer or nvec <= 0");
  LocalDims L{rx1, m, rx2, ry1, n, ry2, ra1, ra2};
  c->ws.reset();
  c->ws.reserve(bfun3_f64_scratch(L, (int)nvec));
  double* scr = c->ws.takeT<double>(bfun3_f64_scratch(L, (int)nvec) / sizeof(double));
  bfun3_f64(L, phi1, A, phi2, x, y, (int)nvec, scr, c->stream);
  TTG_API_END(c)
}

int ttg_zbfun3(ttg_ctx* c, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
               ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1, const double* A,
               const double* phi2, const double* x, double* y, ttg_int nvec) {
  TTG_API_BEGIN(c)
  check_dims(rx1, m, rx2, ry1, n, ry2, ra1, ra2);
  TTG_REQUIRE(phi1 && A && phi2 && x && y && nvec > 0, "null pointer or nvec <= 0");
  LocalDims L{rx1, m, rx2, ry1, n, ry2, ra1, ra2};
  size_t bytes = 2 * bfun3_f64_scratch(L, (int)nvec);
  c->ws.reset();
  c->ws.reserve(bytes);
  double2* scr = (double2*)c->ws.take(bytes);
  bfun3_z(L, (const double2*)phi1, (const double2*)A, (const double2*)phi2, (const double2*)x,
          (double2*)y, (int)nvec, scr, c->stream);
  TTG_API_END(c)
}

int ttg_zbfun3_transp(ttg_ctx* c, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
                      ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1,
                      const double* A, const double* phi2, const double* x, double* y,
                      ttg_int nvec) {
  TTG_API_BEGIN(c)
  check_dims(rx1, m, rx2, ry1, n, ry2, ra1, ra2);
  TTG_REQUIRE(phi1 && A && phi2 && x && y && nvec > 0, "null pointer or nvec <= 0");
  LocalDims L{rx1, m, rx2, ry1, n, ry2, ra1, ra2};
  size_t bytes = (size_t)(rx1 * ra1 * n * ry2 + rx1 * m * ra2 * ry2) * nvec * sizeof(double2);
  c->ws.reset();
  c->ws.reserve(bytes);
  double2* scr = (double2*)c->ws.take(bytes);
  bfun3_transp_z(L, (const double2*)phi1, (const double2*)A, (const double2*)phi2,
                 (const double2*)x, (double2*)y, (int)nvec, scr, c->stream);
  TTG_API_END(c)
}

int ttg_dphi_left(ttg_ctx* c, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
                  ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1_old,
                  const double* A, const double* x, const double* y, double* phi1_new) {
  TTG_API_BEGIN(c)
  check_dims(rx1, m, rx2, ry1, n, ry2, ra1, ra2);
  TTG_REQUIRE(phi1_old && A && x && y && phi1_new, "null pointer");
  LocalDims L{rx1, m, rx2, ry1, n, ry2, ra1, ra2};
  c->ws.reset();
  c->ws.reserve(phi_f64_scratch(L));
  double* scr = (double*)c->ws.take(phi_f64_scratch(L));
  phi_left_f64(L, phi1_old, A, x, y, phi1_new, scr, c->stream);
  TTG_API_END(c)
}

int ttg_dphi_right(ttg_ctx* c, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
                   ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi2_old,
                   const double* A, const double* x, const double* y, double* phi2_new) {
  TTG_API_BEGIN(c)
  check_dims(rx1, m, rx2, ry1, n, ry2, ra1, ra2);
  TTG_REQUIRE(phi2_old && A && x && y && phi2_new, "null pointer");
  LocalDims L{rx1, m, rx2, ry1, n, ry2, ra1, ra2};
  c->ws.reset();
  c->ws.reserve(phi_f64_scratch(L));
  double* scr = (double*)c->ws.take(phi_f64_scratch(L));
  phi_right_f64(L, phi2_old, A, x, y, phi2_new, scr, c->stream);
  TTG_API_END(c)
}

int ttg_zphi_left(ttg_ctx* c, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
                  ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1_old,
                  const double* A, const double* x, const double* y, double* phi1_new) {
  TTG_API_BEGIN(c)
  check_dims(rx1, m, rx2, ry1, n, ry2, ra1, ra2);
  TTG_REQUIRE(phi1_old && A && x && y && phi1_new, "null pointer");
  LocalDims L{rx1, m, rx2, ry1, n, ry2, ra1, ra2};
  c->ws.reset();
  c->ws.reserve(phi_f64_scratch(L) * 2);
  double2* scr = (double2*)c->ws.take(phi_f64_scratch(L) * 2);
  phi_left_z(L, (const double2*)phi1_old, (const double2*)A, (const double2*)x,
             (const double2*)y, (double2*)phi1_new, scr, c->stream);
  TTG_API_END(c)
}

int ttg_zphi_right(ttg_ctx* c, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
                   ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi2_old,
                   const double* A, const double* x, const double* y, double* phi2_new) {
  TTG_API_BEGIN(c)
  check_dims(rx1, m, rx2, ry1, n, ry2, ra1, ra2);
  TTG_REQUIRE(phi2_old && A && x && y && phi2_new, "null pointer");
  LocalDims L{rx1, m, rx2, ry1, n, ry2, ra1, ra2};
  c->ws.reset();
  c->ws.reserve(phi_f64_scratch(L) * 2);
  double2* scr = (double2*)c->ws.take(phi_f64_scratch(L) * 2);
  phi_right_z(L, (const double2*)phi2_old, (const double2*)A, (const double2*)x,
              (const double2*)y, (double2*)phi2_new, scr, c->stream);
  TTG_API_END(c)
}

int ttg_dphi2_left(ttg_ctx* c, ttg_int rx1, ttg_int rx2, ttg_int ry1, ttg_int n, ttg_int ry2,
                   const double* phi1_old, const double* x, const double* y, double* phi1_new) {
  TTG_API_BEGIN(c)
  TTG_REQUIRE(rx1 > 0 && rx2 > 0 && ry1 > 0 && n > 0 && ry2 > 0, "sizes must be positive");
  TTG_REQUIRE(phi1_old && x && y && phi1_new, "null pointer");
  size_t bytes = (size_t)rx1 * n * ry2 * sizeof(double);
  c->ws.reset();
  c->ws.reserve(bytes);
  double* scr = (double*)c->ws.take(bytes);
  phi2_left_f64(rx1, rx2, ry1, n, ry2, phi1_old, x, y, phi1_new, scr, c->stream);
  TTG_API_END(c)
}

int ttg_dphi2_right(ttg_ctx* c, ttg_int rx1, ttg_int rx2, ttg_int ry1, ttg_int n, ttg_int ry2,
                    const double* phi2_old, const double* x, const double* y, double* phi2_new) {
  TTG_API_BEGIN(c)
  TTG_REQUIRE(rx1 > 0 && rx2 > 0 && ry1 > 0 && n > 0 && ry2 > 0, "sizes must be positive");
  TTG_REQUIRE(phi2_old && x && y && phi2_new, "null pointer");
  size_t bytes = (size_t)rx1 * n * ry2 * sizeof(double);
  c->ws.reset();
  c->ws.reserve(bytes);
  double* scr = (double*)c->ws.take(bytes);
  phi2_right_f64(rx1, rx2, ry1, n, ry2, phi2_old, x, y, phi2_new, scr, c->stream);
  TTG_API_END(c)
}

int ttg_d2d_fullmat(ttg_ctx* c, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ra1, ttg_int ra2,
                    const double* phi1, const double* A, const double* phi2, double* B) {
  TTG_API_BEGIN(c)
  TTG_REQUIRE(rx1 > 0 && m > 0 && rx2 > 0 && ra1 > 0 && ra2 > 0, "sizes must be positive");
  TTG_REQUIRE(phi1 && A && phi2 && B, "null pointer");
  fullmat_f64(rx1, m, rx2, ra1, ra2, phi1, A, phi2, B, c->stream);
  TTG_API_END(c)
}

int ttg_dqr(ttg_ctx* c, ttg_int n, ttg_int m, double* A, double* R) {
  TTG_API_BEGIN(c)
  TTG_REQUIRE(n > 0 && m > 0 && A && R, "bad arguments");
  TTG_REQUIRE(n < (1ll << 31) && m < (1ll << 31), "size too large");
  c->ws.reset();
  c->ws.reserve(sizeof(double) * std::min(n, m));
  double* tau = c->ws.takeT<double>(std::min(n, m));
  qr_householder((int)n, (int)m, A, R, tau, c->stream);
  TTG_API_END(c)
}

int ttg_zqr(ttg_ctx* c, ttg_int n, ttg_int m, double* A, double* R) {
  TTG_API_BEGIN(c)
  TTG_REQUIRE(n > 0 && m > 0 && A && R, "bad arguments");
  TTG_REQUIRE(n < (1ll << 31) && m < (1ll << 31), "size too large");
  c->ws.reset();
  c->ws.reserve(sizeof(double2) * std::min(n, m));
  double2* tau = c->ws.takeT<double2>(std::min(n, m));
  qr_householder_z((int)n, (int)m, (double2*)A, (double2*)R, tau, c->stream);
  TTG_API_END(c)
}

int ttg_dsyev(ttg_ctx* c, ttg_int k, double* A, double* w) {
  TTG_API_BEGIN(c)
  TTG_REQUIRE(k > 0 && k <= 512 && A && w, "bad arguments (k <= 512)");
  c->ws.reset();
  c->ws.reserve(sizeof(double) * (2 * k * k + 64));
  double* V = c->ws.takeT<double>(k * k);
  double* Aw = c->ws.takeT<double>(k * k);
  int* st = c->ws.takeT<int>(16);
  TTG_CUDA(cudaMemcpyAsync(Aw, A, sizeof(double) * k * k, cudaMemcpyDeviceToDevice, c->stream));
  syev_jacobi((int)k, Aw, (int)k, w, V, (int)k, st, c->stream);
  TTG_CUDA(cudaMemcpyAsync(A, V, sizeof(double) * k * k, cudaMemcpyDeviceToDevice, c->stream));
  TTG_API_END(c)
}

int ttg_dgesvd(ttg_ctx* c, ttg_int p, ttg_int q, const double* M, double* U, double* s,
               double* Vt) {
  TTG_API_BEGIN(c)
  TTG_REQUIRE(p > 0 && q > 0 && M && U && s && Vt, "bad arguments");
  TTG_REQUIRE(p < (1ll << 31) && q < (1ll << 31), "size too large");
  c->ws.reset();
  size_t bytes = svd_scratch((int)p, (int)q) + 256;
  c->ws.reserve(bytes);
  double* scr = (double*)c->ws.take(svd_scratch((int)p, (int)q));
  int* st = (int*)c->ws.take(64);
  svd_jacobi((int)p, (int)q, M, U, s, Vt, scr, st, c->stream);
  TTG_API_END(c)
}

ttg_int ttg_my_chop3(ttg_int n, const double* s, double eps) {
  if (n <= 0 || !s) return 0;
  double nrm = 0.0;
  for (ttg_int i = 0; i < n; ++i) nrm += s[i] * s[i];
  nrm = std::sqrt(nrm);
  nrm = (nrm * eps) * (nrm * eps);
  double cursum = 0.0;
  ttg_int i = n;
  while (i > 0) {
    cursum += s[i - 1] * s[i - 1];
    if (cursum > nrm) break;
    --i;
  }
  return std::min(i + 1, n);
}

int ttg_result_size(const ttg_ctx* c, ttg_int* nelem) {
  if (!c || !nelem) return TTG_ERR_ARG;
  *nelem = (ttg_int)std::max(c->result_core.size(), c->zresult_core.size());
  return TTG_OK;
}

int ttg_result_copy(const ttg_ctx* c, double* out, ttg_int nelem) {
  if (!c || !out || nelem < (ttg_int)c->result_core.size()) return TTG_ERR_ARG;
  std::memcpy(out, c->result_core.data(), c->result_core.size() * sizeof(double));
  return TTG_OK;
}

int ttg_zresult_copy(const ttg_ctx* c, double* out, ttg_int nelem) {
  if (!c || !out || nelem < (ttg_int)c->zresult_core.size()) return TTG_ERR_ARG;
  std::memcpy(out, c->zresult_core.data(), c->zresult_core.size() * sizeof(double) * 2);
  return TTG_OK;
}

int ttg_free_result(ttg_ctx* c) {
  if (!c) return TTG_ERR_ARG;
  c->result_core.clear();
  c->result_core.shrink_to_fit();
  c->zresult_core.clear();
  c->zresult_core.shrink_to_fit();
  return TTG_OK;
}

int ttg_stats(const ttg_ctx* c, ttg_int* matvecs, ttg_int* sweeps, double* res,
              ttg_int* launches) {
  if (!c) return TTG_ERR_ARG;
  if (matvecs) *matvecs = c->stat_matvecs;
  if (sweeps) *sweeps = c->stat_sweeps;
  if (res) *res = c->stat_res;
  if (launches) *launches = c->stat_launches;
  return TTG_OK;
}

int ttg_set_limits(ttg_ctx* c, ttg_int max_matvecs, ttg_int max_expokit_steps, int strict) {
  if (!c || max_matvecs < 0 || max_expokit_steps < 0) return TTG_ERR_ARG;
  c->lim_matvecs = (int)std::min<ttg_int>(max_matvecs, 1 << 30);
  c->lim_expsteps = (int)std::min<ttg_int>(max_expokit_steps, 1 << 30);
  c->strict = strict ? 1 : 0;
  return TTG_OK;
}

ttg_int ttg_capped(const ttg_ctx* c) { return c ? (ttg_int)c->stat_capped : -1; }

/* total kernel launches issued by this library in this process */
ttg_int ttg_launch_count(void) { return (ttg_int)ttg::g_launches.load(); }

}  // extern "C"
