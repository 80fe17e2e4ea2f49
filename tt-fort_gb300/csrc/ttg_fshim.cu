// Reference-named, by-reference entry points for C and Fortran callers that
// bind tt-fort's bind(c) kernels directly (tt_linalg.f90:30,127,363,497).
//
// gmres_3d.c (gmres_3d.c:3-4) declares
//   void dbfun3(long*, long*, long*, long*, long*, long*, long*, long*,
//               double* phi1, double* A, double* phi2, double* x, double* y,
//               double* res1, double* res2);
//   void djac_apply(char*, long*, long*, long*, double* jacs, double* x,
//                   double* y, double* work1);
// and calls them with HOST arrays, once per Krylov step, sometimes in place
// (x == y, gmres_3d.c:61).  These shims have exactly those signatures, so
// such a caller links against libttgpu.so unchanged: each call copies its
// host inputs into a grow-only device buffer of the calling thread, runs the
// library's kernel (ttg_dbfun3, ttg_djac_gen, ttg_djac_apply, ttg_dqr) on a
// per-thread context, and copies the result back.  Integers are 64-bit
// (`long`, the reference's i8 presets, which gmres_3d.c assumes).  The
// res1/res2/work1/work/lwork/tau workspaces of the Fortran interfaces are
// accepted and left untouched (the device kernels have their own).
//
// This is the compatibility path: every call pays two host<->device copies
// and a stream synchronisation.  Callers that can hold device memory use the
// ttg_* entry points, which take device pointers and run asynchronously.
//
// The Fortran routines cannot report errors (they print and go on).  A failed
// shim call prints one line to stderr, fills its output with NaN (so the
// caller's next norm shows it) and records the status, which
// ttg_fshim_status() returns and clears.
#include "ttg_common.cuh"
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>

namespace {

struct ShimState {
  ttg_ctx* ctx = nullptr;
  double* buf = nullptr;
  size_t cap = 0;   // doubles
  int status = TTG_OK;
  ~ShimState() {
    if (buf) cudaFree(buf);
    if (ctx) ttg_destroy(ctx);
  }
};
thread_local ShimState g_shim;

// the calling thread's context (device $TTG_DEVICE, default 0) and a device
// buffer of at least n doubles
ttg_ctx* shim_ctx() {
  if (!g_shim.ctx) {
    const char* e = std::getenv("TTG_DEVICE");
    const int dev = e ? std::atoi(e) : 0;
    if (ttg_create(dev, &g_shim.ctx) != TTG_OK) {
      g_shim.ctx = nullptr;
      throw ttg::Error{TTG_ERR_CUDA, "cannot create a context on the device"};
    }
  }
  return g_shim.ctx;
}
double* shim_buf(size_t n) {
  if (n > g_shim.cap) {
    if (g_shim.buf) TTG_CUDA(cudaFree(g_shim.buf));
    g_shim.buf = nullptr;
    g_shim.cap = 0;
    TTG_CUDA(cudaMalloc(&g_shim.buf, n * sizeof(double)));
    g_shim.cap = n;
  }
  return g_shim.buf;
}
void up(double* d, const double* h, size_t n, cudaStream_t s) {
  TTG_CUDA(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, s));
}
void down(double* h, const double* d, size_t n, cudaStream_t s) {
  TTG_CUDA(cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, s));
}
void check(ttg_ctx* c, int rc) {
  if (rc != TTG_OK) throw ttg::Error{rc, ttg_last_error(c)};
}
void fail(const char* who, const ttg::Error& e, double* out, size_t n) {
  g_shim.status = e.code;
  std::fprintf(stderr, "%s (libttgpu): %s\n", who, e.msg.c_str());
  if (out)
    for (size_t i = 0; i < n; ++i) out[i] = std::numeric_limits<double>::quiet_NaN();
}

}  // namespace

extern "C" {

int ttg_fshim_status(void) {
  const int s = g_shim.status;
  g_shim.status = TTG_OK;
  return s;
}

void dbfun3(long* rx1, long* m, long* rx2, long* ry1, long* n, long* ry2, long* ra1, long* ra2,
            double* phi1, double* A, double* phi2, double* x, double* y, double* res1,
            double* res2) {
  (void)res1;
  (void)res2;
  size_t ny = 0;
  try {
    TTG_REQUIRE(rx1 && m && rx2 && ry1 && n && ry2 && ra1 && ra2, "null size");
    const size_t n1 = (size_t)*ry1 * *rx1 * *ra1, na = (size_t)*ra1 * *n * *m * *ra2,
                 n2 = (size_t)*rx2 * *ra2 * *ry2, nx = (size_t)*rx1 * *m * *rx2;
    ny = (size_t)*ry1 * *n * *ry2;
    ttg_ctx* c = shim_ctx();
    double* d = shim_buf(n1 + na + n2 + nx + ny);
    double *dp1 = d, *dA = dp1 + n1, *dp2 = dA + na, *dx = dp2 + n2, *dy = dx + nx;
    cudaStream_t s = c->stream;
    up(dp1, phi1, n1, s);
    up(dA, A, na, s);
    up(dp2, phi2, n2, s);
    up(dx, x, nx, s);   // x is read before y is written, so x == y is fine
    check(c, ttg_dbfun3(c, *rx1, *m, *rx2, *ry1, *n, *ry2, *ra1, *ra2, dp1, dA, dp2, dx, dy, 1));
    down(y, dy, ny, s);
    TTG_CUDA(cudaStreamSynchronize(s));
  } catch (const ttg::Error& e) {
    fail("dbfun3", e, y, ny);
  }
}

void djac_gen(char* ptype, long* rx1, long* n, long* rx2, long* ra1, long* ra2, double* Phi1,
              double* A, double* Phi2, double* jacs) {
  size_t nj = 0;
  try {
    TTG_REQUIRE(ptype && rx1 && n && rx2 && ra1 && ra2, "null argument");
    const ttg_int js = ttg_djac_size(*ptype, *rx1, *n, *rx2);
    TTG_REQUIRE(js >= 0, "unknown preconditioner type");
    nj = (size_t)js;
    if (nj == 0) return;   // 'n': no blocks, as the reference generates none
    const size_t n1 = (size_t)*rx1 * *rx1 * *ra1, na = (size_t)*ra1 * *n * *n * *ra2,
                 n2 = (size_t)*rx2 * *ra2 * *rx2;
    ttg_ctx* c = shim_ctx();
    double* d = shim_buf(n1 + na + n2 + nj);
    double *dp1 = d, *dA = dp1 + n1, *dp2 = dA + na, *dj = dp2 + n2;
    cudaStream_t s = c->stream;
    up(dp1, Phi1, n1, s);
    up(dA, A, na, s);
    up(dp2, Phi2, n2, s);
    check(c, ttg_djac_gen(c, *ptype, *rx1, *n, *rx2, *ra1, *ra2, dp1, dA, dp2, dj));
    down(jacs, dj, nj, s);
    TTG_CUDA(cudaStreamSynchronize(s));
  } catch (const ttg::Error& e) {
    fail("djac_gen", e, jacs, nj);
  }
}

void djac_apply(char* ptype, long* rx1, long* n, long* rx2, double* jacs, double* x, double* y,
                double* work1) {
  (void)work1;
  size_t nx = 0;
  try {
    TTG_REQUIRE(ptype && rx1 && n && rx2, "null argument");
    const ttg_int js = ttg_djac_size(*ptype, *rx1, *n, *rx2);
    TTG_REQUIRE(js >= 0, "unknown preconditioner type");
    nx = (size_t)*rx1 * *n * *rx2;
    if (js == 0) {
      // the reference's djac_apply leaves y untouched for any other type
      return;
    }
    ttg_ctx* c = shim_ctx();
    double* d = shim_buf((size_t)js + 2 * nx);
    double *dj = d, *dx = dj + js, *dy = dx + nx;
    cudaStream_t s = c->stream;
    up(dj, jacs, (size_t)js, s);
    up(dx, x, nx, s);
    check(c, ttg_djac_apply(c, *ptype, *rx1, *n, *rx2, dj, dx, dy));
    down(y, dy, nx, s);
    TTG_CUDA(cudaStreamSynchronize(s));
  } catch (const ttg::Error& e) {
    fail("djac_apply", e, y, nx);
  }
}

void dqr(long* n, long* m, double* A, double* R, double* work, long* lwork, double* tau) {
  (void)work;
  (void)lwork;
  (void)tau;
  size_t nr = 0;
  try {
    TTG_REQUIRE(n && m && A && R, "null argument");
    const size_t na = (size_t)*n * *m, k = (size_t)std::min(*n, *m);
    nr = k * (size_t)*m;
    ttg_ctx* c = shim_ctx();
    double* d = shim_buf(na + nr);
    cudaStream_t s = c->stream;
    up(d, A, na, s);
    check(c, ttg_dqr(c, *n, *m, d, d + na));
    // Q (n x min(n, m)) overwrites the leading columns of A, as dorgqr does
    down(A, d, (size_t)*n * k, s);
    down(R, d + na, nr, s);
    TTG_CUDA(cudaStreamSynchronize(s));
  } catch (const ttg::Error& e) {
    fail("dqr", e, R, nr);
  }
}

}  // extern "C"
