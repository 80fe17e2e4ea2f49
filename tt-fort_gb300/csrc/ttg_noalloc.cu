// ttg_dbfun3_noalloc: the local operator y = Phi1 * A * Phi2 * x with its
// intermediates in a fixed, library-owned device array instead of memory the
// library allocates.
//
// Who needs it: callers that must not allocate device memory during a call.
// A Fortran or C host that hands its whole device memory budget to another
// allocator (a framework's caching allocator that has already reserved the
// GPU) sees cudaMalloc fail or fragment that pool; a host inside a solver
// callback (PRIMME's matvec, Expokit's matvec) cannot tolerate the implicit
// device synchronisation of cudaMalloc/cudaFree on every product.  ttg_dbfun3
// sizes its scratch with cudaMalloc on first use and whenever a larger
// problem arrives; this entry point never does.
//
// The scratch is one file-scope __device__ array of TTG_NOALLOC_SCRATCH_DOUBLES
// doubles (16 MiB).  Every GPU that loads the library holds it until the
// process exits.  Host code cannot use the array's name as a device address
// (in host code it names a host-side stand-in), so the device address is
// looked up once per device with cudaGetSymbolAddress while that device is
// current; the first call on each device does this set-up (so make that first
// call before any stream capture).  The address is cached per CUDA context: a
// cudaDeviceReset or a new primary context on the device makes the next call
// look it up again.  All calls on a
// device share the array and it keeps the previous call's contents: calls
// that overlap on the GPU (different streams or contexts on the same device)
// race on it and must be serialised by the caller.  Nothing in the array has
// to start at zero: each GEMM stage overwrites its part before reading it.
#include "ttg_common.cuh"
#include <cuda.h>
#include <mutex>

namespace {

static __device__ __align__(256) double g_bfun3_scratch[TTG_NOALLOC_SCRATCH_DOUBLES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {nullptr};
CUcontext g_scratch_ctx[kMaxDevices] = {nullptr};

// device address of g_bfun3_scratch on the current device (set-up on first
// use, and again whenever the device's current CUDA context has changed)
double* scratch_on(int device) {
  std::lock_guard<std::mutex> lk(g_mu);
  // cudaSetDevice (the caller's first step) made the device's primary context
  // current, so the driver reports it here
  CUcontext cur = nullptr;
  cudaError_t ce = cudaSuccess;
  {
    // the driver call is resolved through the runtime's entry-point table, so
    // the library needs no link against libcuda
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    ce = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q);
    if (ce == cudaSuccess && q == cudaDriverEntryPointSuccess && fn)
      ((CUresult(*)(CUcontext*))fn)(&cur);
  }
  if (!g_scratch_addr[device] || g_scratch_ctx[device] != cur) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_bfun3_scratch);
    if (e != cudaSuccess || !p)
      throw ttg::Error{TTG_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") +
                                         cudaGetErrorString(e)};
    g_scratch_addr[device] = (double*)p;
    g_scratch_ctx[device] = cur;
  }
  return g_scratch_addr[device];
}

}  // namespace

extern "C" int ttg_dbfun3_noalloc(ttg_ctx* c, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1,
                                  ttg_int n, ttg_int ry2, ttg_int ra1, ttg_int ra2,
                                  const double* phi1, const double* A, const double* phi2,
                                  const double* x, double* y, ttg_int nvec) {
  if (!c) return TTG_ERR_ARG;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    TTG_REQUIRE(rx1 > 0 && m > 0 && rx2 > 0 && ry1 > 0 && n > 0 && ry2 > 0 && ra1 > 0 && ra2 > 0,
                "all sizes must be positive");
    TTG_REQUIRE(phi1 && A && phi2 && x && y && nvec > 0, "null pointer or nvec <= 0");
    long long xs = 0, ys = 0;
    TTG_REQUIRE(!__builtin_mul_overflow(rx1, m, &xs) && !__builtin_mul_overflow(xs, rx2, &xs) &&
                    !__builtin_mul_overflow(ry1, n, &ys) && !__builtin_mul_overflow(ys, ry2, &ys) &&
                    xs < (1ll << 31) && ys < (1ll << 31),
                "local problem too large for 32-bit tile indexing");
    TTG_REQUIRE(c->device >= 0 && c->device < kMaxDevices, "device index out of range");
    ttg::LocalDims L{rx1, m, rx2, ry1, n, ry2, ra1, ra2};
    // (rx1*m*ra2*ry2 + rx1*ra1*n*ry2) * nvec with every product checked: a
    // size that overflows 64 bits is rejected like one above the maximum
    long long t1 = 0, t2 = 0, need = 0;
    bool ovf = __builtin_mul_overflow(rx1, m, &t1) || __builtin_mul_overflow(t1, ra2, &t1) ||
               __builtin_mul_overflow(t1, ry2, &t1) || __builtin_mul_overflow(rx1, ra1, &t2) ||
               __builtin_mul_overflow(t2, n, &t2) || __builtin_mul_overflow(t2, ry2, &t2) ||
               __builtin_add_overflow(t1, t2, &need) || __builtin_mul_overflow(need, nvec, &need);
    if (ovf || need > (long long)TTG_NOALLOC_SCRATCH_DOUBLES) {
      if (ovf) need = -1;
      c->last_error = "ttg_dbfun3_noalloc: needs " +
                      (need < 0 ? std::string("more than 2^63") : std::to_string(need)) +
                      " doubles of scratch, the fixed maximum is " +
                      std::to_string((long long)TTG_NOALLOC_SCRATCH_DOUBLES) +
                      " ((rx1*m*ra2*ry2 + rx1*ra1*n*ry2) * nvec); use ttg_dbfun3";
      return TTG_ERR_ARG;
    }
    double* scr = scratch_on(c->device);
    ttg::bfun3_f64(L, phi1, A, phi2, x, y, (int)nvec, scr, c->stream);
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  } catch (const std::exception& e) {
    c->last_error = e.what();
    return TTG_ERR_ARG;
  }
  return TTG_OK;
}
