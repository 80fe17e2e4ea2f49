// Krylov exponential (Expokit ZGEXPV/ZGPADM) and the block 1-norm estimate
// (znormest_higham/ZLACN1) on the device, for the KSL time stepper.
#pragma once
#include "ttg_common.cuh"
#include <functional>

namespace ttg {

// complex (interleaved double2) block matvec: Y (n x t) = op(X (n x t))
using ZMatvecFn = std::function<void(const double2* X, double2* Y, int t)>;

struct ExpStats {
  long long nmult = 0, nstep = 0, nreject = 0, syncs = 0;
  int mxstep = 500;          // ZGEXPV's step cap (expokit.f:2506)
  bool strict = false;       // a capped exponential throws TTG_ERR_NOCONV
  long long capped = 0;      // exponentials that stopped at the cap short of t
};

// Workspace for both: n is the largest problem size, m the Krylov order.
struct ExpWork {
  i64 nmax = 0;
  int m = 8;
  double2* V = nullptr;     // nmax x (m + 1)
  double2* tmp = nullptr;   // nmax
  double2* X = nullptr;     // nmax x 4   (norm estimate blocks)
  double2* Y = nullptr;     // nmax x 4
  double2* H = nullptr;     // (m+2)^2
  double2* E = nullptr;     // (m+2) first column of exp(tH)
  double* red = nullptr;    // small reduction outputs
  int* ired = nullptr;      // small integer outputs
  double2* part = nullptr;  // per-CTA partial sums of the cooperative Gram-Schmidt
  double* hbuf = nullptr;   // pinned host mirror (4096 doubles)
  static size_t bytes(i64 nmax, int m);
  void bind(void* mem, i64 nmax_, int m_, double* pinned);
};

// ||A||_1 estimate (t columns, ITMAX 5), transp == nullptr reproduces the
// S-step estimator whose adjoint product is replaced by the identity.
double znormest_dev(ExpWork& w, i64 n, int t0, const ZMatvecFn& mv, const ZMatvecFn* transp,
                    unsigned long long& counter, cudaStream_t s, ExpStats* st);

// w = exp(tau A) v  (zexp_mv, explib.f90:53-125); v and w are device vectors
void zexp_mv_dev(ExpWork& w, i64 n, int m, double tau, const double2* v, double2* out,
                 double tol, double anorm, const ZMatvecFn& mv, cudaStream_t s, ExpStats* st);

}  // namespace ttg
