/* Test infrastructure (oracle): a C driver that runs the reference's own
 * PRIMME eigensolver (the C sources vendored in tt-fort's primme/ directory,
 * compiled unchanged by oracle/build_ref.py into oracle/_ref/) the way
 * tt_eigb.f90:252-283 sets it up, so the oracle's local eigensolver and the
 * GPU's can be checked against the reference's inner solver itself.
 *
 * BLAS/LAPACK: PRIMME calls the Fortran-convention routines dcopy_, dgemm_,
 * ..., dsytrs_, dlamch_ with 32-bit integers (the reference's i4 presets,
 * Makefile.in:27-66).  This image has no system BLAS, so each of those names
 * is defined here as a forwarder to a function pointer that the Python side
 * (oracle/primme.py) takes from scipy's cython_blas / cython_lapack tables
 * (LP64, same argument lists, no hidden string lengths) before the first
 * solve.  Nothing here is product code, and nothing in the product links it.
 */
#include <stdio.h>
#include <string.h>
#include "primme.h"

/* ---------------------------------------------------------------- BLAS table */
typedef void (*fn_dcopy)(int*, double*, int*, double*, int*);
typedef void (*fn_dswap)(int*, double*, int*, double*, int*);
typedef void (*fn_dgemm)(char*, char*, int*, int*, int*, double*, double*, int*, double*, int*,
                         double*, double*, int*);
typedef void (*fn_dsymm)(char*, char*, int*, int*, double*, double*, int*, double*, int*, double*,
                         double*, int*);
typedef void (*fn_daxpy)(int*, double*, double*, int*, double*, int*);
typedef void (*fn_dgemv)(char*, int*, int*, double*, double*, int*, double*, int*, double*,
                         double*, int*);
typedef double (*fn_ddot)(int*, double*, int*, double*, int*);
typedef void (*fn_dscal)(int*, double*, double*, int*);
typedef void (*fn_dlarnv)(int*, int*, int*, double*);
typedef void (*fn_dsyev)(char*, char*, int*, double*, int*, double*, double*, int*, int*);
typedef void (*fn_dsytrf)(char*, int*, double*, int*, int*, double*, int*, int*);
typedef void (*fn_dsytrs)(char*, int*, int*, double*, int*, int*, double*, int*, int*);
typedef double (*fn_dlamch)(char*);

static struct {
  fn_dcopy dcopy;
  fn_dswap dswap;
  fn_dgemm dgemm;
  fn_dsymm dsymm;
  fn_daxpy daxpy;
  fn_dgemv dgemv;
  fn_ddot ddot;
  fn_dscal dscal;
  fn_dlarnv dlarnv;
  fn_dsyev dsyev;
  fn_dsytrf dsytrf;
  fn_dsytrs dsytrs;
  fn_dlamch dlamch;
} T;

/* set one entry of the table; returns 0 on success, -1 for an unknown name */
int ttref_set_fn(const char* name, void* fn) {
#define SETF(nm)                      \
  if (strcmp(name, #nm) == 0) {       \
    T.nm = (fn_##nm)fn;               \
    return 0;                         \
  }
  SETF(dcopy) SETF(dswap) SETF(dgemm) SETF(dsymm) SETF(daxpy) SETF(dgemv)
  SETF(ddot) SETF(dscal) SETF(dlarnv) SETF(dsyev) SETF(dsytrf) SETF(dsytrs) SETF(dlamch)
#undef SETF
  return -1;
}

/* 1 when every entry is set */
int ttref_blas_ready(void) {
  return T.dcopy && T.dswap && T.dgemm && T.dsymm && T.daxpy && T.dgemv && T.ddot && T.dscal &&
         T.dlarnv && T.dsyev && T.dsytrf && T.dsytrs && T.dlamch;
}

void dcopy_(int* n, double* x, int* ix, double* y, int* iy) { T.dcopy(n, x, ix, y, iy); }
void dswap_(int* n, double* x, int* ix, double* y, int* iy) { T.dswap(n, x, ix, y, iy); }
void dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* al, double* a, int* lda,
            double* b, int* ldb, double* be, double* c, int* ldc) {
  T.dgemm(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc);
}
void dsymm_(char* side, char* uplo, int* m, int* n, double* al, double* a, int* lda, double* b,
            int* ldb, double* be, double* c, int* ldc) {
  T.dsymm(side, uplo, m, n, al, a, lda, b, ldb, be, c, ldc);
}
void daxpy_(int* n, double* a, double* x, int* ix, double* y, int* iy) { T.daxpy(n, a, x, ix, y, iy); }
void dgemv_(char* t, int* m, int* n, double* al, double* a, int* lda, double* x, int* ix,
            double* be, double* y, int* iy) {
  T.dgemv(t, m, n, al, a, lda, x, ix, be, y, iy);
}
double ddot_(int* n, double* x, int* ix, double* y, int* iy) { return T.ddot(n, x, ix, y, iy); }
void dscal_(int* n, double* a, double* x, int* ix) { T.dscal(n, a, x, ix); }
void dlarnv_(int* idist, int* iseed, int* n, double* x) { T.dlarnv(idist, iseed, n, x); }
void dsyev_(char* jobz, char* uplo, int* n, double* a, int* lda, double* w, double* work,
            int* lwork, int* info) {
  T.dsyev(jobz, uplo, n, a, lda, w, work, lwork, info);
}
void dsytrf_(char* uplo, int* n, double* a, int* lda, int* ipiv, double* work, int* lwork,
             int* info) {
  T.dsytrf(uplo, n, a, lda, ipiv, work, lwork, info);
}
void dsytrs_(char* uplo, int* n, int* nrhs, double* a, int* lda, int* ipiv, double* b, int* ldb,
             int* info) {
  T.dsytrs(uplo, n, nrhs, a, lda, ipiv, b, ldb, info);
}

double dlamch_(char* cmach) { return T.dlamch(cmach); }

/* ------------------------------------------------------------- the solve */
/* the caller's block matvec y (n x k) = A x (n x k), both column-major */
typedef void (*ttref_matvec)(double* x, double* y, int k);
static ttref_matvec g_mv = NULL;

static void matvec_tramp(void* x, void* y, int* blockSize, primme_params* p) {
  (void)p;
  g_mv((double*)x, (double*)y, *blockSize);
}

/* Lowest numEvals eigenpairs of the operator behind mv, with the settings of
 * tt_eigb.f90:252-283: method (DYNAMIC = 0 in tt_eigb, GD_plusK = 5 for a
 * deterministic run), n, printLevel, maxMatvecs, minRestartSize =
 * min(B+1, n-1), maxBasisSize, eps, initSize = B, start block in evecs
 * (n x numEvals).  Returns PRIMME's ierr; evals, evecs, rnorms and the matvec
 * count are written back. */
int ttref_dprimme(int n, int numEvals, int method, int maxBasisSize, int maxMatvecs, double eps,
                  int printLevel, ttref_matvec mv, double* evals, double* evecs, double* rnorms,
                  int* numMatvecs) {
  if (!ttref_blas_ready()) return -100;
  primme_params p;
  primme_initialize(&p);
  p.numEvals = numEvals;
  int e = primme_set_method((primme_preset_method)method, &p);
  if (e < 0) return -101;
  p.n = n;
  g_mv = mv;
  p.matrixMatvec = matvec_tramp;
  p.printLevel = printLevel;
  p.maxMatvecs = maxMatvecs;
  p.minRestartSize = numEvals + 1 < n - 1 ? numEvals + 1 : n - 1;
  p.maxBasisSize = maxBasisSize;
  p.eps = eps;
  p.initSize = numEvals;
  int ierr = dprimme(evals, evecs, rnorms, &p);
  if (numMatvecs) *numMatvecs = p.stats.numMatvecs;
  primme_Free(&p);
  g_mv = NULL;
  return ierr;
}
