/* Test infrastructure (oracle): the BLAS routines that tt-fort's gmres_3d.c
 * calls, with its 64-bit integer arguments (`long*`, gmres_3d.c:6-7 and the
 * i8 presets), forwarded to the LP64 routines of scipy's cython_blas table
 * whose pointers oracle/primme.py-style code sets with ttref64_set_fn.
 * Built with gmres_3d.c (unchanged, from the tt-fort source tree) by
 * oracle/build_ref.py to check that the reference's C caller links against
 * libttgpu.so's by-reference dbfun3 / djac_apply without edits. */
#include <string.h>

typedef void (*fn_daxpy)(int*, double*, double*, int*, double*, int*);
typedef void (*fn_dcopy)(int*, double*, int*, double*, int*);
typedef double (*fn_ddot)(int*, double*, int*, double*, int*);
typedef double (*fn_dnrm2)(int*, double*, int*);
typedef void (*fn_dscal)(int*, double*, double*, int*);
typedef void (*fn_dtrsv)(char*, char*, char*, int*, double*, int*, double*, int*);

static struct {
  fn_daxpy daxpy;
  fn_dcopy dcopy;
  fn_ddot ddot;
  fn_dnrm2 dnrm2;
  fn_dscal dscal;
  fn_dtrsv dtrsv;
} T64;

int ttref64_set_fn(const char* name, void* fn) {
#define SETF(nm)                  \
  if (strcmp(name, #nm) == 0) {   \
    T64.nm = (fn_##nm)fn;         \
    return 0;                     \
  }
  SETF(daxpy) SETF(dcopy) SETF(ddot) SETF(dnrm2) SETF(dscal) SETF(dtrsv)
#undef SETF
  return -1;
}

void daxpy_(long* n, double* a, double* x, long* ix, double* y, long* iy) {
  int n_ = (int)*n, i_ = (int)*ix, j_ = (int)*iy;
  T64.daxpy(&n_, a, x, &i_, y, &j_);
}
void dcopy_(long* n, double* x, long* ix, double* y, long* iy) {
  int n_ = (int)*n, i_ = (int)*ix, j_ = (int)*iy;
  T64.dcopy(&n_, x, &i_, y, &j_);
}
double ddot_(long* n, double* x, long* ix, double* y, long* iy) {
  int n_ = (int)*n, i_ = (int)*ix, j_ = (int)*iy;
  return T64.ddot(&n_, x, &i_, y, &j_);
}
double dnrm2_(long* n, double* x, long* ix) {
  int n_ = (int)*n, i_ = (int)*ix;
  return T64.dnrm2(&n_, x, &i_);
}
void dscal_(long* n, double* a, double* x, long* ix) {
  int n_ = (int)*n, i_ = (int)*ix;
  T64.dscal(&n_, a, x, &i_);
}
void dtrsv_(char* uplo, char* trans, char* diag, long* n, double* a, long* lda, double* x,
            long* ix) {
  int n_ = (int)*n, l_ = (int)*lda, i_ = (int)*ix;
  T64.dtrsv(uplo, trans, diag, &n_, a, &l_, x, &i_);
}
