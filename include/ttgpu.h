/*
 * ttgpu.h -- C-ABI of the GB300 tensor-train sweep library (libttgpu.so).
 *
 * Drop-in boundary for the hot path of oseledets/tt-fort: the ALS/AMEn/KSL
 * sweep.  A Fortran host binds these symbols through ISO_C_BINDING (a
 * bind(c) interface module that mirrors these declarations); C and Python
 * (ctypes) callers use them directly.
 *
 * Conventions
 *   - integers are 64-bit (ttg_int), fixed for every build (the reference's
 *     i4/i8 presets, Makefile.in:7-106, become one documented width);
 *   - all arrays are flat column-major, exactly the reference layouts;
 *   - complex arrays are interleaved (re, im) double pairs, i.e. Fortran
 *     complex(8) / C99 double _Complex;
 *   - every call returns an int status (TTG_OK = 0, negative = error) and
 *     never stops the process (the reference prints and `stop`s,
 *     ttamen.f90:140,144; expokit.f:483);
 *   - kernel-level entry points take DEVICE pointers and run on the context's
 *     stream; driver entry points take HOST pointers;
 *   - one context per host thread: the context replaces the reference's
 *     module globals (tt_eigb.f90:1-50, tt_ksl.f90:1-166) and module result
 *     arrays (result_core tt_eigb.f90:57, zresult_core tt_ksl.f90:171).
 */
#ifndef TTGPU_H
#define TTGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int64_t ttg_int;
typedef struct ttg_ctx ttg_ctx;

enum {
  TTG_OK = 0,
  TTG_ERR_ARG = -1,         /* inconsistent sizes / ranks / null pointers   */
  TTG_ERR_CUDA = -2,        /* a CUDA runtime call failed                  */
  TTG_ERR_NOMEM = -3,       /* device allocation failed                    */
  TTG_ERR_NOCONV = -4,      /* an iteration cap was reached                */
  TTG_ERR_NAN = -5,         /* non-finite value detected                   */
  TTG_ERR_UNSUPPORTED = -7  /* shape outside what a kernel supports        */
};

enum {
  TTG_METHOD_PLAIN = 0,     /* FP64 contractions, the reference's arithmetic */
  TTG_METHOD_SPLIT = 1,     /* BF16x3 tensor-core contractions, FP32 accumulate,
                               FP64 Rayleigh-Ritz / QR / SVD / Pade          */
  TTG_METHOD_JD64 = 2       /* ttg_eigb only: the SPLIT method's local solver
                               (Jacobi-Davidson with CG corrections) on FP64
                               contractions; separates what the algorithm
                               gains from what split precision gains        */
};

/* ---------------------------------------------------------------- context */
int ttg_create(int device, ttg_ctx** ctx);
int ttg_destroy(ttg_ctx* ctx);
const char* ttg_last_error(const ttg_ctx* ctx);
/* run on a caller-owned cudaStream_t from now on (NULL = the legacy default
 * stream); the context's own stream is released */
int ttg_set_stream(ttg_ctx* ctx, void* cuda_stream);
int ttg_synchronize(ttg_ctx* ctx);
int ttg_version(void);

/* ------------------------------------------------ local operator (device) */
/* y = Phi1 * A * Phi2 * x for nvec vectors stored back to back.
 * Replaces dbfun3 ttals.f90:9-32 (also d2d_mv ttlocsolve.f90:49-88, the
 * bind(c) dbfun3 tt_linalg.f90:127-159) and the per-vector loop of
 * primme_matvec tt_eigb.f90:15-27. */
int ttg_dbfun3(ttg_ctx* ctx, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
               ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1, const double* A,
               const double* phi2, const double* x, double* y, ttg_int nvec);
/* Same product on the tensor cores: BF16x3 split operands, FP32 accumulation
 * (tcgen05.mma, accumulators in TMEM).  The chosen form's local matvec. */
int ttg_dbfun3_split(ttg_ctx* ctx, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1,
                     ttg_int n, ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1,
                     const double* A, const double* phi2, const double* x, double* y,
                     ttg_int nvec);
/* Allocation-free variant of ttg_dbfun3 (no counterpart in the reference).
 * For callers that must not allocate device memory during a call: hosts whose
 * device memory belongs to another allocator, and callers inside a solver
 * callback that cannot absorb the device synchronisation of cudaMalloc/cudaFree.
 * The intermediates live in one library-owned device array of
 * TTG_NOALLOC_SCRATCH_DOUBLES doubles (16 MiB, held by every GPU that loads the
 * library until exit).  The first call on a device looks up that array's
 * device address (set-up, once per device and CUDA context, so make that first
 * call before any stream capture).  Sizes with
 * (rx1*m*ra2*ry2 + rx1*ra1*n*ry2) * nvec > TTG_NOALLOC_SCRATCH_DOUBLES are
 * rejected with TTG_ERR_ARG, and so are sizes whose products overflow 64 bits.
 * All calls share the array: calls that overlap on
 * the GPU race and must be serialised by the caller.  Calls no cudaMalloc,
 * cudaFree or other allocating routine. */
#define TTG_NOALLOC_SCRATCH_DOUBLES 2097152
int ttg_dbfun3_noalloc(ttg_ctx* ctx, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1,
                       ttg_int n, ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1,
                       const double* A, const double* phi2, const double* x, double* y,
                       ttg_int nvec);
/* Local eigensolve of tt_eigb (the dprimme call of tt_eigb.f90:252-283):
 * lowest B eigenpairs of y = Phi1 A Phi2 x on the square local problem
 * (r1, n, r2), operator ranks ra1, ra2, device operands.  X (device,
 * N x B, N = r1 n r2) holds the start block (initSize = B) on entry and the
 * Ritz vectors on return; lambda (host, B) the eigenvalues; res (host,
 * optional) the 2-norm of the B residual norms; matvecs (optional) the
 * matvec count.  tol is PRIMME's eps (residual relative to the operator's
 * largest Ritz value magnitude), max_matvecs its maxMatvecs (<= 0: 500).
 * method PLAIN: block GD+k Davidson with FP64 matvecs; SPLIT: Jacobi-Davidson
 * with BF16x3 tensor-core corrections judged by FP64 residuals; JD64: the
 * SPLIT solver on FP64 matvecs.  A capped solve is counted (ttg_capped) or,
 * with strict limits, returns TTG_ERR_NOCONV. */
int ttg_local_eig(ttg_ctx* ctx, ttg_int r1, ttg_int n, ttg_int r2, ttg_int ra1, ttg_int ra2,
                  const double* phi1, const double* A, const double* phi2, double* X, ttg_int B,
                  double tol, ttg_int max_matvecs, int method, double* lambda, double* res,
                  ttg_int* matvecs);
/* Prepared local operator: the GPU counterpart of init_bfun_sizes +
 * init_bfun_main + primme_matvec (tt_eigb.f90:15-49, tt_ksl.f90:1-84).
 * create() binds Phi1, A, Phi2 (device pointers, kept by reference) for up to
 * nvec_max vectors per apply and, for TTG_METHOD_SPLIT, splits Phi1/Phi2 into
 * BF16 hi/lo tiles once; apply() is asynchronous on the context's stream. */
typedef struct ttg_localop ttg_localop;
int ttg_localop_create(ttg_ctx* ctx, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
                       ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1, const double* A,
                       const double* phi2, ttg_int nvec_max, int method, ttg_localop** op);
int ttg_localop_apply(ttg_localop* op, const double* x, double* y, ttg_int nvec);
int ttg_localop_destroy(ttg_localop* op);
/* Complex product, zbfun3 ttals.f90:34-57. */
int ttg_zbfun3(ttg_ctx* ctx, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
               ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1, const double* A,
               const double* phi2, const double* x, double* y, ttg_int nvec);
/* Adjoint product for the 1-norm estimate, zbfun3_transp ttals.f90:85-108. */
int ttg_zbfun3_transp(ttg_ctx* ctx, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1,
                      ttg_int n, ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1,
                      const double* A, const double* phi2, const double* x, double* y,
                      ttg_int nvec);

/* ------------------------------------------------- interface updates (device) */
/* phi1_new (ry2, rx2, ra2): dphi_left ttals.f90:203-227 */
int ttg_dphi_left(ttg_ctx* ctx, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
                  ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1_old,
                  const double* A, const double* x, const double* y, double* phi1_new);
/* phi2_new (rx1, ra1, ry1): dphi_right ttals.f90:150-173 */
int ttg_dphi_right(ttg_ctx* ctx, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
                   ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi2_old,
                   const double* A, const double* x, const double* y, double* phi2_new);
/* complex, y conjugated: zphi_left ttals.f90:229-256, zphi_right :176-200 */
int ttg_zphi_left(ttg_ctx* ctx, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
                  ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi1_old,
                  const double* A, const double* x, const double* y, double* phi1_new);
int ttg_zphi_right(ttg_ctx* ctx, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1, ttg_int n,
                   ttg_int ry2, ttg_int ra1, ttg_int ra2, const double* phi2_old,
                   const double* A, const double* x, const double* y, double* phi2_new);
/* Y'X projections: dphi2_left ttals.f90:296-314, dphi2_right :260-277 */
int ttg_dphi2_left(ttg_ctx* ctx, ttg_int rx1, ttg_int rx2, ttg_int ry1, ttg_int n,
                   ttg_int ry2, const double* phi1_old, const double* x, const double* y,
                   double* phi1_new);
int ttg_dphi2_right(ttg_ctx* ctx, ttg_int rx1, ttg_int rx2, ttg_int ry1, ttg_int n,
                    ttg_int ry2, const double* phi2_old, const double* x, const double* y,
                    double* phi2_new);
/* dense local matrix, d2d_fullmat tt_eigb.f90:88-105 / ttlocsolve.f90:133-150 */
int ttg_d2d_fullmat(ttg_ctx* ctx, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ra1,
                    ttg_int ra2, const double* phi1, const double* A, const double* phi2,
                    double* B);

/* Block-Jacobi preconditioner of the local system, djac_gen
 * tt_linalg.f90:363-494 (bind(c)): ptype 'c' (diagonals of Phi1 and Phi2, an
 * n x n block per (b1,b2)), 'l' (Phi1 and the diagonal of Phi2, an
 * (rx1 n)^2 block per b2) or 'r' (the diagonal of Phi1 and Phi2, an
 * (n rx2)^2 block per b1); each block inverted by LU with partial pivoting.
 * Device pointers; jacs receives ttg_djac_size(ptype, rx1, n, rx2) doubles in
 * the reference's layout.  Blocks larger than 4096 are rejected. */
ttg_int ttg_djac_size(char ptype, ttg_int rx1, ttg_int n, ttg_int rx2);
int ttg_djac_gen(ttg_ctx* ctx, char ptype, ttg_int rx1, ttg_int n, ttg_int rx2, ttg_int ra1,
                 ttg_int ra2, const double* phi1, const double* A, const double* phi2,
                 double* jacs);
/* y = P x with the blocks of ttg_djac_gen, djac_apply tt_linalg.f90:497-531;
 * x and y (rx1, n, rx2) may be the same array. */
int ttg_djac_apply(ttg_ctx* ctx, char ptype, ttg_int rx1, ttg_int n, ttg_int rx2,
                   const double* jacs, const double* x, double* y);

/* ------------------------------- reference-named by-reference entry points
 * The bind(c) kernels of tt_linalg.f90 under their own names and argument
 * lists, for C and Fortran callers that bind them directly (gmres_3d.c:3-4
 * declares dbfun3 and djac_apply this way and links against them unchanged).
 * All sizes are 64-bit (`long`, the i8 presets) and all arrays are HOST
 * arrays: each call copies its inputs to the device, runs the ttg_* kernel on
 * a per-thread context (device $TTG_DEVICE, default 0) and copies the result
 * back.  The workspace arguments of the Fortran interfaces are accepted and
 * not used.  These routines return nothing, like the reference's; a failed
 * call prints one line to stderr, fills its output with NaN and sets the
 * status that ttg_fshim_status() returns (and clears). */
/* y = Phi1 A Phi2 x, dbfun3 tt_linalg.f90:127-159; x and y may be one array */
void dbfun3(long* rx1, long* m, long* rx2, long* ry1, long* n, long* ry2, long* ra1, long* ra2,
            double* phi1, double* A, double* phi2, double* x, double* y, double* res1,
            double* res2);
/* block-Jacobi blocks, djac_gen tt_linalg.f90:363-494 */
void djac_gen(char* ptype, long* rx1, long* n, long* rx2, long* ra1, long* ra2, double* Phi1,
              double* A, double* Phi2, double* jacs);
/* y = P x, djac_apply tt_linalg.f90:497-531; x and y may be one array */
void djac_apply(char* ptype, long* rx1, long* n, long* rx2, double* jacs, double* x, double* y,
                double* work1);
/* Householder QR, dqr tt_linalg.f90:30-52: Q overwrites A (n x min(n, m)),
 * R is min(n, m) x m */
void dqr(long* n, long* m, double* A, double* R, double* work, long* lwork, double* tau);
/* status of the last failed by-reference call on this thread (TTG_OK if
 * none), cleared by the call */
int ttg_fshim_status(void);

/* ------------------------------------------------ TT files (host) */
/* The reference's binary TT format (.sdv): dtt_write / ztt_write and
 * dtt_read / ztt_read, ttio.f90:29-399.  Host arrays; cores back to back,
 * core k of r[k] x n[k] x r[k+1] column-major, float64, or complex128 stored
 * as interleaved pairs when is_complex (the file does not record which).
 * Modes are written as l = 1 .. m = d; d <= 1023 (tt_size).  The reader
 * checks the 'TT' magic and version 1, sets d and nelem (scalars of the
 * cores), and fills n (d), r (d + 1) and cores when they are not NULL
 * (nmax = capacity of n; cores must hold nelem scalars).  Both return
 * TTG_ERR_ARG on I/O or format errors; they need no context or GPU. */
int ttg_sdv_write(const char* path, ttg_int d, const ttg_int* n, const ttg_int* r,
                  const double* cores, int is_complex);
int ttg_sdv_read(const char* path, int is_complex, ttg_int* d, ttg_int* n, ttg_int* r,
                 ttg_int nmax, double* cores, ttg_int* nelem);

/* ------------------------------------------------ dense algebra (device) */
/* A (n x m) -> Q (n x min(n,m)) in place, R (min(n,m) x m): dqr
 * matrix_util.f90:37-61 (bind(c) twin tt_linalg.f90:30); zqr :64-90. */
int ttg_dqr(ttg_ctx* ctx, ttg_int n, ttg_int m, double* A, double* R);
int ttg_zqr(ttg_ctx* ctx, ttg_int n, ttg_int m, double* A, double* R);
/* symmetric eigen, ascending; eigenvectors overwrite A (dsyev 'V','U',
 * tt_eigb.f90:238).  k <= 512. */
int ttg_dsyev(ttg_ctx* ctx, ttg_int k, double* A, double* w);
/* thin SVD M (p x q) = U diag(s) Vt, descending s (dgesvd tt_eigb.f90:312,361). */
int ttg_dgesvd(ttg_ctx* ctx, ttg_int p, ttg_int q, const double* M, double* U, double* s,
               double* Vt);
/* rank kept by my_chop3 (matrix_util.f90:254-275) for n singular values
 * (host array). */
ttg_int ttg_my_chop3(ttg_int n, const double* s, double eps);
/* maxvol row selection of a tall n x r matrix (maxvol0_d maxvol.f90:27-119
 * and maxvol_d :197-288): writes r row indices (0-based) to p (device) and
 * the coefficient matrix Z = A * A(p,:)^{-1} (n x r) when Z != NULL. */
int ttg_dmaxvol(ttg_ctx* ctx, ttg_int n, ttg_int r, const double* A, ttg_int* p, double* Z,
                double tol, ttg_int maxiters);

/* ------------------------------------------- learned preconditioner (new) */
/* No counterpart in the reference: PRIMME's applyPreconditioner hook is left
 * unset by tt_eigb (primme/primme.h:144-145, tt_eigb.f90:252-283).  A ReLU MLP
 * (3 features -> depth x width -> 1; layer products in BF16 on the tensor
 * cores with FP32 accumulation, or FP32, see ttg_mlp_set_precision; FP32
 * parameters, activations and Adam state) corrects the classical diagonal
 * Davidson preconditioner of the plain method's local solves; it is trained
 * on local problems that the sweeps record.  Parameters are one flat float
 * array, layer by layer: W_l (in x out, row-major) then b_l. */
typedef struct ttg_mlp ttg_mlp;
int ttg_mlp_create(ttg_ctx* ctx, ttg_int width, ttg_int depth, ttg_int seed, ttg_mlp** out);
int ttg_mlp_destroy(ttg_mlp* mlp);
ttg_int ttg_mlp_nparams(const ttg_mlp* mlp);
int ttg_mlp_get_params(ttg_mlp* mlp, float* host, ttg_int n);
int ttg_mlp_set_params(ttg_mlp* mlp, const float* host, ttg_int n);
int ttg_mlp_get_grads(ttg_mlp* mlp, float* host, ttg_int n);
/* h (P, device) = network(F (P x 3 row-major, device)) */
int ttg_mlp_forward(ttg_mlp* mlp, ttg_int P, const float* F, float* h);
/* loss and parameter gradient (kept in the network) of one recorded local
 * problem, all device arrays: D (N) operator diagonal, theta (B), X (N x B)
 * start Ritz block, R (N x B) its residuals, V (N x B) ideal corrections */
int ttg_mlp_loss_grad(ttg_mlp* mlp, ttg_int N, ttg_int B, const double* D, const double* theta,
                      const double* X, const double* R, const double* V, double* loss);
int ttg_mlp_adam_step(ttg_mlp* mlp, double lr);
/* layer products of the forward and backward passes: bf16 = 1 (the default)
 * runs them in BF16 on the tensor cores (tcgen05, FP32 accumulate), 0 in
 * FP32 on the CUDA cores */
int ttg_mlp_set_precision(ttg_mlp* mlp, int bf16);
/* TTG_ERR_CUDA when a tensor-core product of the network gave up waiting on
 * its bounded mbarrier waits (synchronises the network's stream) */
int ttg_mlp_check(ttg_mlp* mlp);
/* mode bit 0: precondition the plain method's Davidson expansions with mlp;
 * bit 1: record every iterative local problem of the plain method */
int ttg_set_learned(ttg_ctx* ctx, ttg_mlp* mlp, int mode);
int ttg_record_count(const ttg_ctx* ctx, ttg_int* nprob, ttg_int* npoints);
int ttg_record_clear(ttg_ctx* ctx);
/* Adam over the problems recorded in rec; mean loss before and after (the
 * parameters before training are kept when the loss did not decrease) */
int ttg_mlp_train_recorded(ttg_mlp* mlp, const ttg_ctx* rec, ttg_int steps, double lr,
                           ttg_int seed, double* loss_first, double* loss_last);

/* ---------------------------------------------------------- drivers (host) */
/* Block eigensolver, tt_eigb tt_eigb.f90:110-436.  ry (d+1) is updated in
 * place, ry[d] = B on input and output; lambda receives B eigenvalues; the
 * cores are kept in the context (ttg_result_*).  method = TTG_METHOD_*. */
int ttg_eigb(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* m, const ttg_int* ra,
             const double* crA, const double* crY0, ttg_int* ry, double eps, ttg_int rmax,
             double* lambda, ttg_int B, ttg_int nswp, ttg_int max_full_size, int verb,
             int method);
/* KSL time stepping, ztt_ksl tt_ksl.f90:431-668 (complex, interleaved):
 * nsteps consecutive calls of the reference's one-step routine (nsteps <= 0
 * means 1) with the state kept on the device; ry updated in place (ranks can
 * only shrink); the result cores are read with ttg_zresult_copy.  typ 1 =
 * KSL, 2 = symmetric KSL; order = Krylov dimension (8 in the reference);
 * rmax is accepted and unused, as in the reference. */
int ttg_ksl_z(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* m, const ttg_int* ra,
              const double* crA, const double* crY0, ttg_int* ry, double tau, ttg_int rmax,
              int verb, int typ, int order, int method, ttg_int nsteps);
/* KSL time stepping with real data, tt_ksl tt_ksl.f90:191-428: the real
 * routine's own sweep (backward half sweep with the S-step on the bond to
 * the right of each core, forward half sweep with the S-step before each
 * K-step), always symmetric (typ is read and unused, as in the reference).
 * The S operator multiplies with 1 and 0 where the reference's dsfun_matvec
 * uses its undeclared ONE and ZERO (tt_ksl.f90:122-130).  Every rank must
 * pass both QR sweeps unchanged.  With d = 1 one call is a forward half step,
 * as in the reference.  Arguments as ttg_ksl_z, real arrays; results through
 * ttg_result_copy. */
int ttg_ksl_d(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* m, const ttg_int* ra,
              const double* crA, const double* crY0, ttg_int* ry, double tau, ttg_int rmax,
              int verb, int typ, int order, int method, ttg_int nsteps);
/* KSL for an operator diagonal in the physical index, ztt_diag_ksl
 * tt_diag_ksl.f90:560-804 (complex, interleaved) and dtt_diag_ksl :315-558
 * (real): crA holds the cores A(a1, i, a2) (ra[k] x n[k] x ra[k+1]); each
 * K-step runs one Krylov exponential per slice i of the core, every
 * exponential with anorm = 1, as the reference does.  Other arguments and
 * results as ttg_ksl_z (real results through ttg_result_copy, complex through
 * ttg_zresult_copy); FP64 only.  The real entry runs the same scheme in
 * complex arithmetic on real data. */
int ttg_diag_ksl_z(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* ra,
                   const double* crA, const double* crY0, ttg_int* ry, double tau, ttg_int rmax,
                   int verb, int typ, int order, ttg_int nsteps);
int ttg_diag_ksl_d(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* ra,
                   const double* crA, const double* crY0, ttg_int* ry, double tau, ttg_int rmax,
                   int verb, int typ, int order, ttg_int nsteps);
/* AMEn matvec y ~ A x, tt_mvk4 tt_adapt_als.f90:67-500 (argument order
 * follows it; crY0 with ranks ry is the start, ry updated in place).
 * kickrank 5 and nswp 20 are the reference's defaults (nswp <= 0: 20); the
 * sweep stops when a sweep's largest relative core change is below eps.  The
 * reference's rmax only sizes its work arrays; here it caps the kept ranks.
 * The result cores are read with ttg_result_copy. */
int ttg_mvk4(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* m, const ttg_int* rx,
             const ttg_int* ra, const double* crA, const double* crX, const double* crY0,
             ttg_int* ry, double eps, ttg_int rmax, ttg_int kickrank, ttg_int nswp, int verb);
/* AMEn linear solve A x = y, tt_amen_solve tt_adapt_als.f90:513-1132
 * (argument order follows it; rx updated in place).  kickrank 4, nswp 20,
 * prec 'n', nrestart 40, niters 2 are the reference's defaults (pass them,
 * or values <= 0 / 0 for the defaults of nswp, nrestart, niters); prec 'c',
 * 'l', 'r' right-precondition each local GMRES with the block-Jacobi blocks
 * of ttg_djac_gen, regenerated per local system as the reference does.  rmax
 * caps the kept ranks (<= 0: no cap, as in the reference). */
int ttg_amen_solve(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* m,
                   const ttg_int* ry, const ttg_int* ra, const double* crA, const double* crY,
                   const double* crX0, ttg_int* rx, double eps, ttg_int kickrank, ttg_int nswp,
                   int verb, char prec, ttg_int nrestart, ttg_int niters, ttg_int rmax,
                   int method);
/* AMEn of ttamen.f90 (dtt_amen_solve, ttamen.f90:29-252) with the packed
 * cores of the arguments above in place of the dtt type; rmax caps the
 * ranks (<= 0: no cap).  method TTG_METHOD_SPLIT runs the local GMRES on the
 * BF16x3 tensor-core operator inside FP64 iterative refinement; the FP64
 * residual is the stopping test in both methods. */
int ttg_dtt_amen_solve(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* m,
                       const ttg_int* ry, const ttg_int* ra, const double* crA,
                       const double* crY, const double* crX0, ttg_int* rx, double eps,
                       ttg_int rmax, ttg_int kickrank, ttg_int nswp, int verb, int method);
/* Batched eigen sweeps (no counterpart in the reference, whose tt_eigb
 * solves one chain per call): chains are queued with their inputs copied,
 * then ttg_batch_run solves all of them on nworkers host threads, each with
 * its own non-blocking stream, so the chains' kernels overlap on the GPU
 * (longest chains first).  Arguments of ttg_batch_add_eigb mean what they
 * mean for ttg_eigb; ry[d] must equal B. */
typedef struct ttg_batch ttg_batch;
int ttg_batch_create(ttg_ctx* ctx, int nworkers, ttg_batch** out);
int ttg_batch_destroy(ttg_batch* batch);
int ttg_batch_add_eigb(ttg_batch* batch, ttg_int d, const ttg_int* n, const ttg_int* m,
                       const ttg_int* ra, const double* crA, const double* crY0,
                       const ttg_int* ry, double eps, ttg_int rmax, ttg_int B, ttg_int nswp,
                       ttg_int max_full_size, int method, ttg_int* index);
int ttg_batch_run(ttg_batch* batch);
/* per chain: B eigenvalues, d+1 ranks, number of core elements, local
 * matvecs, wall seconds on its worker, status (0, 1 = not run, < 0 error) */
int ttg_batch_result(const ttg_batch* batch, ttg_int i, double* lambda, ttg_int* ry,
                     ttg_int* ncore, ttg_int* matvecs, double* seconds, int* status);
int ttg_batch_cores(const ttg_batch* batch, ttg_int i, double* out, ttg_int nelem);
/* Results of the last driver call. */
int ttg_result_size(const ttg_ctx* ctx, ttg_int* nelem);
int ttg_result_copy(const ttg_ctx* ctx, double* out, ttg_int nelem);   /* real */
int ttg_zresult_copy(const ttg_ctx* ctx, double* out, ttg_int nelem);  /* complex */
int ttg_free_result(ttg_ctx* ctx);      /* deallocate_result tt_eigb.f90:60-64 */
/* counters of the last driver call: total local matvecs, sweeps, residual */
int ttg_stats(const ttg_ctx* ctx, ttg_int* matvecs, ttg_int* sweeps, double* res,
              ttg_int* launches);
/* Iteration caps of the local solvers, for the next driver calls on ctx.
 * max_matvecs: matvec budget of each local eigensolve (PRIMME's maxMatvecs,
 * 500, tt_eigb.f90:152,269); max_expokit_steps: integration steps of each
 * Krylov exponential (mxstep of ZGEXPV, 500, expokit.f:2506); 0 keeps the
 * reference's value.  The reference tolerates a reached cap (PRIMME returns
 * -3, Expokit sets iflag = 1, its GMRES stops after nrestart x niters, and the
 * sweep goes on, tt_eigb.f90:285-288, explib.f90:108-111): so does the library
 * with strict = 0, counting such local solves (ttg_capped).  With strict = 1
 * the first capped local solve ends the driver call with TTG_ERR_NOCONV. */
int ttg_set_limits(ttg_ctx* ctx, ttg_int max_matvecs, ttg_int max_expokit_steps, int strict);
/* local solves of the last driver call that stopped at an iteration cap
 * before reaching their tolerance (-1 for a null context) */
ttg_int ttg_capped(const ttg_ctx* ctx);
/* kernel launches issued by the library since it was loaded (all contexts) */
ttg_int ttg_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* TTGPU_H */
