// Block generalized-Davidson (GD+k) local eigensolver on the device.
//
// Replaces the vendored PRIMME call of tt_eigb (tt_eigb.f90:252-290): the
// start block is the current TT core (initSize = B), the tolerance is
// eps/sqrt(d)/10 relative to max|theta|, the matvec budget is maxMatvecs =
// 500, and the restart keeps the current and the previous Ritz vectors
// (GD+k, primme/restart_d.c:120).  Expansion is blocked (all unconverged
// residuals per iteration) so that every matvec call is one batched launch
// sequence.  The basis is kept orthonormal by BCGS2 (block Gram-Schmidt +
// Cholesky QR, twice).  Every FP64 product runs on the device; the host only
// reads B residual norms per iteration to decide convergence.
#pragma once
#include "ttg_common.cuh"
#include <functional>

namespace ttg {

using MatvecFn = std::function<void(const double* X, double* Y, int nvec)>;

// Chosen-form local operator y = Phi1 A Phi2 x on the BF16x3 tensor-core
// kernels (ttg_tc.cu): operands prepared once in mem (mem_bytes long, sized
// with split_matvec_bytes for the largest local problem it serves),
// two prepared operators (slot 0 and 1) per host thread; preparing a slot
// again replaces its operator.  split_matvec_check reads the bounded-wait
// flags of slots [0, nslots), which the caller must have prepared itself,
// and throws when a GEMM gave up waiting.
void split_matvec_factory(const LocalDims& L, const double* phi1, const double* A,
                          const double* phi2, int nvec_max, void* mem, size_t mem_bytes,
                          cudaStream_t s, MatvecFn* out, int slot = 0);
size_t split_matvec_bytes(const LocalDims& L, int nvec_max);
void split_matvec_check(cudaStream_t s, int nslots = 1);
// Expansion-vector transform: on entry T (N x t) holds residual columns, X
// (N x nb) the current Ritz vectors and theta (device, t) their Ritz values;
// on exit T holds the correction directions.
using PrecFn = std::function<void(double* T, int t, const double* X, int nb, const double* theta)>;

// optional phase timing (host wall clock with stream syncs), TTG_PROFILE
struct DavTimer {
  cudaStream_t s = nullptr;
  double t[8] = {0};
  long long iters = 0, restarts = 0, jac_sweeps = 0;
};

struct DavidsonStats {
  int iters = 0;
  int matvecs = 0;
  double res = 0.0;      // 2-norm of the B residual norms
  double anorm = 0.0;
  bool converged = false;
};

class Davidson {
 public:
  // N: problem size, B: eigenpairs, maxb: basis limit, keep: restart size
  static size_t bytes(i64 N, int B, int maxb);
  Davidson(i64 N, int B, int maxb, int keep, void* mem, double* hostbuf, cudaStream_t s);
  // X0 (N x B) start block; on return X (N x B) Ritz vectors, theta (B, host)
  DavidsonStats solve(const MatvecFn& mv, const double* X0, double tol, int max_matvecs,
                      double* X, double* theta_host);
  DavTimer* timer = nullptr;
  PrecFn prec;          // optional correction-equation solver (JD expansion)
  bool gdk = true;      // keep the previous Ritz vectors at a restart (GD+k)

 private:
  i64 N_;
  int B_, maxb_, keep_;
  cudaStream_t s_;
  double *V_, *W_, *Vt_, *Wt_;
  double *H_, *Hs_, *S_, *theta_, *AX_, *R_, *rn2_;
  double *T_, *T2_, *Ct_, *G_, *Mfull_, *Sprev_, *C_, *HC_, *S2_;
  int kwarm_ = 0;
  double* theta_sel_ = nullptr;   // size of the previous Rayleigh-Ritz solve still valid as a warm start
  int *ikept_, *idx_;
  double* hbuf_;
  int k_ = 0;
  int kprev_ = 0;
  bool have_prev_ = false;
  int orth_block(double* T, int t, double* out);   // returns columns kept
  void sync();
};

// small kernels shared with other drivers
void residual_cols(i64 N, int nb, const double* AX, const double* X, const double* theta,
                   double* R, double* rn2, cudaStream_t s);
void gather_cols(i64 N, int t, const int* idx, const double* src, double* dst, cudaStream_t s);
int splitk_for(i64 K);

// learned preconditioner (ttg_learned.cu): the Davidson expansion hook of one
// local problem (D receives the operator's diagonal, N doubles), and the
// recorder of training problems
PrecFn make_learned_prec(ttg_mlp* M, const LocalDims& L, const double* phi1, const double* A,
                         const double* phi2, double* D, cudaStream_t s);
void learned_record(ttg_ctx* ctx, const LocalDims& L, const double* phi1, const double* A,
                    const double* phi2, const double* X0, const double* Xs, int B,
                    const MatvecFn& mv, cudaStream_t s);

}  // namespace ttg
