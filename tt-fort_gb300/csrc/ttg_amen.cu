// AMEn linear solver (dtt_amen_solve, ttamen.f90:29-252) on the GPU, behind
// the flat-array entry point of tt_amen_solve (tt_adapt_als.f90:513).
//
// Every core, interface (X'AX, X'Y, Z'AX, Z'Y) and Krylov basis stays in
// HBM.  The sweep follows the reference step by step:
//   right-to-left: (z update), QR of x (and z) pushing R left, Phi updates
//   left-to-right: local rhs = Phi_XY y Phi_XY, residual, local solve
//     (dense LU below max_full_size, GMRES(40) x 2 otherwise), residual-based
//     SVD truncation (dtt_trunc), enrichment with the projected residual,
//     z update, QR of x and z to the right, Phi updates
//   stop when the largest local residual is below tol.
// Two GPU-shaped restatements keep the arithmetic but change the order:
//   * GMRES uses Arnoldi with classical Gram-Schmidt applied twice (the
//     reference applies Householder reflectors, ttlocsolve.f90:509-682);
//     both minimise the same residual over the same Krylov space;
//   * the truncation scan evaluates the candidate ranks from the top in
//     batches of 8 local matvecs and keeps the reference's rule: the chosen
//     rank is one more than the largest rank whose residual exceeds tol.
// The enrichment TT z starts from the splitmix64/Box-Muller stream shared
// with the oracle.
#include "ttg_davidson.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>

namespace ttg {

void gemm_tn_small(int M, int N, i64 K, const double* A, i64 lda, const double* B, i64 ldb,
                   double* C, int ldc, double alpha, double beta, cudaStream_t s);
void gemm_nn_small(i64 R, int N, int K, const double* A, i64 lda, const double* B, int ldb,
                   double* C, i64 ldc, double alpha, double beta, cudaStream_t s);

namespace {

inline int eb(i64 n) { return (int)std::max<i64>(1, std::min<i64>(4096, (n + 255) / 256)); }

__global__ void axpy_kernel(i64 n, double a, const double* x, double* y) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    y[i] = fma(a, x[i], y[i]);
}
// y = x - z
__global__ void sub_kernel(i64 n, const double* x, const double* z, double* y) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    y[i] = x[i] - z[i];
}
__global__ void scal_kernel(i64 n, const double* sdev, int invert, double* x) {
  const double s = invert ? 1.0 / sdev[0] : sdev[0];
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    x[i] *= s;
}
// out[j] += sum_i x[i + ld*j]^2  (pre-zeroed), grid (bx, ncols)
__global__ void sqnorm_cols_kernel(i64 n, const double* x, i64 ld, double* out) {
  const int j = blockIdx.y;
  double acc = 0.0;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const double v = x[i + ld * j];
    acc = fma(v, v, acc);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) atomicAdd(&out[j], t);
  }
}
__global__ void sqrt_kernel(int n, double* x) {
  if (threadIdx.x < n) x[threadIdx.x] = sqrt(x[threadIdx.x]);
}
// Y (n x c) = X[:, j] - rhs for every column j (residuals of candidates)
__global__ void sub_cols_kernel(i64 n, int c, const double* X, const double* rhs, double* Y) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n * c; e += (i64)gridDim.x * blockDim.x)
    Y[e] = X[e] - rhs[e % n];
}

// dense solve B x = b (N <= 64), partial pivoting (dgesv), one CTA
__global__ void lu_solve_kernel(int N, double* B, double* x, int* info) {
  __shared__ int piv;
  __shared__ double pv;
  for (int k = 0; k < N; ++k) {
    if (threadIdx.x == 0) {
      int p = k;
      double best = fabs(B[k + N * k]);
      for (int i = k + 1; i < N; ++i) {
        double v = fabs(B[i + N * k]);
        if (v > best) { best = v; p = i; }
      }
      piv = p;
      pv = best;
      if (best == 0.0) info[0] = k + 1;
    }
    __syncthreads();
    if (pv == 0.0) return;
    const int p = piv;
    if (p != k) {
      for (int j = threadIdx.x; j < N; j += blockDim.x) {
        double t = B[k + N * j]; B[k + N * j] = B[p + N * j]; B[p + N * j] = t;
      }
      if (threadIdx.x == 0) { double t = x[k]; x[k] = x[p]; x[p] = t; }
    }
    __syncthreads();
    const double d = B[k + N * k];
    for (int i = k + 1 + threadIdx.x; i < N; i += blockDim.x) B[i + N * k] /= d;
    __syncthreads();
    for (int e = threadIdx.x; e < (N - k - 1) * (N - k - 1); e += blockDim.x) {
      const int i = k + 1 + e % (N - k - 1), j = k + 1 + e / (N - k - 1);
      B[i + N * j] -= B[i + N * k] * B[k + N * j];
    }
    if (threadIdx.x == 0)
      for (int i = k + 1; i < N; ++i) x[i] -= B[i + N * k] * x[k];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int i = N - 1; i >= 0; --i) {
      double v = x[i];
      for (int j = i + 1; j < N; ++j) v -= B[i + N * j] * x[j];
      x[i] = v / B[i + N * i];
    }
  }
}

// GMRES Hessenberg column j (h[0..j+1]): apply previous rotations, make a
// new one, update g; res[0] = |g[j+1]|.  One thread.
__global__ void givens_kernel(int j, double* h, double* cs, double* sn, double* g, double* R,
                              int ldr, double* res) {
  for (int i = 0; i < j; ++i) {
    const double a = h[i], b = h[i + 1];
    h[i] = cs[i] * a + sn[i] * b;
    h[i + 1] = -sn[i] * a + cs[i] * b;
  }
  const double a = h[j], b = h[j + 1];
  const double den = hypot(a, b);
  const double c = den > 0 ? a / den : 1.0, s = den > 0 ? b / den : 0.0;
  cs[j] = c;
  sn[j] = s;
  h[j] = den;
  h[j + 1] = 0.0;
  g[j + 1] = -s * g[j];
  g[j] = c * g[j];
  for (int i = 0; i <= j; ++i) R[i + ldr * j] = h[i];
  res[0] = fabs(g[j + 1]);
}

// y = R^{-1} g (upper triangular k x k); one thread
__global__ void trsv_kernel(int k, const double* R, int ldr, const double* g, double* y) {
  for (int i = k - 1; i >= 0; --i) {
    double v = g[i];
    for (int j = i + 1; j < k; ++j) v -= R[i + ldr * j] * y[j];
    y[i] = v / R[i + ldr * i];
  }
}

// core_{k+1} with rho zero rows appended: out ((r+rho) x p) from in (r x p)
__global__ void pad_rows_kernel(i64 r, i64 rho, i64 p, const double* in, double* out) {
  const i64 R = r + rho;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < R * p; e += (i64)gridDim.x * blockDim.x) {
    const i64 i = e % R, c = e / R;
    out[e] = i < r ? in[i + r * c] : 0.0;
  }
}

// the identity block of ort0 for wide matrices: m x m identity
__global__ void eye_kernel(i64 m, double* out) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < m * m; e += (i64)gridDim.x * blockDim.x)
    out[e] = (e % m == e / m) ? 1.0 : 0.0;
}

}  // namespace

// splitmix64 uniform in (0, 1] and standard normal (Box-Muller), the stream
// the oracle uses for the enrichment TT z
static inline double sm_uniform(unsigned long long k) {
  unsigned long long z = k * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return ((double)(z >> 11) + 1.0) * 0x1.0p-53;
}
void sm_normals(unsigned long long seed, i64 count, double* out) {
  for (i64 i = 0; i < count; ++i) {
    const double u1 = sm_uniform(seed * 1000003ull + 2 * (unsigned long long)i + 1);
    const double u2 = sm_uniform(seed * 1000003ull + 2 * (unsigned long long)i + 2);
    out[i] = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.141592653589793 * u2);
  }
}


// ---------------------------------------------------------------------------
// the solver
// ---------------------------------------------------------------------------
namespace {

struct DevTT {
  std::vector<i64> n, r, cap;
  std::vector<double*> c;
  i64 size(int k) const { return r[k] * n[k] * r[k + 1]; }
};

struct Arena {
  char* base = nullptr;
  size_t top = 0, capb = 0;
  ~Arena() { if (base) cudaFree(base); }
  void alloc(size_t b) {
    if (cudaMalloc(&base, b) != cudaSuccess) {
      base = nullptr;
      throw Error{TTG_ERR_NOMEM, "amen: device allocation failed"};
    }
    capb = b;
  }
  double* take(size_t count) {
    size_t b = (count * sizeof(double) + 255) & ~size_t(255);
    if (top + b > capb) throw Error{TTG_ERR_NOMEM, "amen: device arena exhausted"};
    double* p = (double*)(base + top);
    top += b;
    return p;
  }
};

inline size_t al8(size_t count) { return (count * sizeof(double) + 255) & ~size_t(255); }

}  // namespace

struct AmenParams {
  int d;
  std::vector<i64> n, ra, ry, rx;
  const double *crA, *crY, *crX0;
  double tol;
  i64 rmax;
  int kick, nswp, local_iters, local_restart, max_full_size, verb;
  unsigned long long seed;
};

struct AmenOut {
  std::vector<double> cores;
  std::vector<i64> rx;
  int sweeps = 0;
  double res_max = 0.0;
  long long matvecs = 0;
};

class AmenSolver {
 public:
  AmenSolver(ttg_ctx* ctx, const AmenParams& P) : P_(P), s_(ctx->stream) {}
  void run(AmenOut& out);

 private:
  AmenParams P_;
  cudaStream_t s_;
  Arena mem_;
  DevTT x_, y_, z_;
  std::vector<double*> A_;
  std::vector<double*> pxax_, pxy_, pzax_, pzy_;
  double *tmpA_, *tmpB_, *tmpC_, *R_, *tau_, *rhs_, *resid_, *sol_, *xnew_, *scr_, *svU_, *svS_,
      *svVt_, *svScr_, *cand_, *candY_, *red_, *V_, *w_, *gm_, *dense_;
  double* h_ = nullptr;   // pinned
  long long nmv_ = 0;
  double real_tol_ = 0.0;
  static constexpr int kBatch = 8;

  void sync() { TTG_CUDA(cudaStreamSynchronize(s_)); }
  LocalDims dims(const DevTT& xx, const DevTT& yy, int k) const {
    return LocalDims{xx.r[k], xx.n[k], xx.r[k + 1], yy.r[k], yy.n[k], yy.r[k + 1], P_.ra[k], P_.ra[k + 1]};
  }
  double norm2(const double* v, i64 n) {
    TTG_CUDA(cudaMemsetAsync(red_, 0, sizeof(double), s_));
    int bx = (int)std::max<i64>(1, std::min<i64>(256, (n + 2047) / 2048));
    sqnorm_cols_kernel<<<dim3(bx, 1), 256, 0, s_>>>(n, v, n, red_);
    TTG_CHECK_LAUNCH();
    TTG_CUDA(cudaMemcpyAsync(h_, red_, sizeof(double), cudaMemcpyDeviceToHost, s_));
    sync();
    return std::sqrt(h_[0]);
  }
  void gemm(int M, int N, int K, const double* A, i64 sAm, i64 sAk, const double* B, i64 sBk,
            i64 sBn, double* C, i64 sCm, i64 sCn, double alpha = 1.0, double beta = 0.0) {
    GemmF64 g;
    g.M = M; g.N = N; g.K = K;
    g.A = A; g.sAm = sAm; g.sAk = sAk;
    g.B = B; g.sBk = sBk; g.sBn = sBn;
    g.C = C; g.sCm = sCm; g.sCn = sCn;
    g.alpha = alpha; g.beta = beta;
    gemm_f64(g, s_);
  }
  void qr(DevTT& t, int k, int dir);
  void yax(double* phi_new, const double* phi_old, const DevTT& yy, const DevTT& xx, int k, int dir,
           bool withA);
  // out (a.r[k] n x b.r[k+1]) = phi_l (a.r[k] x y.r[k]) y_k phi_r (y.r[k+1] x b.r[k+1])
  void project_y(const double* pl, const double* pr, i64 rl, i64 rr, int k, double* out);
  void local_mv(const LocalDims& L, const double* p1, const double* p2, int k, const double* x,
                double* yv, int nvec) {
    bfun3_f64(L, p1, A_[k], p2, x, yv, nvec, scr_, s_);
    nmv_ += nvec;
  }
  void gmres(const LocalDims& L, int k, const double* b, double* x, double tol);
  void trunc(int k, double tol, const double* rhs, double rhs_norm);
};

void AmenSolver::qr(DevTT& t, int k, int dir) {
  auto& n = t.n;
  auto& r = t.r;
  if (dir > 0) {
    const i64 m = r[k] * n[k], rr = r[k + 1], p = n[k + 1] * r[k + 2];
    if (m >= rr) {
      TTG_CUDA(cudaMemcpyAsync(tmpA_, t.c[k], sizeof(double) * m * rr, cudaMemcpyDeviceToDevice, s_));
      qr_householder((int)m, (int)rr, tmpA_, R_, tau_, s_);
      TTG_CUDA(cudaMemcpyAsync(t.c[k], tmpA_, sizeof(double) * m * rr, cudaMemcpyDeviceToDevice, s_));
      gemm((int)rr, (int)p, (int)rr, R_, 1, rr, t.c[k + 1], 1, rr, tmpB_, 1, rr);
      TTG_CUDA(cudaMemcpyAsync(t.c[k + 1], tmpB_, sizeof(double) * rr * p, cudaMemcpyDeviceToDevice, s_));
    } else {
      // ort0 of a wide block: identity core, the block moves right
      gemm((int)m, (int)p, (int)rr, t.c[k], 1, m, t.c[k + 1], 1, rr, tmpB_, 1, m);
      TTG_CUDA(cudaMemcpyAsync(t.c[k + 1], tmpB_, sizeof(double) * m * p, cudaMemcpyDeviceToDevice, s_));
      eye_kernel<<<eb(m * m), 256, 0, s_>>>(m, t.c[k]);
      TTG_CHECK_LAUNCH();
      r[k + 1] = m;
    }
  } else {
    const i64 m = n[k] * r[k + 1], rr = r[k], p = r[k - 1] * n[k - 1];
    transpose_f64(rr, m, t.c[k], tmpA_, s_);    // m x rr
    if (m >= rr) {
      qr_householder((int)m, (int)rr, tmpA_, R_, tau_, s_);
      transpose_f64(m, rr, tmpA_, t.c[k], s_);   // rr x m
      // core_{k-1} (p x rr) R^T
      gemm((int)p, (int)rr, (int)rr, t.c[k - 1], 1, p, R_, rr, 1, tmpB_, 1, p);
      TTG_CUDA(cudaMemcpyAsync(t.c[k - 1], tmpB_, sizeof(double) * p * rr, cudaMemcpyDeviceToDevice, s_));
    } else {
      // core_{k-1} (p x rr) * core_k (rr x m), core_k = I_m
      gemm((int)p, (int)m, (int)rr, t.c[k - 1], 1, p, t.c[k], 1, rr, tmpB_, 1, p);
      TTG_CUDA(cudaMemcpyAsync(t.c[k - 1], tmpB_, sizeof(double) * p * m, cudaMemcpyDeviceToDevice, s_));
      eye_kernel<<<eb(m * m), 256, 0, s_>>>(m, t.c[k]);
      TTG_CHECK_LAUNCH();
      r[k] = m;
    }
  }
}

void AmenSolver::yax(double* phi_new, const double* phi_old, const DevTT& yy, const DevTT& xx, int k,
                     int dir, bool withA) {
  if (withA) {
    LocalDims L = dims(xx, yy, k);
    if (dir > 0) phi_left_f64(L, phi_old, A_[k], xx.c[k], yy.c[k], phi_new, scr_, s_);
    else phi_right_f64(L, phi_old, A_[k], xx.c[k], yy.c[k], phi_new, scr_, s_);
  } else {
    if (dir > 0) phi2_left_f64(xx.r[k], xx.r[k + 1], yy.r[k], xx.n[k], yy.r[k + 1], phi_old, xx.c[k], yy.c[k], phi_new, scr_, s_);
    else phi2_right_f64(xx.r[k], xx.r[k + 1], yy.r[k], xx.n[k], yy.r[k + 1], phi_old, xx.c[k], yy.c[k], phi_new, scr_, s_);
  }
}

void AmenSolver::project_y(const double* pl, const double* pr, i64 rl, i64 rr, int k, double* out) {
  const i64 n = y_.n[k], y1 = y_.r[k], y2 = y_.r[k + 1];
  gemm((int)rl, (int)(n * y2), (int)y1, pl, 1, rl, y_.c[k], 1, y1, tmpC_, 1, rl);
  gemm((int)(rl * n), (int)rr, (int)y2, tmpC_, 1, rl * n, pr, 1, y2, out, 1, rl * n);
}


// GMRES(local_restart) x local_iters for L x = b (x0 = 0), Arnoldi with
// classical Gram-Schmidt twice, relative tolerance against ||b||.
void AmenSolver::gmres(const LocalDims& L, int k, const double* b, double* x, double tol) {
  const i64 N = L.xsize();
  const int nr = (int)std::min<i64>(std::min<i64>(N, P_.local_restart), 60);
  const double* p1 = pxax_[k];
  const double* p2 = pxax_[k + 1];
  double* H = gm_;                     // Hessenberg column (first pass)
  double* H2 = gm_ + 64;               // second Gram-Schmidt pass
  double* cs = gm_ + 128;
  double* sn = gm_ + 192;
  double* g = gm_ + 256;
  double* y = gm_ + 320;
  double* hres = gm_ + 384;
  double* Rm = gm_ + 448;              // (nr+1) x nr, nr <= 60
  const int ldr = nr + 1;
  TTG_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * N, s_));
  double nrmb = -1.0, curres = 1.0;
  for (int it = 0; it < P_.local_iters; ++it) {
    // w = b - L x
    local_mv(L, p1, p2, k, x, w_, 1);
    sub_kernel<<<eb(N), 256, 0, s_>>>(N, b, w_, w_);
    TTG_CHECK_LAUNCH();
    const double beta = norm2(w_, N);
    if (it == 0) nrmb = beta;
    if (beta == 0.0) break;
    TTG_CUDA(cudaMemcpyAsync(V_, w_, sizeof(double) * N, cudaMemcpyDeviceToDevice, s_));
    h_[1] = 1.0 / beta;
    TTG_CUDA(cudaMemcpyAsync(red_ + 8, h_ + 1, sizeof(double), cudaMemcpyHostToDevice, s_));
    scal_kernel<<<eb(N), 256, 0, s_>>>(N, red_ + 8, 0, V_);
    TTG_CHECK_LAUNCH();
    TTG_CUDA(cudaMemsetAsync(g, 0, sizeof(double) * 64, s_));
    h_[2] = beta;
    TTG_CUDA(cudaMemcpyAsync(g, h_ + 2, sizeof(double), cudaMemcpyHostToDevice, s_));
    int jdone = 0;
    for (int j = 0; j < nr; ++j) {
      double* vj = V_ + N * j;
      double* wv = V_ + N * (j + 1);
      local_mv(L, p1, p2, k, vj, wv, 1);
      // CGS2 against V[:, 0..j]
      gemm_tn_small(j + 1, 1, N, V_, N, wv, N, H, j + 2, 1.0, 0.0, s_);
      gemm_nn_small(N, 1, j + 1, V_, N, H, j + 2, wv, N, -1.0, 1.0, s_);
      gemm_tn_small(j + 1, 1, N, V_, N, wv, N, H2, j + 2, 1.0, 0.0, s_);
      gemm_nn_small(N, 1, j + 1, V_, N, H2, j + 2, wv, N, -1.0, 1.0, s_);
      axpy_kernel<<<1, 64, 0, s_>>>(j + 1, 1.0, H2, H);
      TTG_CHECK_LAUNCH();
      TTG_CUDA(cudaMemsetAsync(red_, 0, sizeof(double), s_));
      int bx = (int)std::max<i64>(1, std::min<i64>(256, (N + 2047) / 2048));
      sqnorm_cols_kernel<<<dim3(bx, 1), 256, 0, s_>>>(N, wv, N, red_);
      TTG_CHECK_LAUNCH();
      sqrt_kernel<<<1, 32, 0, s_>>>(1, red_);
      TTG_CHECK_LAUNCH();
      TTG_CUDA(cudaMemcpyAsync(H + j + 1, red_, sizeof(double), cudaMemcpyDeviceToDevice, s_));
      scal_kernel<<<eb(N), 256, 0, s_>>>(N, red_, 1, wv);
      TTG_CHECK_LAUNCH();
      givens_kernel<<<1, 1, 0, s_>>>(j, H, cs, sn, g, Rm, ldr, hres);
      TTG_CHECK_LAUNCH();
      TTG_CUDA(cudaMemcpyAsync(h_, hres, sizeof(double), cudaMemcpyDeviceToHost, s_));
      sync();
      jdone = j + 1;
      curres = h_[0] / nrmb;
      if (curres < tol) break;
    }
    trsv_kernel<<<1, 1, 0, s_>>>(jdone, Rm, ldr, g, y);
    TTG_CHECK_LAUNCH();
    gemm_nn_small(N, 1, jdone, V_, N, y, jdone, x, N, 1.0, 1.0, s_);
    if (curres < tol) break;
  }
}

// dtt_trunc dir=+1 with the residual criterion (ttnodeop.f90:227-302)
void AmenSolver::trunc(int k, double tol, const double* rhs, double rhs_norm) {
  auto& r = x_.r;
  const i64 n = x_.n[k];
  const i64 m = r[k] * n, rr = r[k + 1], p = x_.n[k + 1] * r[k + 2];
  const int rmin = (int)std::min(m, rr);
  // SVD of core k (m x rr): U (m x rmin), s, Vt (rmin x rr)
  svd_jacobi((int)m, (int)rr, x_.c[k], svU_, svS_, svVt_, svScr_, (int*)(red_ + 16), s_);
  // Vt rows scaled by s: W = diag(s) Vt
  scale_rows_f64(rmin, rr, svVt_, rmin, svS_, s_);
  LocalDims L = dims(x_, x_, k);
  const i64 N = L.xsize();
  int rnew = rmin - 1;
  int fail = 0;   // largest candidate rank whose residual exceeds tol (0: none)
  while (rnew >= 1 && !fail) {
    const int cnt = std::min(kBatch, rnew);
    // candidates rank rnew, rnew-1, ..., rnew-cnt+1: core_c = U[:, :rc] W[:rc, :]
    for (int c = 0; c < cnt; ++c) {
      const int rc = rnew - c;
      gemm((int)m, (int)rr, rc, svU_, 1, m, svVt_, 1, rmin, cand_ + N * c, 1, m);
    }
    local_mv(L, pxax_[k], pxax_[k + 1], k, cand_, candY_, cnt);
    sub_cols_kernel<<<eb(N * cnt), 256, 0, s_>>>(N, cnt, candY_, rhs, candY_);
    TTG_CHECK_LAUNCH();
    TTG_CUDA(cudaMemsetAsync(red_, 0, sizeof(double) * cnt, s_));
    int bx = (int)std::max<i64>(1, std::min<i64>(128, (N + 2047) / 2048));
    sqnorm_cols_kernel<<<dim3(bx, cnt), 256, 0, s_>>>(N, candY_, N, red_);
    TTG_CHECK_LAUNCH();
    TTG_CUDA(cudaMemcpyAsync(h_, red_, sizeof(double) * cnt, cudaMemcpyDeviceToHost, s_));
    sync();
    for (int c = 0; c < cnt; ++c) {
      if (std::sqrt(h_[c]) / rhs_norm > tol) {
        fail = rnew - c;
        break;
      }
    }
    rnew -= cnt;
  }
  int rk = fail + 1;
  if (rk > rmin) rk = rmin;
  rk = (int)std::min<i64>(rk, P_.rmax);
  // xnew = U[:, :rk] W[:rk, :] (m x rr), core k = U[:, :rk], core k+1 = W[:rk,:] core_{k+1}
  gemm((int)m, (int)rr, rk, svU_, 1, m, svVt_, 1, rmin, xnew_, 1, m);
  TTG_CUDA(cudaMemcpyAsync(x_.c[k], svU_, sizeof(double) * m * rk, cudaMemcpyDeviceToDevice, s_));
  gemm(rk, (int)p, (int)rr, svVt_, 1, rmin, x_.c[k + 1], 1, rr, tmpB_, 1, rk);
  TTG_CUDA(cudaMemcpyAsync(x_.c[k + 1], tmpB_, sizeof(double) * rk * p, cudaMemcpyDeviceToDevice, s_));
  r[k + 1] = rk;
}


void AmenSolver::run(AmenOut& out) {
  const int d = P_.d;
  auto& n = P_.n;
  const int kick = P_.kick;
  TTG_REQUIRE(d >= 2, "amen: d must be >= 2");
  TTG_REQUIRE(P_.rx[0] == 1 && P_.rx[d] == 1 && P_.ry[0] == 1 && P_.ry[d] == 1 &&
              P_.ra[0] == 1 && P_.ra[d] == 1, "boundary ranks must be 1");
  real_tol_ = P_.tol / std::sqrt((double)(d - 1)) / 2.0;   // resid_damp = 2
  // capacities: x ranks never exceed max(initial, rmax + kickrank) nor the
  // size of either side of the bond
  std::vector<i64> left(d + 1, 1), right(d + 1, 1);
  for (int k = 1; k <= d; ++k) left[k] = std::min<i64>(left[k - 1] * n[k - 1], 1ll << 40);
  for (int k = d - 1; k >= 0; --k) right[k] = std::min<i64>(right[k + 1] * n[k], 1ll << 40);
  x_.n = n; y_.n = n; z_.n = n;
  x_.r = P_.rx; y_.r = P_.ry;
  x_.cap.assign(d + 1, 1);
  for (int k = 1; k < d; ++k)
    x_.cap[k] = std::min(std::max(P_.rx[k], P_.rmax + kick), std::min(left[k], right[k]) + kick);
  z_.r.assign(d + 1, 1);
  for (int k = 1; k < d; ++k) z_.r[k] = kick > 0 ? kick : 1;
  i64 Nmax = 1, cmax = 1, pmax = 1, ramax = 1, ymax = 1;
  for (int k = 0; k < d; ++k) {
    Nmax = std::max(Nmax, x_.cap[k] * n[k] * x_.cap[k + 1]);
    ramax = std::max(ramax, P_.ra[k + 1]);
    ymax = std::max(ymax, P_.ry[k + 1]);
  }
  cmax = Nmax;
  for (int k = 0; k <= d; ++k) pmax = std::max(pmax, x_.cap[k] * x_.cap[k] * P_.ra[k]);
  size_t scr = 0;
  for (int k = 0; k < d; ++k) {
    LocalDims L{x_.cap[k], n[k], x_.cap[k + 1], x_.cap[k], n[k], x_.cap[k + 1], P_.ra[k], P_.ra[k + 1]};
    scr = std::max(scr, bfun3_f64_scratch(L, kBatch));
    scr = std::max(scr, phi_f64_scratch(L));
  }
  size_t svds = 0;
  for (int k = 0; k < d; ++k) svds = std::max(svds, svd_scratch((int)(x_.cap[k] * n[k]), (int)x_.cap[k + 1]));
  const int nr = (int)std::min<i64>(std::min<i64>(Nmax, P_.local_restart), 60);
  i64 yt = 0;
  for (int k = 0; k < d; ++k) yt += P_.ry[k] * n[k] * P_.ry[k + 1];
  i64 at = 0;
  for (int k = 0; k < d; ++k) at += P_.ra[k] * n[k] * n[k] * P_.ra[k + 1];
  i64 tcap = cmax;
  for (int k = 0; k < d; ++k)
    tcap = std::max(tcap, std::max(x_.cap[k], z_.r[k]) * n[k] * std::max(ymax, P_.ry[k]));
  size_t total = al8(at);
  for (int k = 0; k < d; ++k) total += al8(x_.cap[k] * n[k] * x_.cap[k + 1]) + al8(P_.ry[k] * n[k] * P_.ry[k + 1]) +
                                       al8(z_.r[k] * n[k] * z_.r[k + 1]);
  for (int k = 0; k <= d; ++k)
    total += al8(x_.cap[k] * x_.cap[k] * P_.ra[k]) + al8(x_.cap[k] * P_.ry[k]) +
             al8(z_.r[k] * x_.cap[k] * P_.ra[k]) + al8(z_.r[k] * P_.ry[k]);
  total += 2 * al8(cmax) + al8(tcap) + al8(Nmax) * 5 + al8(cmax) + al8(8192) + scr + 256;
  total += svds + 256 + 3 * al8(cmax) + al8(8192);
  total += 2 * al8(Nmax * kBatch) + al8(Nmax * (nr + 1)) + al8(Nmax) + al8(4096) +
           al8((size_t)std::min<i64>(P_.max_full_size, 64) * 64) + (1 << 16);
  mem_.alloc(total);
  double* dA = mem_.take(at);
  A_.resize(d);
  {
    i64 off = 0;
    for (int k = 0; k < d; ++k) { A_[k] = dA + off; off += P_.ra[k] * n[k] * n[k] * P_.ra[k + 1]; }
  }
  x_.c.resize(d); y_.c.resize(d); z_.c.resize(d);
  for (int k = 0; k < d; ++k) {
    x_.c[k] = mem_.take(x_.cap[k] * n[k] * x_.cap[k + 1]);
    y_.c[k] = mem_.take(P_.ry[k] * n[k] * P_.ry[k + 1]);
    z_.c[k] = mem_.take(z_.r[k] * n[k] * z_.r[k + 1]);
  }
  pxax_.resize(d + 1); pxy_.resize(d + 1); pzax_.resize(d + 1); pzy_.resize(d + 1);
  for (int k = 0; k <= d; ++k) {
    pxax_[k] = mem_.take(x_.cap[k] * x_.cap[k] * P_.ra[k]);
    pxy_[k] = mem_.take(x_.cap[k] * P_.ry[k]);
    pzax_[k] = mem_.take(z_.r[k] * x_.cap[k] * P_.ra[k]);
    pzy_[k] = mem_.take(z_.r[k] * P_.ry[k]);
  }
  tmpA_ = mem_.take(cmax); tmpB_ = mem_.take(cmax); tmpC_ = mem_.take(tcap);
  rhs_ = mem_.take(Nmax); resid_ = mem_.take(Nmax); sol_ = mem_.take(Nmax); xnew_ = mem_.take(Nmax);
  w_ = mem_.take(Nmax);
  R_ = mem_.take(cmax);
  tau_ = mem_.take(8192);
  scr_ = (double*)mem_.take(scr / sizeof(double) + 1);
  svScr_ = (double*)mem_.take(svds / sizeof(double) + 1);
  svU_ = mem_.take(cmax); svS_ = mem_.take(8192); svVt_ = mem_.take(cmax);
  cand_ = mem_.take(Nmax * kBatch); candY_ = mem_.take(Nmax * kBatch);
  V_ = mem_.take(Nmax * (nr + 1));
  red_ = mem_.take(64);
  gm_ = mem_.take(4096);
  dense_ = mem_.take(64 * 64);
  TTG_CUDA(cudaMallocHost(&h_, 4096 * sizeof(double)));
  struct HG { double* p; ~HG() { if (p) cudaFreeHost(p); } } hg{h_};

  // upload
  TTG_CUDA(cudaMemcpyAsync(dA, P_.crA, sizeof(double) * at, cudaMemcpyHostToDevice, s_));
  {
    i64 ox = 0, oy = 0;
    for (int k = 0; k < d; ++k) {
      TTG_CUDA(cudaMemcpyAsync(x_.c[k], P_.crX0 + ox, sizeof(double) * x_.size(k), cudaMemcpyHostToDevice, s_));
      TTG_CUDA(cudaMemcpyAsync(y_.c[k], P_.crY + oy, sizeof(double) * y_.size(k), cudaMemcpyHostToDevice, s_));
      ox += x_.size(k);
      oy += y_.size(k);
    }
  }
  if (kick > 0) {
    i64 zt = 0;
    for (int k = 0; k < d; ++k) zt += z_.size(k);
    std::vector<double> zh(zt);
    sm_normals(P_.seed, zt, zh.data());
    i64 oz = 0;
    for (int k = 0; k < d; ++k) {
      TTG_CUDA(cudaMemcpyAsync(z_.c[k], zh.data() + oz, sizeof(double) * z_.size(k), cudaMemcpyHostToDevice, s_));
      oz += z_.size(k);
    }
    sync();
  }
  for (double* ph : {pxax_[0], pxax_[d], pxy_[0], pxy_[d], pzax_[0], pzax_[d], pzy_[0], pzy_[d]})
    fill_f64(ph, 1, 1.0, s_);

  int swp_done = 0;
  double res_max = 0.0;
  for (int swp = 1; swp <= P_.nswp; ++swp) {
    swp_done = swp;
    for (int k = d - 1; k >= 1; --k) {
      if (kick > 0 && swp > 1) {
        LocalDims Lz = dims(x_, z_, k);
        local_mv(Lz, pzax_[k], pzax_[k + 1], k, x_.c[k], z_.c[k], 1);
        project_y(pzy_[k], pzy_[k + 1], z_.r[k], z_.r[k + 1], k, rhs_);
        sub_kernel<<<eb(z_.size(k)), 256, 0, s_>>>(z_.size(k), z_.c[k], rhs_, z_.c[k]);
        TTG_CHECK_LAUNCH();
      }
      qr(x_, k, -1);
      yax(pxax_[k], pxax_[k + 1], x_, x_, k, -1, true);
      yax(pxy_[k], pxy_[k + 1], x_, y_, k, -1, false);
      if (kick > 0) {
        qr(z_, k, -1);
        yax(pzax_[k], pzax_[k + 1], z_, x_, k, -1, true);
        yax(pzy_[k], pzy_[k + 1], z_, y_, k, -1, false);
      }
    }
    res_max = 0.0;
    double err_max = 0.0;
    for (int k = 0; k < d; ++k) {
      const i64 rx1 = x_.r[k], rx2 = x_.r[k + 1];
      LocalDims L = dims(x_, x_, k);
      const i64 N = L.xsize();
      project_y(pxy_[k], pxy_[k + 1], rx1, rx2, k, rhs_);
      local_mv(L, pxax_[k], pxax_[k + 1], k, x_.c[k], resid_, 1);
      sub_kernel<<<eb(N), 256, 0, s_>>>(N, resid_, rhs_, resid_);
      TTG_CHECK_LAUNCH();
      const double nr_rhs = norm2(rhs_, N);
      double err = norm2(resid_, N) / nr_rhs;
      res_max = std::max(res_max, err);
      if (err > real_tol_) {
        if (N < P_.max_full_size && N <= 64) {
          fullmat_f64(rx1, n[k], rx2, P_.ra[k], P_.ra[k + 1], pxax_[k], A_[k], pxax_[k + 1], dense_, s_);
          TTG_CUDA(cudaMemcpyAsync(sol_, resid_, sizeof(double) * N, cudaMemcpyDeviceToDevice, s_));
          TTG_CUDA(cudaMemsetAsync(red_ + 32, 0, sizeof(int), s_));
          lu_solve_kernel<<<1, 256, 0, s_>>>((int)N, dense_, sol_, (int*)(red_ + 32));
          TTG_CHECK_LAUNCH();
        } else {
          gmres(L, k, resid_, sol_, real_tol_ / err);
        }
        sub_kernel<<<eb(N), 256, 0, s_>>>(N, x_.c[k], sol_, x_.c[k]);
        TTG_CHECK_LAUNCH();
        err_max = std::max(err_max, norm2(sol_, N) / norm2(x_.c[k], N));
        local_mv(L, pxax_[k], pxax_[k + 1], k, x_.c[k], resid_, 1);
        sub_kernel<<<eb(N), 256, 0, s_>>>(N, resid_, rhs_, resid_);
        TTG_CHECK_LAUNCH();
        err = norm2(resid_, N) / nr_rhs;
      }
      if (k < d - 1) {
        if (kick > 0) {
          err = std::max(err, real_tol_ * 2.0);
          trunc(k, err, rhs_, nr_rhs);
          // sol = A xnew projected on (x-left, z-right) - Phi_XY y Phi_ZY
          LocalDims Lxz{rx1, n[k], rx2, rx1, n[k], z_.r[k + 1], P_.ra[k], P_.ra[k + 1]};
          local_mv(Lxz, pxax_[k], pzax_[k + 1], k, xnew_, sol_, 1);
          LocalDims Lzz{rx1, n[k], rx2, z_.r[k], n[k], z_.r[k + 1], P_.ra[k], P_.ra[k + 1]};
          local_mv(Lzz, pzax_[k], pzax_[k + 1], k, xnew_, z_.c[k], 1);
          project_y(pxy_[k], pzy_[k + 1], rx1, z_.r[k + 1], k, rhs_);
          sub_kernel<<<eb(rx1 * n[k] * z_.r[k + 1]), 256, 0, s_>>>(rx1 * n[k] * z_.r[k + 1], sol_, rhs_, sol_);
          TTG_CHECK_LAUNCH();
          project_y(pzy_[k], pzy_[k + 1], z_.r[k], z_.r[k + 1], k, rhs_);
          sub_kernel<<<eb(z_.size(k)), 256, 0, s_>>>(z_.size(k), z_.c[k], rhs_, z_.c[k]);
          TTG_CHECK_LAUNCH();
          // enrich: core k = [core k | sol], core k+1 gets zero rows
          const i64 rho = z_.r[k + 1];
          const i64 m = x_.r[k] * n[k], rk = x_.r[k + 1], p = n[k + 1] * x_.r[k + 2];
          TTG_REQUIRE(rk + rho <= x_.cap[k + 1], "amen: rank capacity exceeded");
          TTG_CUDA(cudaMemcpyAsync(x_.c[k] + m * rk, sol_, sizeof(double) * m * rho,
                                   cudaMemcpyDeviceToDevice, s_));
          pad_rows_kernel<<<eb((rk + rho) * p), 256, 0, s_>>>(rk, rho, p, x_.c[k + 1], tmpB_);
          TTG_CHECK_LAUNCH();
          TTG_CUDA(cudaMemcpyAsync(x_.c[k + 1], tmpB_, sizeof(double) * (rk + rho) * p,
                                   cudaMemcpyDeviceToDevice, s_));
          x_.r[k + 1] = rk + rho;
          qr(x_, k, +1);
          qr(z_, k, +1);
          yax(pzax_[k + 1], pzax_[k], z_, x_, k, +1, true);
          yax(pzy_[k + 1], pzy_[k], z_, y_, k, +1, false);
        } else {
          qr(x_, k, +1);
        }
        yax(pxax_[k + 1], pxax_[k], x_, x_, k, +1, true);
        yax(pxy_[k + 1], pxy_[k], x_, y_, k, +1, false);
      }
    }
    if (P_.verb > 0) {
      i64 mr = *std::max_element(x_.r.begin(), x_.r.end());
      fprintf(stderr, "amen_solve: swp=%d, max_dx=%.3e, max_res=%.3e, max_rank=%lld\n", swp,
              err_max, res_max, (long long)mr);
    }
    if (res_max < P_.tol) break;
  }
  sync();
  i64 tot = 0;
  for (int k = 0; k < d; ++k) tot += x_.size(k);
  out.cores.resize(tot);
  i64 off = 0;
  for (int k = 0; k < d; ++k) {
    TTG_CUDA(cudaMemcpyAsync(out.cores.data() + off, x_.c[k], sizeof(double) * x_.size(k),
                             cudaMemcpyDeviceToHost, s_));
    off += x_.size(k);
  }
  sync();
  out.rx = x_.r;
  out.sweeps = swp_done;
  out.res_max = res_max;
  out.matvecs = nmv_;
}

}  // namespace ttg

using namespace ttg;

extern "C" int ttg_amen_solve(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* m,
                              const ttg_int* ry, const ttg_int* ra, const double* crA,
                              const double* crY, const double* crX0, ttg_int* rx, double eps,
                              ttg_int rmax, ttg_int kickrank, ttg_int nswp, int verb, int method) {
  if (!ctx) return TTG_ERR_ARG;
  try {
    TTG_CUDA(cudaSetDevice(ctx->device));
    TTG_REQUIRE(d > 1 && n && m && ry && ra && crA && crY && crX0 && rx, "null argument");
    TTG_REQUIRE(method == TTG_METHOD_PLAIN, "amen: only the FP64 method is built");
    for (int k = 0; k < d; ++k) TTG_REQUIRE(n[k] == m[k], "amen needs square cores (n == m)");
    AmenParams P;
    P.d = (int)d;
    P.n.assign(n, n + d);
    P.ry.assign(ry, ry + d + 1);
    P.ra.assign(ra, ra + d + 1);
    P.rx.assign(rx, rx + d + 1);
    P.crA = crA; P.crY = crY; P.crX0 = crX0;
    P.tol = eps;
    P.rmax = rmax > 0 ? rmax : (1ll << 30);
    P.kick = kickrank >= 0 ? (int)kickrank : 4;
    P.nswp = nswp > 0 ? (int)nswp : 20;
    P.local_iters = 2;
    P.local_restart = 40;
    P.max_full_size = 50;
    P.verb = verb;
    P.seed = 0;
    long long l0 = g_launches;
    AmenOut out;
    AmenSolver solver(ctx, P);
    solver.run(out);
    for (int k = 0; k <= d; ++k) rx[k] = out.rx[k];
    ctx->result_core = std::move(out.cores);
    ctx->zresult_core.clear();
    ctx->stat_matvecs = out.matvecs;
    ctx->stat_sweeps = out.sweeps;
    ctx->stat_res = out.res_max;
    ctx->stat_launches = g_launches - l0;
  } catch (const ttg::Error& e) {
    ctx->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}
