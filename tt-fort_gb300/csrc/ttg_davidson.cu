// Device block Davidson (GD+k).  Step-by-step twin of oracle/davidson.py.
#include "ttg_davidson.cuh"
#include <algorithm>
#include <chrono>
#include <cmath>

namespace ttg {

static constexpr double CHOL_DROP = 1e-14;
static constexpr double RESTART_DROP = 1e-10;

// ---------------------------------------------------------------------------
// Tall-skinny FP64 products of the Davidson basis.  GB300 runs FP64 at a few
// GFLOP/s per SM, so these spread the long dimension over every SM instead of
// padding small tiles.
// ---------------------------------------------------------------------------
constexpr int TS_MAXN = 16;

// C (M x N, ldc) = alpha * A^T B + beta * C, A (K x M, lda), B (K x N, ldb),
// N <= 16.  Grid (M, nk), one cluster of nk CTAs per column m of A: CTA
// (m, c) reduces k-chunk c against all N columns of B, then rank 0 adds the
// nk partials in rank order (deterministic, no atomics, no pre-scaling pass).
__global__ void tn_small_kernel(int M, int N, i64 K, const double* __restrict__ A, i64 lda,
                                const double* __restrict__ B, i64 ldb, double* __restrict__ C,
                                int ldc, double alpha, double beta, i64 kchunk) {
  namespace cgr = cooperative_groups;
  pdl_trigger();
  pdl_wait();
  const int m = blockIdx.x;
  const i64 k0 = blockIdx.y * kchunk, k1 = min(K, k0 + kchunk);
  double acc[TS_MAXN];
#pragma unroll
  for (int n = 0; n < TS_MAXN; ++n) acc[n] = 0.0;
  const double* a = A + lda * m;
  for (i64 k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    const double av = a[k];
#pragma unroll
    for (int n = 0; n < TS_MAXN; ++n)
      if (n < N) acc[n] = fma(av, B[k + ldb * n], acc[n]);
  }
  __shared__ double red[TS_MAXN][8];
  __shared__ double part[TS_MAXN];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int n = 0; n < TS_MAXN; ++n) {
    if (n >= N) break;
    double v = acc[n];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[n][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < N) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[threadIdx.x][w];
    part[threadIdx.x] = v;
  }
  cgr::cluster_group cl = cgr::this_cluster();
  cl.sync();
  if (cl.block_rank() == 0 && threadIdx.x < N) {
    double v = 0.0;
    for (unsigned r = 0; r < cl.num_blocks(); ++r) v += cl.map_shared_rank(part, r)[threadIdx.x];
    double* p = C + m + (i64)ldc * threadIdx.x;
    *p = beta == 0.0 ? alpha * v : fma(beta, *p, alpha * v);
  }
  cl.sync();
}

void gemm_tn_small(int M, int N, i64 K, const double* A, i64 lda, const double* B, i64 ldb,
                   double* C, int ldc, double alpha, double beta, cudaStream_t s) {
  if (M <= 0 || N <= 0) return;
  TTG_REQUIRE(N <= TS_MAXN, "gemm_tn_small: N > 16");
  TTG_REQUIRE(M < 65536, "gemm_tn_small: M too large");
  // about 2 CTAs per SM in total, at least 256 k per CTA, at most one cluster
  // of kMaxCluster CTAs per column
  i64 nk = std::max<i64>(1, std::min<i64>((304 + M - 1) / M, (K + 255) / 256));
  nk = std::min<i64>(nk, kMaxCluster);
  i64 kchunk = std::max<i64>(1, (K + nk - 1) / nk);
  launch_ex(tn_small_kernel, dim3(M, (unsigned)nk), dim3(256), dim3(1, (unsigned)nk, 1), true, 0, s,
            M, N, K, A, lda, B, ldb, C, ldc, alpha, beta, kchunk);
}

// C (R x N, ldc) = alpha * A (R x K, lda) * B (K x N, ldb) + beta * C, with
// K <= 128 and N <= 16: one thread per row, B in shared memory.
__global__ void nn_small_kernel(i64 R, int N, int K, const double* __restrict__ A, i64 lda,
                                const double* __restrict__ B, int ldb, double* __restrict__ C,
                                i64 ldc, double alpha, double beta) {
  __shared__ double Bs[128 * TS_MAXN];
  pdl_trigger();
  pdl_wait();
  for (int e = threadIdx.x; e < K * N; e += blockDim.x) Bs[e] = B[(e % K) + (i64)ldb * (e / K)];
  __syncthreads();
  for (i64 r = blockIdx.x * (i64)blockDim.x + threadIdx.x; r < R; r += (i64)gridDim.x * blockDim.x) {
    double acc[TS_MAXN];
#pragma unroll
    for (int n = 0; n < TS_MAXN; ++n) acc[n] = 0.0;
    for (int k = 0; k < K; ++k) {
      const double av = A[r + lda * k];
#pragma unroll
      for (int n = 0; n < TS_MAXN; ++n)
        if (n < N) acc[n] = fma(av, Bs[k + K * n], acc[n]);
    }
#pragma unroll
    for (int n = 0; n < TS_MAXN; ++n) {
      if (n >= N) break;
      double* p = C + r + ldc * n;
      *p = beta == 0.0 ? alpha * acc[n] : fma(beta, *p, alpha * acc[n]);
    }
  }
}

void gemm_nn_small(i64 R, int N, int K, const double* A, i64 lda, const double* B, int ldb,
                   double* C, i64 ldc, double alpha, double beta, cudaStream_t s) {
  if (R <= 0 || N <= 0) return;
  TTG_REQUIRE(N <= TS_MAXN && K <= 128, "gemm_nn_small: N > 16 or K > 128");
  int blocks = (int)std::min<i64>(2048, (R + 127) / 128);
  launch_pdl(nn_small_kernel, dim3(blocks), dim3(128), 0, s, R, N, K, A, lda, B, ldb, C, ldc, alpha,
             beta);
}

// R[:, j] = AX[:, j] - theta_j X[:, j];  rn2[j] = ||R[:, j]||^2.  Grid (bx, nb),
// the bx CTAs of column j are one cluster and add their partial sums in rank
// order (deterministic).
__global__ void residual_kernel(i64 N, const double* __restrict__ AX, const double* __restrict__ X,
                                const double* __restrict__ theta, double* __restrict__ R,
                                double* __restrict__ rn2) {
  pdl_trigger();
  pdl_wait();
  const int j = blockIdx.y;
  const double th = theta[j];
  double acc = 0.0;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += (i64)gridDim.x * blockDim.x) {
    double r = AX[i + N * j] - th * X[i + N * j];
    R[i + N * j] = r;
    acc = fma(r, r, acc);
  }
  const double t = cluster_sum(acc);
  if (blockIdx.x == 0 && threadIdx.x == 0) rn2[j] = t;
}

void residual_cols(i64 N, int nb, const double* AX, const double* X, const double* theta,
                   double* R, double* rn2, cudaStream_t s) {
  int bx = (int)std::max<i64>(1, std::min<i64>(kMaxCluster, (N + 1023) / 1024));
  launch_ex(residual_kernel, dim3(bx, nb), dim3(256), dim3(bx, 1, 1), true, 0, s, N, AX, X, theta,
            R, rn2);
}

__global__ void gather_cols_kernel(i64 N, int t, const int* idx, const double* src, double* dst) {
  pdl_trigger();
  pdl_wait();
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < N * t; e += (i64)gridDim.x * blockDim.x) {
    i64 i = e % N;
    int c = (int)(e / N);
    dst[e] = src[i + N * idx[c]];
  }
}

void gather_cols(i64 N, int t, const int* idx, const double* src, double* dst, cudaStream_t s) {
  int blocks = (int)std::min<i64>(4096, (N * t + 255) / 256);
  launch_pdl(gather_cols_kernel, dim3(blocks), dim3(256), 0, s, N, t, idx, src, dst);
}

// Cholesky with dropping of dependent columns (oracle.davidson.chol_drop).
// G (t x t, ld t).  Writes Mfull (t x t, ld t): rows of dropped columns are
// zero, the first nk columns hold L_k^{-T} scattered to the kept rows; kept[t]
// receives nk.  One warp, t <= 16; lane i owns row i.
__global__ void chol_drop_kernel(int t, const double* G, double* Mfull, int* kept, double tol) {
  __shared__ double L[16][17];
  __shared__ double Mi[16][17];
  __shared__ int kp[16];
  __shared__ int nk_s;
  const int lane = threadIdx.x;
  if (lane < 16)
    for (int j = 0; j < 16; ++j) L[lane][j] = 0.0;
  if (lane == 0) nk_s = 0;
  __syncwarp();
  for (int j = 0; j < t; ++j) {
    const int nk = nk_s;
    double gjj = G[j + t * j];
    double d = gjj;
    for (int q = 0; q < nk; ++q) d -= L[j][kp[q]] * L[j][kp[q]];
    const bool keep = (gjj > 0.0) && d > tol * gjj;
    if (keep) {
      const double ljj = sqrt(d);
      if (lane > j && lane < t) {
        double v = G[lane + t * j];
        for (int q = 0; q < nk; ++q) v -= L[lane][kp[q]] * L[j][kp[q]];
        L[lane][j] = v / ljj;
      }
      __syncwarp();
      if (lane == 0) { L[j][j] = ljj; kp[nk] = j; nk_s = nk + 1; }
    }
    __syncwarp();
  }
  const int nk = nk_s;
  // column c of Lk^{-T} (lane c): back substitution of Lk^T x = e_c
  if (lane < nk) {
    const int c = lane;
    for (int r = nk - 1; r >= 0; --r) {
      double v = (r == c) ? 1.0 : 0.0;
      for (int q = r + 1; q < nk; ++q) v -= L[kp[q]][kp[r]] * Mi[q][c];
      Mi[r][c] = v / L[kp[r]][kp[r]];
    }
  }
  __syncwarp();
  for (int e = lane; e < t * t; e += 32) Mfull[e] = 0.0;
  __syncwarp();
  for (int e = lane; e < nk * nk; e += 32) {
    const int r = e % nk, c = e / nk;
    Mfull[kp[r] + t * c] = Mi[r][c];
  }
  if (lane == 0) kept[t] = nk;
  if (lane < nk) kept[lane] = kp[lane];
}

// GD+k restart coefficients (oracle.davidson.restart_coeffs), one CTA.
// S (k x k, ld ldS): current Ritz vectors; Sprev (kprev x nb, ld ldP).
// C (k x kc, ld k) and out[0] = kc.
__global__ void restart_coeffs_kernel(int k, const double* S, int ldS, int kr, const double* Sprev,
                                      int kprev, int nb, int ldP, double* C, int* out, int maxkc) {
  extern __shared__ double sh[];
  double* Cs = sh;                  // k x (kr + nb)
  double* p = sh + (size_t)k * (kr + nb);
  __shared__ double red[33];
  __shared__ int kc_s;
  const int tid = threadIdx.x;
  for (int e = tid; e < k * kr; e += blockDim.x) Cs[e] = S[(e % k) + (size_t)ldS * (e / k)];
  if (tid == 0) kc_s = kr;
  __syncthreads();
  for (int b = 0; b < nb && Sprev; ++b) {
    if (kc_s >= maxkc) break;
    for (int i = tid; i < k; i += blockDim.x) p[i] = i < kprev ? Sprev[i + (size_t)ldP * b] : 0.0;
    __syncthreads();
    const int kc = kc_s;
    for (int pass = 0; pass < 2; ++pass) {
      for (int c = 0; c < kc; ++c) {
        // dot = C_c . p  (block reduction)
        double t = 0.0;
        for (int i = tid; i < k; i += blockDim.x) t += Cs[i + (size_t)k * c] * p[i];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if ((tid & 31) == 0) red[tid >> 5] = t;
        __syncthreads();
        if (tid < 32) {
          double u = tid < (int)(blockDim.x >> 5) ? red[tid] : 0.0;
          for (int o = 16; o > 0; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
          if (tid == 0) red[32] = u;
        }
        __syncthreads();
        double dot = red[32];
        for (int i = tid; i < k; i += blockDim.x) p[i] -= Cs[i + (size_t)k * c] * dot;
        __syncthreads();
      }
    }
    double t = 0.0;
    for (int i = tid; i < k; i += blockDim.x) t += p[i] * p[i];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((tid & 31) == 0) red[tid >> 5] = t;
    __syncthreads();
    if (tid < 32) {
      double u = tid < (int)(blockDim.x >> 5) ? red[tid] : 0.0;
      for (int o = 16; o > 0; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
      if (tid == 0) red[32] = u;
    }
    __syncthreads();
    double nrm = sqrt(red[32]);
    if (nrm > RESTART_DROP) {
      for (int i = tid; i < k; i += blockDim.x) Cs[i + (size_t)k * kc] = p[i] / nrm;
      __syncthreads();
      if (tid == 0) kc_s = kc + 1;
    }
    __syncthreads();
  }
  const int kc = kc_s;
  for (int e = tid; e < k * kc; e += blockDim.x) C[e] = Cs[e];
  if (tid == 0) out[0] = kc;
}

// H (ld ldh): H[0:k+t, k:k+t] = Hn; H[k:k+t, 0:k] = Hn[0:k,:]^T; H[k:,k:] sym.
__global__ void h_update_kernel(int k, int t, const double* Hn, double* H, int ldh) {
  const int K = k + t;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < K * t; e += gridDim.x * blockDim.x) {
    int r = e % K, c = e / K;
    double v = Hn[r + K * c];
    if (r < k) {
      H[r + ldh * (k + c)] = v;
      H[(k + c) + ldh * r] = v;
    } else {
      double w = Hn[(k + c) + K * (r - k)];
      H[r + ldh * (k + c)] = 0.5 * (v + w);
    }
  }
}

// H = 0.5 (H + H^T), k x k (ld ldh)
__global__ void symmetrize_kernel(int k, double* H, int ldh) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < k * k; e += gridDim.x * blockDim.x) {
    int r = e % k, c = e / k;
    if (r < c) {
      double v = 0.5 * (H[r + ldh * c] + H[c + ldh * r]);
      H[r + ldh * c] = v;
      H[c + ldh * r] = v;
    }
  }
}

__global__ void copy_mat_kernel(int rows, int cols, const double* src, int lds, double* dst, int ldd) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < rows * cols; e += gridDim.x * blockDim.x) {
    int r = e % rows, c = e / rows;
    dst[r + ldd * c] = src[r + lds * c];
  }
}

static void copy_mat(int rows, int cols, const double* src, int lds, double* dst, int ldd,
                     cudaStream_t s) {
  if (rows * cols <= 0) return;
  int blocks = std::min(1024, (rows * cols + 255) / 256);
  copy_mat_kernel<<<blocks, 256, 0, s>>>(rows, cols, src, lds, dst, ldd);
  TTG_CHECK_LAUNCH();
}

size_t Davidson::bytes(i64 N, int B, int maxb) {
  size_t nm = (size_t)N * maxb;
  size_t b = (size_t)maxb * maxb;
  size_t tot = 0;
  auto add = [&](size_t cnt) { tot += (cnt * sizeof(double) + 255) & ~size_t(255); };
  add(nm); add(nm); add(nm); add(nm);            // V W Vt Wt
  add(b); add(b); add(b); add(maxb);             // H Hs S theta
  add((size_t)N * B); add((size_t)N * B); add(64);   // AX R rn2
  add((size_t)N * B); add((size_t)N * B);        // T T2
  add((size_t)maxb * B); add(64 * 64); add(64 * 64); add((size_t)maxb * B);   // Ct G Mfull Sprev
  add(b); add(b); add(b); add(64);               // C HC S2 theta_sel
  add(64); add(64);                              // ikept idx
  return tot + 4096;
}

Davidson::Davidson(i64 N, int B, int maxb, int keep, void* mem, double* hostbuf, cudaStream_t s)
    : N_(N), B_(B), maxb_(maxb), keep_(keep), s_(s), hbuf_(hostbuf) {
  char* p = (char*)mem;
  auto take = [&](size_t cnt) {
    double* r = (double*)p;
    p += (cnt * sizeof(double) + 255) & ~size_t(255);
    return r;
  };
  size_t nm = (size_t)N * maxb, b = (size_t)maxb * maxb;
  V_ = take(nm); W_ = take(nm); Vt_ = take(nm); Wt_ = take(nm);
  H_ = take(b); Hs_ = take(b); S_ = take(b); theta_ = take(maxb);
  AX_ = take((size_t)N * B); R_ = take((size_t)N * B); rn2_ = take(64);
  T_ = take((size_t)N * B); T2_ = take((size_t)N * B);
  Ct_ = take((size_t)maxb * B); G_ = take(64 * 64); Mfull_ = take(64 * 64); Sprev_ = take((size_t)maxb * B);
  C_ = take(b); HC_ = take(b); S2_ = take(b);
  theta_sel_ = take(64);
  ikept_ = (int*)take(64); idx_ = (int*)take(64);
}

void Davidson::sync() { TTG_CUDA(cudaStreamSynchronize(s_)); }

// BCGS2 of T (N x t) against V[:, :k_]; result written to out (N x nk).
// Both passes are queued back to back: pass 1 writes its kept columns to the
// front of a t-column block and zeros behind them, which pass 2 drops again,
// so the host reads the final column count once.
int Davidson::orth_block(double* T, int t, double* out) {
  TTG_REQUIRE(t <= 16, "davidson: expansion block > 16");
  double* cur = T;
  for (int pass = 0; pass < 2; ++pass) {
    if (k_ > 0) {
      gemm_tn_small(k_, t, N_, V_, N_, cur, N_, Ct_, k_, 1.0, 0.0, s_);        // Ct = V^T cur
      gemm_nn_small(N_, t, k_, V_, N_, Ct_, k_, cur, N_, -1.0, 1.0, s_);      // cur -= V Ct
    }
    gemm_tn_small(t, t, N_, cur, N_, cur, N_, G_, t, 1.0, 0.0, s_);           // G = cur^T cur
    chol_drop_kernel<<<1, 32, 0, s_>>>(t, G_, Mfull_, ikept_ + 64 * pass, CHOL_DROP);
    TTG_CHECK_LAUNCH();
    double* dst = (pass == 0) ? (cur == T2_ ? T_ : T2_) : out;
    gemm_nn_small(N_, t, t, cur, N_, Mfull_, t, dst, N_, 1.0, 0.0, s_);       // dst = cur Mfull
    cur = dst;
  }
  TTG_CUDA(cudaMemcpyAsync(hbuf_, ikept_ + 64 + t, sizeof(int), cudaMemcpyDeviceToHost, s_));
  sync();
  return *(int*)hbuf_;
}

namespace {
struct Lap {
  DavTimer* t;
  std::chrono::steady_clock::time_point a;
  explicit Lap(DavTimer* tt) : t(tt) {
    if (t) { cudaStreamSynchronize(t->s); a = std::chrono::steady_clock::now(); }
  }
  void mark(int k) {
    if (!t) return;
    cudaStreamSynchronize(t->s);
    auto b = std::chrono::steady_clock::now();
    t->t[k] += std::chrono::duration<double>(b - a).count();
    a = b;
  }
};
}  // namespace

DavidsonStats Davidson::solve(const MatvecFn& mv, const double* X0, double tol, int max_matvecs,
                              double* X, double* theta_host) {
  DavidsonStats st;
  Lap lap(timer);
  const int ldh = maxb_;
  k_ = 0;
  kwarm_ = 0;
  have_prev_ = false;
  // initial basis: orth(X0), W = A V, H = V^T W
  TTG_CUDA(cudaMemcpyAsync(T_, X0, sizeof(double) * N_ * B_, cudaMemcpyDeviceToDevice, s_));
  int t = orth_block(T_, B_, V_);
  TTG_REQUIRE(t > 0, "davidson: start block has rank zero");
  mv(V_, W_, t);
  st.matvecs = t;
  k_ = t;
  gemm_tn_small(k_, k_, N_, V_, N_, W_, N_, H_, ldh, 1.0, 0.0, s_);   // H = V^T W
  symmetrize_kernel<<<1, 256, 0, s_>>>(k_, H_, ldh);
  TTG_CHECK_LAUNCH();
  double anorm = 0.0;
  int* status = (int*)(hbuf_ + 200);
  lap.mark(0);
  while (true) {
    st.iters++;
    if (timer) timer->iters++;
    const int k = k_;
    const int nb = std::min(B_, k);
    copy_mat(k, k, H_, ldh, Hs_, k, s_);
    // the previous eigenvectors (S_, kwarm_ x kwarm_) warm-start this solve
    syev_jacobi(k, Hs_, k, theta_, S2_, k, ikept_ + 40, s_, kwarm_ > 0 ? S_ : nullptr, kwarm_,
                kwarm_);
    std::swap(S_, S2_);
    kwarm_ = k;
    if (timer) {
      int js = 0;
      cudaMemcpyAsync(&js, ikept_ + 40, sizeof(int), cudaMemcpyDeviceToHost, s_);
      cudaStreamSynchronize(s_);
      timer->jac_sweeps += js;
    }
    lap.mark(1);
    gemm_nn_small(N_, nb, k, V_, N_, S_, k, X, N_, 1.0, 0.0, s_);     // X = V S[:, :nb]
    gemm_nn_small(N_, nb, k, W_, N_, S_, k, AX_, N_, 1.0, 0.0, s_);   // AX = W S[:, :nb]
    residual_cols(N_, nb, AX_, X, theta_, R_, rn2_, s_);
    TTG_CUDA(cudaMemcpyAsync(hbuf_, theta_, sizeof(double) * k, cudaMemcpyDeviceToHost, s_));
    TTG_CUDA(cudaMemcpyAsync(hbuf_ + 128, rn2_, sizeof(double) * nb, cudaMemcpyDeviceToHost, s_));
    sync();
    (void)status;
    lap.mark(2);
    const double* th = hbuf_;
    anorm = std::max(anorm, std::max(std::fabs(th[0]), std::fabs(th[k - 1])));
    int conv[64];
    int nconv = 0;
    double res2 = 0.0;
    for (int j = 0; j < nb; ++j) {
      double rn = std::sqrt(std::max(0.0, hbuf_[128 + j]));
      res2 += rn * rn;
      conv[j] = rn <= tol * anorm;
      nconv += conv[j];
      if (!std::isfinite(rn)) throw Error{TTG_ERR_NAN, "davidson: non-finite residual"};
    }
    for (int j = 0; j < nb; ++j) theta_host[j] = th[j];
    st.res = std::sqrt(res2);
    st.anorm = anorm;
    if (nconv == nb || st.matvecs >= max_matvecs || k >= N_) {
      st.converged = (nconv == nb);
      return st;
    }
    // expansion block: unconverged residual columns, in order
    int* hidx = (int*)(hbuf_ + 256);
    int tt = 0;
    for (int j = 0; j < nb; ++j)
      if (!conv[j]) hidx[tt++] = j;
    if (k + tt > maxb_) {
      // GD+k restart
      const int kr = std::min(keep_, k);
      size_t shm = sizeof(double) * ((size_t)k * (kr + B_) + k);
      restart_coeffs_kernel<<<1, 256, shm, s_>>>(k, S_, k, kr, have_prev_ ? Sprev_ : nullptr,
                                                 kprev_, (have_prev_ && gdk) ? B_ : 0, maxb_, C_,
                                                 ikept_ + 48, maxb_ - 1);
      TTG_CHECK_LAUNCH();
      TTG_CUDA(cudaMemcpyAsync(hbuf_ + 300, ikept_ + 48, sizeof(int), cudaMemcpyDeviceToHost, s_));
      sync();
      const int kc = *(int*)(hbuf_ + 300);
      if (kc <= 16) {
        gemm_nn_small(N_, kc, k, V_, N_, C_, k, Vt_, N_, 1.0, 0.0, s_);   // Vt = V C
        gemm_nn_small(N_, kc, k, W_, N_, C_, k, Wt_, N_, 1.0, 0.0, s_);   // Wt = W C
      } else {
        GemmF64 g;
        g.M = (int)N_; g.N = kc; g.K = k;
        g.A = V_; g.sAm = 1; g.sAk = N_;
        g.B = C_; g.sBk = 1; g.sBn = k;
        g.C = Vt_; g.sCm = 1; g.sCn = N_;
        gemm_f64(g, s_);
        g.A = W_; g.C = Wt_;
        gemm_f64(g, s_);
      }
      std::swap(V_, Vt_);
      std::swap(W_, Wt_);
      GemmF64 h;   // HC = H C (k x kc)
      h.M = k; h.N = kc; h.K = k;
      h.A = H_; h.sAm = 1; h.sAk = ldh;
      h.B = C_; h.sBk = 1; h.sBn = k;
      h.C = HC_; h.sCm = 1; h.sCn = k;
      gemm_f64(h, s_);
      GemmF64 q;   // H = C^T HC (kc x kc)
      q.M = kc; q.N = kc; q.K = k;
      q.A = C_; q.sAm = k; q.sAk = 1;
      q.B = HC_; q.sBk = 1; q.sBn = k;
      q.C = H_; q.sCm = 1; q.sCn = ldh;
      gemm_f64(q, s_);
      symmetrize_kernel<<<1, 256, 0, s_>>>(kc, H_, ldh);
      TTG_CHECK_LAUNCH();
      have_prev_ = false;
      k_ = kc;
      kwarm_ = 0;
      tt = std::max(1, std::min(tt, maxb_ - kc));
      if (timer) timer->restarts++;
      lap.mark(3);
    } else {
      copy_mat(k, nb, S_, k, Sprev_, maxb_, s_);
      kprev_ = k;
      have_prev_ = true;
    }
    TTG_CUDA(cudaMemcpyAsync(idx_, hidx, sizeof(int) * tt, cudaMemcpyHostToDevice, s_));
    gather_cols(N_, tt, idx_, R_, T_, s_);
    if (prec) {
      // shifts of the gathered columns for the correction equation
      double* hth = hbuf_ + 320;
      for (int q = 0; q < tt; ++q) hth[q] = theta_host[hidx[q]];
      TTG_CUDA(cudaMemcpyAsync(theta_sel_, hth, sizeof(double) * tt, cudaMemcpyHostToDevice, s_));
      prec(T_, tt, X, nb, theta_sel_);
    }
    const int kk = k_;
    int tn = orth_block(T_, tt, V_ + N_ * kk);
    if (tn == 0 && prec) {
      // Every transformed residual lay in span(V) (near convergence the
      // correction equation solved on the split operator returns directions
      // the basis already holds): expand with the FP64 residuals, which are
      // orthogonal to the Ritz vectors, so the iteration still progresses to
      // the FP64 tolerance instead of stopping short of it.
      gather_cols(N_, tt, idx_, R_, T_, s_);
      tn = orth_block(T_, tt, V_ + N_ * kk);
    }
    lap.mark(4);
    if (tn == 0) {
      st.converged = false;
      return st;
    }
    mv(V_ + N_ * kk, W_ + N_ * kk, tn);
    st.matvecs += tn;
    lap.mark(5);
    // Hn ((kk+tn) x tn) = V[:, :kk+tn]^T W[:, kk:kk+tn]
    gemm_tn_small(kk + tn, tn, N_, V_, N_, W_ + N_ * kk, N_, HC_, kk + tn, 1.0, 0.0, s_);
    h_update_kernel<<<1, 256, 0, s_>>>(kk, tn, HC_, H_, ldh);
    TTG_CHECK_LAUNCH();
    k_ = kk + tn;
    lap.mark(6);
  }
}

}  // namespace ttg
