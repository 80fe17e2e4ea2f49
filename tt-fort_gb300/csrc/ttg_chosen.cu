// Chosen-form local eigensolver: split-precision tensor-core matvecs with an
// FP64 judge.
//
// Phase A: Jacobi-Davidson (basis <= 2B, restarted to the B Ritz vectors
//          every iteration) driven entirely by the BF16x3 tensor-core
//          operator (ttg_tc.cu) until its residual, measured with that
//          operator, is below max(tol, 1e-4) * max|theta|.
// Phase B: Jacobi-Davidson refinement in FP64.  The Rayleigh-Ritz projection,
//          the residuals and the convergence test use FP64 matvecs; the new
//          directions solve the correction equation
//              (I - X X^T)(A~ - theta_j I)(I - X X^T) t_j = -r_j
//          approximately by a fixed number of CG steps with the split operator
//          A~ (batched over the unconverged columns, every scalar kept on the
//          device, no host synchronisation inside).  The projected operator
//          is positive definite on the complement of the wanted eigenvectors,
//          so CG applies; each outer step gains about the accuracy of A~
//          (1e-5) times the conditioning of the correction equation.
// The FP64 matvecs of phase B are the judge: the returned eigenpairs meet the
// same FP64 residual test as the plain method.
#include "ttg_davidson.cuh"
#include <algorithm>
#include <cstdlib>

namespace ttg {

// ---------------------------------------------------------------------------
// Deterministic grid sums.  The blocks of a group each write one partial sum
// to part[group * nblk + block]; the block that finishes last (a ticket
// counter, zero between uses) adds the partials in block order with a fixed
// lane assignment and shuffle tree, writes the total and resets the counter.
// The result does not depend on which block finishes first, so the CG
// correction below is bit-reproducible.
// ---------------------------------------------------------------------------
constexpr int CG_MAXT = 16;        // columns of a CG block
constexpr int CG_MAXBX = 128;      // blocks per column of col_dots / cg_update
constexpr int CG_MAXPB = 1024;     // blocks of proj_dot

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block sum of v, in thread 0
__device__ __forceinline__ double block_sum_d(double v, double* red) {
  v = warp_sum_d(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    t = warp_sum_d(t);
  }
  return t;
}

// Called by every thread after thread 0 stored this block's partials
// (ngroups of them at part[g * nblk + blk]).  Returns true in all threads of
// the last block to arrive.
__device__ __forceinline__ bool grid_sum_arrive(unsigned int* count, unsigned int nblk) {
  __shared__ int last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(count, 1u) == nblk - 1;
  }
  __syncthreads();
  return last != 0;
}

// In the last block: out[g] = sum_b part[g * nblk + b] for g < ngroups (warp w
// takes groups w, w + nwarps, ...), then the counter is reset.
__device__ __forceinline__ void grid_sum_finish(const double* part, int nblk, int ngroups,
                                                double* out, unsigned int* count) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int g = w; g < ngroups; g += nw) {
    double v = 0.0;
    for (int b = lane; b < nblk; b += 32) v += __ldcg(part + (size_t)g * nblk + b);
    v = warp_sum_d(v);
    if (lane == 0) out[g] = v;
  }
  if (threadIdx.x == 0) *count = 0u;
}

// out[j] = sum_i U[i,j] V[i,j]; grid (bx, t), deterministic (part: t x bx,
// count: t counters)
__global__ void col_dots_kernel(i64 N, const double* __restrict__ U, const double* __restrict__ V,
                                double* __restrict__ out, double* __restrict__ part,
                                unsigned int* __restrict__ count) {
  pdl_trigger();
  pdl_wait();
  const int j = blockIdx.y;
  double acc = 0.0;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += (i64)gridDim.x * blockDim.x)
    acc = fma(U[i + N * j], V[i + N * j], acc);
  __shared__ double red[32];
  const double t = block_sum_d(acc, red);
  if (threadIdx.x == 0) part[(size_t)j * gridDim.x + blockIdx.x] = t;
  if (grid_sum_arrive(count + j, gridDim.x))
    grid_sum_finish(part + (size_t)j * gridDim.x, gridDim.x, 1, out + j, count + j);
}

static void col_dots(i64 N, int t, const double* U, const double* V, double* out, double* part,
                     unsigned int* count, cudaStream_t s) {
  TTG_REQUIRE(t <= CG_MAXT, "col_dots: too many columns");
  int bx = (int)std::max<i64>(1, std::min<i64>(CG_MAXBX, (N + 2047) / 2048));
  launch_pdl(col_dots_kernel, dim3(bx, t), dim3(256), 0, s, N, U, V, out, part, count);
}

// q[:, j] -= theta_j p[:, j]; block 0 also clears the step's accumulators
// pq and rr_new (nothing reads them before they are summed again)
__global__ void shift_kernel(i64 N, int t, const double* __restrict__ theta,
                             const double* __restrict__ p, double* __restrict__ q,
                             double* __restrict__ pq, double* __restrict__ rr_new) {
  pdl_trigger();
  pdl_wait();
  if (blockIdx.x == 0 && threadIdx.x < t) {
    pq[threadIdx.x] = 0.0;
    rr_new[threadIdx.x] = 0.0;
  }
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < N * t; e += (i64)gridDim.x * blockDim.x)
    q[e] -= theta[e / N] * p[e];
}

// q -= X C (X: N x nb, C: nb x t) and pq[j] = p[:, j]^T q[:, j]: the
// projection of the CG step fused with its p^T q (deterministic grid sum:
// part t x gridDim.x, one counter)
constexpr int PD_MAXT = 16;
__global__ void __launch_bounds__(128) proj_dot_kernel(i64 N, int t, int nb,
                                                       const double* __restrict__ X,
                                                       const double* __restrict__ C,
                                                       const double* __restrict__ p,
                                                       double* __restrict__ q,
                                                       double* __restrict__ pq,
                                                       double* __restrict__ part,
                                                       unsigned int* __restrict__ count) {
  __shared__ double Cs[PD_MAXT * PD_MAXT];
  __shared__ double red[4][PD_MAXT];
  pdl_trigger();
  pdl_wait();
  for (int e = threadIdx.x; e < nb * t; e += blockDim.x) Cs[e] = C[e];
  __syncthreads();
  double acc[PD_MAXT];
#pragma unroll
  for (int j = 0; j < PD_MAXT; ++j) acc[j] = 0.0;
  for (i64 r = blockIdx.x * (i64)blockDim.x + threadIdx.x; r < N; r += (i64)gridDim.x * blockDim.x) {
    double xr[PD_MAXT];
#pragma unroll
    for (int k = 0; k < PD_MAXT; ++k) xr[k] = k < nb ? X[r + N * k] : 0.0;
#pragma unroll
    for (int j = 0; j < PD_MAXT; ++j) {
      if (j >= t) break;
      double v = q[r + N * j];
#pragma unroll
      for (int k = 0; k < PD_MAXT; ++k)
        if (k < nb) v = fma(-xr[k], Cs[k + nb * j], v);
      q[r + N * j] = v;
      acc[j] = fma(p[r + N * j], v, acc[j]);
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < PD_MAXT; ++j) {
    if (j >= t) break;
    double v = acc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[w][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < t) {
    const double v = red[0][threadIdx.x] + red[1][threadIdx.x] + red[2][threadIdx.x] + red[3][threadIdx.x];
    part[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = v;
    __threadfence();
  }
  __syncthreads();
  if (grid_sum_arrive(count, gridDim.x)) grid_sum_finish(part, gridDim.x, t, pq, count);
}

// CG step on column j (frozen when inactive or when p^T q <= 0):
//   alpha = rr/pq; x += alpha p; r -= alpha q; rr_new = |r|^2 (deterministic
//   grid sum over the bx blocks of the column)
__global__ void cg_update_kernel(i64 N, const double* __restrict__ rr, const double* __restrict__ pq,
                                 const double* __restrict__ rr0, double tol2,
                                 const double* __restrict__ p, const double* __restrict__ q,
                                 double* __restrict__ x, double* __restrict__ r,
                                 double* __restrict__ rr_new, double* __restrict__ part,
                                 unsigned int* __restrict__ count) {
  pdl_trigger();
  pdl_wait();
  const int j = blockIdx.y;
  const bool active = pq[j] > 0.0 && rr[j] > tol2 * rr0[j];
  const double alpha = active ? rr[j] / pq[j] : 0.0;
  double acc = 0.0;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += (i64)gridDim.x * blockDim.x) {
    const i64 e = i + N * j;
    double rv = r[e];
    if (active) {
      x[e] = fma(alpha, p[e], x[e]);
      rv = fma(-alpha, q[e], rv);
      r[e] = rv;
    }
    acc = fma(rv, rv, acc);
  }
  __shared__ double red[32];
  const double t = block_sum_d(acc, red);
  if (threadIdx.x == 0) part[(size_t)j * gridDim.x + blockIdx.x] = t;
  if (grid_sum_arrive(count + j, gridDim.x))
    grid_sum_finish(part + (size_t)j * gridDim.x, gridDim.x, 1, rr_new + j, count + j);
}

// p = r + beta p, beta = rr_new / rr (0 for frozen columns)
__global__ void cg_dir_kernel(i64 N, int t, const double* __restrict__ rr,
                              const double* __restrict__ rr_new, const double* __restrict__ pq,
                              const double* __restrict__ rr0, double tol2,
                              const double* __restrict__ r, double* __restrict__ p) {
  pdl_trigger();
  pdl_wait();
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < N * t; e += (i64)gridDim.x * blockDim.x) {
    const int j = (int)(e / N);
    const bool active = pq[j] > 0.0 && rr[j] > tol2 * rr0[j];
    const double beta = (active && rr[j] > 0.0) ? rr_new[j] / rr[j] : 0.0;
    p[e] = r[e] + beta * p[e];
  }
}

void gemm_tn_small(int M, int N, i64 K, const double* A, i64 lda, const double* B, i64 ldb,
                   double* C, int ldc, double alpha, double beta, cudaStream_t s);
void gemm_nn_small(i64 R, int N, int K, const double* A, i64 lda, const double* B, int ldb,
                   double* C, i64 ldc, double alpha, double beta, cudaStream_t s);

struct JdCg {
  i64 N;
  int Bmax;
  int iters;
  double rel_tol;      // inner residual reduction at which a column freezes
  MatvecFn low;        // split-precision operator
  cudaStream_t s;
  double *x, *r, *p, *q, *sc;   // N x Bmax each; sc: scalars
  double *part_cd, *part_cu, *part_pd;   // partial sums of the grid reductions
  unsigned int* cnt;                     // their ticket counters (zero between uses)

  static constexpr size_t kParts = 2 * (size_t)CG_MAXT * CG_MAXBX + (size_t)CG_MAXT * CG_MAXPB;
  static size_t bytes(i64 N, int Bmax) {
    return (4 * (size_t)N * Bmax + 16 * 64 + kParts + 64) * sizeof(double) + 4096;
  }

  void bind(void* mem) {
    TTG_REQUIRE(Bmax <= CG_MAXT, "jd cg: block wider than 16 columns");
    double* m = (double*)mem;
    x = m; r = x + N * Bmax; p = r + N * Bmax; q = p + N * Bmax; sc = q + N * Bmax;
    part_cd = sc + 16 * 64;
    part_cu = part_cd + (size_t)CG_MAXT * CG_MAXBX;
    part_pd = part_cu + (size_t)CG_MAXT * CG_MAXBX;
    cnt = (unsigned int*)(part_pd + (size_t)CG_MAXT * CG_MAXPB);   // 3 x 16 counters
    TTG_CUDA(cudaMemsetAsync(cnt, 0, 64 * sizeof(double), s));
  }

  // project out X (N x nb): v -= X (X^T v)
  void project(double* v, int t, const double* X, int nb) {
    double* c = sc + 6 * 64;
    gemm_tn_small(nb, t, N, X, N, v, N, c, nb, 1.0, 0.0, s);
    gemm_nn_small(N, t, nb, X, N, c, nb, v, N, -1.0, 1.0, s);
  }

  // The fixed-length CG solve issues ~12 launches per step and has no host
  // synchronisation, so after its first call for a given (block, shift,
  // Ritz-vector) set of buffers and widths it is captured once into a CUDA
  // graph and replayed: one launch per correction solve instead of ~150.
  bool use_graph = true;
  struct Cached {
    double* T;
    const double* X;
    const double* theta;
    int t, nb;
    cudaGraphExec_t exec;
    long long nlaunch;
  };
  std::vector<Cached> graphs;
  JdCg() = default;
  JdCg(const JdCg&) = delete;
  JdCg& operator=(const JdCg&) = delete;
  ~JdCg() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.exec);
  }

  void operator()(double* T, int t, const double* X, int nb, const double* theta) {
    // the legacy default stream cannot be captured
    if (!use_graph || s == nullptr || s == cudaStreamLegacy) { run(T, t, X, nb, theta); return; }
    for (auto& g : graphs)
      if (g.T == T && g.X == X && g.theta == theta && g.t == t && g.nb == nb) {
        TTG_CUDA(cudaGraphLaunch(g.exec, s));
        g_launches += g.nlaunch;
        return;
      }
    const long long l0 = g_launches;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      use_graph = false;
      run(T, t, X, nb, theta);
      return;
    }
    cudaGraph_t graph = nullptr;
    try {
      run(T, t, X, nb, theta);
    } catch (...) {
      cudaStreamEndCapture(s, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    TTG_CUDA(cudaStreamEndCapture(s, &graph));
    const long long nl = g_launches - l0;
    g_launches -= nl;                     // captured, not yet run
    cudaGraphExec_t exec = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    TTG_CUDA(e);
    graphs.push_back(Cached{T, X, theta, t, nb, exec, nl});
    TTG_CUDA(cudaGraphLaunch(exec, s));
    g_launches += nl;
  }

  void run(double* T, int t, const double* X, int nb, const double* theta) {
    double* rr = sc;
    double* rr_new = sc + 64;
    double* pq = sc + 2 * 64;
    double* rr0 = sc + 3 * 64;
    const double tol2 = rel_tol * rel_tol;
    const size_t bytes_t = sizeof(double) * N * t;
    int bx = (int)std::max<i64>(1, std::min<i64>(CG_MAXBX, (N + 2047) / 2048));
    int eb = (int)std::min<i64>(4096, (N * t + 255) / 256);
    // x = 0, r = -rhs (already orthogonal to X), p = r
    TTG_CUDA(cudaMemsetAsync(x, 0, bytes_t, s));
    TTG_CUDA(cudaMemcpyAsync(r, T, bytes_t, cudaMemcpyDeviceToDevice, s));
    project(r, t, X, nb);
    scale_cols_neg(r, t);
    TTG_CUDA(cudaMemcpyAsync(p, r, bytes_t, cudaMemcpyDeviceToDevice, s));
    col_dots(N, t, r, r, rr, part_cd, cnt, s);
    TTG_CUDA(cudaMemcpyAsync(rr0, rr, sizeof(double) * t, cudaMemcpyDeviceToDevice, s));
    const bool fused = t <= PD_MAXT && nb <= PD_MAXT;
    int pb = (int)std::max<i64>(1, std::min<i64>(CG_MAXPB, (N + 127) / 128));
    for (int it = 0; it < iters; ++it) {
      low(p, q, t);                                   // q = A~ p
      launch_pdl(shift_kernel, dim3(eb), dim3(256), 0, s, N, t, theta, (const double*)p, q, pq,
                 rr_new);                               // q -= theta p
      if (fused) {
        // q = P q with pq = p^T q in the same pass
        double* c = sc + 6 * 64;
        gemm_tn_small(nb, t, N, X, N, q, N, c, nb, 1.0, 0.0, s);
        launch_pdl(proj_dot_kernel, dim3(pb), dim3(128), 0, s, N, t, nb, X, (const double*)c,
                   (const double*)p, q, pq, part_pd, cnt + 2 * CG_MAXT);
      } else {
        project(q, t, X, nb);                         // q = P q
        col_dots(N, t, p, q, pq, part_cd, cnt, s);
      }
      launch_pdl(cg_update_kernel, dim3(bx, t), dim3(256), 0, s, N, (const double*)rr,
                 (const double*)pq, (const double*)rr0, tol2, (const double*)p, (const double*)q, x,
                 r, rr_new, part_cu, cnt + CG_MAXT);
      launch_pdl(cg_dir_kernel, dim3(eb), dim3(256), 0, s, N, t, (const double*)rr,
                 (const double*)rr_new, (const double*)pq, (const double*)rr0, tol2,
                 (const double*)r, p);
      std::swap(rr, rr_new);
    }
    // keep the correction orthogonal to X (rounding of the split products)
    project(x, t, X, nb);
    TTG_CUDA(cudaMemcpyAsync(T, x, bytes_t, cudaMemcpyDeviceToDevice, s));
  }

  void scale_cols_neg(double* v, int t);
};

__global__ void neg_kernel(i64 n, double* v) {
  pdl_trigger();
  pdl_wait();
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x)
    v[e] = -v[e];
}

void JdCg::scale_cols_neg(double* v, int t) {
  int eb = (int)std::min<i64>(4096, (N * t + 255) / 256);
  launch_pdl(neg_kernel, dim3(eb), dim3(256), 0, s, N * t, v);
}

size_t chosen_bytes(i64 N, int B) { return JdCg::bytes(N, B); }

// Chosen local solve: phase A (split Davidson) then phase B (FP64 JD + CG on
// the split operator).  X0, X: N x B.  Returns the FP64-judged statistics.
DavidsonStats chosen_solve(i64 N, int B, void* dav_mem, double* hbuf, void* jd_mem,
                           const MatvecFn& mv64, const MatvecFn& mvlow, const double* X0,
                           double tol, int max_matvecs, double* X, double* theta_host,
                           cudaStream_t s, DavTimer* timer, int* fp64_matvecs) {
  JdCg jd;
  // 16 CG steps per correction.  On the d=20 Heisenberg chain (GB300, the
  // deterministic solver) 8/10/12/16/20/24/32 steps take 1.08/1.23/1.03/
  // 0.98/0.98/0.94/1.01 s: fewer outer iterations and FP64 matvecs balance
  // the longer inner solves, with no clear trend beyond noise of the
  // iteration path; 4-6 steps were 1.3-3.5x slower
  static const int cg_steps = [] {
    const char* v = std::getenv("TTG_JD_CG_STEPS");   // tuning override (default 16)
    const int k = v ? std::atoi(v) : 0;
    return k >= 1 && k <= 256 ? k : 16;
  }();
  jd.N = N; jd.Bmax = B; jd.iters = cg_steps; jd.rel_tol = 1e-3; jd.low = mvlow; jd.s = s;
  jd.use_graph = timer == nullptr;      // the profiler synchronises inside matvecs
  jd.bind(jd_mem);
  const int maxb2 = (int)std::min<i64>(2 * B, N);
  auto jd_prec = [&jd](double* T, int t, const double* Xr, int nb, const double* th) {
    jd(T, t, Xr, nb, th);
  };
  // phase A: Jacobi-Davidson entirely on the split operator (small
  // Rayleigh-Ritz problems of size <= 2B), to the split operator's accuracy
  DavidsonStats a;
  {
    Davidson dav(N, B, maxb2, B, dav_mem, hbuf, s);
    dav.timer = timer;
    dav.gdk = false;
    dav.prec = jd_prec;
    a = dav.solve(mvlow, X0, std::max(tol, 1e-4), 4 * max_matvecs, X, theta_host);
  }
  // phase B: the same iteration with FP64 matvecs as the judge
  Davidson ref(N, B, maxb2, B, dav_mem, hbuf, s);
  ref.timer = timer;
  ref.gdk = false;
  ref.prec = jd_prec;
  DavidsonStats b = ref.solve(mv64, X, tol, max_matvecs, X, theta_host);
  if (fp64_matvecs) *fp64_matvecs = b.matvecs;
  b.matvecs += a.matvecs;
  b.iters += a.iters;
  return b;
}

}  // namespace ttg
