// Dense FP64 linear algebra of the sweep, on the device.
//
//   syev_jacobi   symmetric eigenproblems: the dense local branch
//                 (dsyev, tt_eigb.f90:238) and the Rayleigh-Ritz projection of
//                 the local Davidson solver (dsyev in primme/solve_H_d.c:141).
//                 Cyclic Jacobi, round-robin parallel ordering, one CTA.
//   svd_jacobi    truncation SVD (dgesvd, tt_eigb.f90:312,361;
//                 ttnodeop.f90:254).  One-sided (Hestenes) Jacobi on the
//                 columns, one warp per column pair, all pairs of a round in
//                 parallel, rounds separated by a grid-wide barrier of one
//                 cooperative launch.  High relative accuracy of the small
//                 singular values, which my_chop3 sums.
//   qr_householder  dgeqrf+dorgqr (dqr, matrix_util.f90:37-61) and
//                 zgeqrf+zungqr (zqr, :64-90) with LAPACK's reflector
//                 convention (beta = -sign(alpha)*||x||), so Q and R match the
//                 reference's up to rounding.
#include "ttg_common.cuh"
#include <cooperative_groups.h>
#include <cfloat>
#include <cstdlib>

namespace cg = cooperative_groups;

namespace ttg {

// ---------------------------------------------------------------------------
// small element-wise helpers
// ---------------------------------------------------------------------------
template <class T>
__global__ void transpose_kernel(i64 rows, i64 cols, const T* __restrict__ in, T* __restrict__ out) {
  __shared__ T tile[32][33];
  i64 c0 = (i64)blockIdx.x * 32, r0 = (i64)blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    i64 r = r0 + threadIdx.x, c = c0 + k;
    if (r < rows && c < cols) tile[k][threadIdx.x] = in[r + rows * c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    i64 c = c0 + threadIdx.x, r = r0 + k;
    if (r < rows && c < cols) out[c + cols * r] = tile[threadIdx.x][k];
  }
}

void transpose_f64(i64 rows, i64 cols, const double* in, double* out, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  dim3 grid(ceil_div(cols, 32), ceil_div(rows, 32));
  TTG_REQUIRE(grid.y < 65536, "transpose: too many rows");
  transpose_kernel<double><<<grid, dim3(32, 8), 0, s>>>(rows, cols, in, out);
  TTG_CHECK_LAUNCH();
}
void transpose_z(i64 rows, i64 cols, const double2* in, double2* out, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  dim3 grid(ceil_div(cols, 32), ceil_div(rows, 32));
  TTG_REQUIRE(grid.y < 65536, "transpose: too many rows");
  transpose_kernel<double2><<<grid, dim3(32, 8), 0, s>>>(rows, cols, in, out);
  TTG_CHECK_LAUNCH();
}

__global__ void copy_rows_kernel(i64 rin, i64 rout, i64 cols, const double* in, double* out) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < rout * cols;
       e += (i64)gridDim.x * blockDim.x) {
    i64 r = e % rout, c = e / rout;
    out[e] = in[r + rin * c];
  }
}
void copy_rows_f64(i64 rows_in, i64 rows_out, i64 cols, const double* in, double* out,
                   cudaStream_t s) {
  if (rows_out * cols <= 0) return;
  int blocks = (int)std::min<i64>(4096, (rows_out * cols + 255) / 256);
  copy_rows_kernel<<<blocks, 256, 0, s>>>(rows_in, rows_out, cols, in, out);
  TTG_CHECK_LAUNCH();
}

__global__ void scale_cols_kernel(i64 rows, i64 cols, double* A, i64 lda, const double* sv) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < rows * cols;
       e += (i64)gridDim.x * blockDim.x) {
    i64 r = e % rows, c = e / rows;
    A[r + lda * c] *= sv[c];
  }
}
__global__ void scale_rows_kernel(i64 rows, i64 cols, double* A, i64 lda, const double* sv) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < rows * cols;
       e += (i64)gridDim.x * blockDim.x) {
    i64 r = e % rows, c = e / rows;
    A[r + lda * c] *= sv[r];
  }
}
void scale_cols_f64(i64 rows, i64 cols, double* A, i64 lda, const double* sv, cudaStream_t s) {
  if (rows * cols <= 0) return;
  int blocks = (int)std::min<i64>(4096, (rows * cols + 255) / 256);
  scale_cols_kernel<<<blocks, 256, 0, s>>>(rows, cols, A, lda, sv);
  TTG_CHECK_LAUNCH();
}
void scale_rows_f64(i64 rows, i64 cols, double* A, i64 lda, const double* sv, cudaStream_t s) {
  if (rows * cols <= 0) return;
  int blocks = (int)std::min<i64>(4096, (rows * cols + 255) / 256);
  scale_rows_kernel<<<blocks, 256, 0, s>>>(rows, cols, A, lda, sv);
  TTG_CHECK_LAUNCH();
}

__global__ void fill_kernel(double* p, i64 n, double v) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x)
    p[e] = v;
}
void fill_f64(double* p, i64 n, double v, cudaStream_t s) {
  if (n <= 0) return;
  int blocks = (int)std::min<i64>(4096, (n + 255) / 256);
  fill_kernel<<<blocks, 256, 0, s>>>(p, n, v);
  TTG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// block reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int NT>
__device__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double t = lane < NT / 32 ? red[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) red[32] = t;
  }
  __syncthreads();
  return red[32];
}

// round-robin ("circle") pairing of K (even) players, round r in [0, K-1)
__device__ __forceinline__ void rr_pair(int K, int r, int i, int& a, int& b) {
  if (i == 0) { a = r; b = K - 1; }
  else { a = (r + i) % (K - 1); b = (r - i + K - 1) % (K - 1); }
}

// ---------------------------------------------------------------------------
// symmetric eigensolver: cyclic Jacobi in one CTA
// ---------------------------------------------------------------------------
constexpr int JAC_NT = 1024;
constexpr int JAC_MAX_SWEEPS = 40;

__global__ void __launch_bounds__(JAC_NT) syev_jacobi_kernel(int k, double* Ag, int lda,
                                                             double* w, double* Vg, int ldv,
                                                             int* status, int smem_mode,
                                                             const double* P0, int kp, int ldp) {
  extern __shared__ double dyn[];
  __shared__ double red[33];
  __shared__ double cs[512], sn[512];
  __shared__ int rot_count;
  const int tid = threadIdx.x;
  double* A;
  double* V;
  int la, lv;
  if (smem_mode) {
    A = dyn; V = dyn + (i64)k * k; la = k; lv = k;
    for (int e = tid; e < k * k; e += JAC_NT) A[e] = Ag[(e % k) + (i64)lda * (e / k)];
  } else {
    A = Ag; V = Vg; la = lda; lv = ldv;
  }
  for (int e = tid; e < k * k; e += JAC_NT) V[(e % k) + (i64)lv * (e / k)] = (e % k == e / k) ? 1.0 : 0.0;
  __syncthreads();
  if (smem_mode && P0 && kp > 0) {
    // warm start: V = diag(P0, I), A = V^T A V  (P0: eigenvectors of the
    // leading kp x kp block from the previous call, so A becomes diagonal
    // except for its last k - kp rows and columns)
    double* T = dyn + 2 * (i64)k * k;
    for (int e = tid; e < kp * kp; e += JAC_NT) V[(e % kp) + (i64)lv * (e / kp)] = P0[(e % kp) + (i64)ldp * (e / kp)];
    __syncthreads();
    for (int e = tid; e < k * k; e += JAC_NT) {
      int i = e % k, j = e / k;
      double v;
      if (j < kp) {
        v = 0.0;
        for (int l = 0; l < kp; ++l) v = fma(A[i + (i64)la * l], V[l + (i64)lv * j], v);
      } else {
        v = A[i + (i64)la * j];
      }
      T[e] = v;
    }
    __syncthreads();
    for (int e = tid; e < k * k; e += JAC_NT) {
      int i = e % k, j = e / k;
      double v;
      if (i < kp) {
        v = 0.0;
        for (int l = 0; l < kp; ++l) v = fma(V[l + (i64)lv * i], T[l + (i64)k * j], v);
      } else {
        v = T[e];
      }
      A[i + (i64)la * j] = v;
    }
    __syncthreads();
    for (int e = tid; e < k * k; e += JAC_NT) {
      int i = e % k, j = e / k;
      if (i < j) {
        double v = 0.5 * (A[i + (i64)la * j] + A[j + (i64)la * i]);
        A[i + (i64)la * j] = v;
        A[j + (i64)la * i] = v;
      }
    }
    __syncthreads();
  }
  const int K = (k + 1) & ~1;
  const int npairs = K / 2;
  int sweep = 0;
  double fro2 = 0.0;
  {
    double t = 0.0;
    for (int e = tid; e < k * k; e += JAC_NT) { double v = A[(e % k) + (i64)la * (e / k)]; t += v * v; }
    fro2 = block_sum<JAC_NT>(t, red);
  }
  for (sweep = 0; sweep < JAC_MAX_SWEEPS && k > 1; ++sweep) {
    if (tid == 0) rot_count = 0;
    __syncthreads();
    for (int r = 0; r < K - 1; ++r) {
      // rotation parameters of every pair of this round
      for (int pi = tid; pi < npairs; pi += JAC_NT) {
        int p, q;
        rr_pair(K, r, pi, p, q);
        double c = 1.0, s = 0.0;
        if (p < k && q < k) {
          double app = A[p + (i64)la * p], aqq = A[q + (i64)la * q], apq = A[p + (i64)la * q];
          if (apq != 0.0 && fabs(apq) > 1e-18 * sqrt(fro2) &&
              fabs(apq) > DBL_EPSILON * 0.5 * sqrt(fabs(app) * fabs(aqq))) {
            double theta = (aqq - app) / (2.0 * apq);
            double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            c = 1.0 / sqrt(t * t + 1.0);
            s = t * c;
            atomicAdd(&rot_count, 1);
          }
        }
        cs[pi] = c; sn[pi] = s;
      }
      __syncthreads();
      // rows: A <- J^T A
      for (int e = tid; e < npairs * k; e += JAC_NT) {
        int pi = e / k, j = e % k;
        double c = cs[pi], s = sn[pi];
        if (s == 0.0) continue;
        int p, q;
        rr_pair(K, r, pi, p, q);
        double ap = A[p + (i64)la * j], aq = A[q + (i64)la * j];
        A[p + (i64)la * j] = c * ap - s * aq;
        A[q + (i64)la * j] = s * ap + c * aq;
      }
      __syncthreads();
      // columns: A <- A J, V <- V J
      for (int e = tid; e < npairs * k; e += JAC_NT) {
        int pi = e / k, i = e % k;
        double c = cs[pi], s = sn[pi];
        if (s == 0.0) continue;
        int p, q;
        rr_pair(K, r, pi, p, q);
        double ap = A[i + (i64)la * p], aq = A[i + (i64)la * q];
        A[i + (i64)la * p] = c * ap - s * aq;
        A[i + (i64)la * q] = s * ap + c * aq;
        double vp = V[i + (i64)lv * p], vq = V[i + (i64)lv * q];
        V[i + (i64)lv * p] = c * vp - s * vq;
        V[i + (i64)lv * q] = s * vp + c * vq;
      }
      __syncthreads();
    }
    if (rot_count == 0) break;
    __syncthreads();
  }
  // eigenvalues ascending (stable rank sort), vectors permuted accordingly
  __shared__ int rank_s[512];
  double* wtmp = cs;   // k <= 512
  for (int i = tid; i < k; i += JAC_NT) wtmp[i] = A[i + (i64)la * i];
  __syncthreads();
  // when V is the output buffer itself, stash it in A's storage first
  double* Vsrc = V;
  int lsrc = lv;
  if (!smem_mode) {
    for (int e = tid; e < k * k; e += JAC_NT)
      A[(e % k) + (i64)la * (e / k)] = V[(e % k) + (i64)lv * (e / k)];
    Vsrc = A; lsrc = la;
  }
  for (int i = tid; i < k; i += JAC_NT) {
    double wi = wtmp[i];
    int rk = 0;
    for (int j = 0; j < k; ++j) {
      double wj = wtmp[j];
      rk += (wj < wi) || (wj == wi && j < i);
    }
    rank_s[i] = rk;
  }
  __syncthreads();
  for (int e = tid; e < k * k; e += JAC_NT) {
    int i = e % k, j = e / k;
    Vg[i + (i64)ldv * rank_s[j]] = Vsrc[i + (i64)lsrc * j];
  }
  for (int i = tid; i < k; i += JAC_NT) w[rank_s[i]] = wtmp[i];
  if (tid == 0 && status) *status = sweep;
}

void syev_jacobi(int k, double* A, int lda, double* w, double* V, int ldv, int* status,
                 cudaStream_t s, const double* P0, int kp, int ldp) {
  if (k <= 0) return;
  TTG_REQUIRE(k <= 512, "syev_jacobi: k > 512");
  const bool warm = P0 && kp > 0 && (size_t)3 * k * k * sizeof(double) <= 200 * 1024;
  size_t smem = (size_t)(warm ? 3 : 2) * k * k * sizeof(double);
  int mode = smem <= 200 * 1024 ? 1 : 0;
  if (mode) {
    // thread-safe one-time set-up (C++ static initialisation)
    static const cudaError_t attr_rc = cudaFuncSetAttribute(
        syev_jacobi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    TTG_CUDA(attr_rc);
  } else {
    smem = 0;
  }
  syev_jacobi_kernel<<<1, JAC_NT, smem, s>>>(k, A, lda, w, V, ldv, status, mode,
                                             warm ? P0 : nullptr, warm ? kp : 0, ldp);
  TTG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// one-sided Jacobi SVD (cooperative launch, grid barrier between rounds)
// ---------------------------------------------------------------------------
#ifndef TTG_SVD_CT
#define TTG_SVD_CT 128
#endif
// one CTA per column pair; its warps share the rows (measured on GB300, 128
// threads: 7.6 ms at 320x128 and 54 ms at 2048x512; 64: 8.3 and 60; 32: 9.2
// and 81)
constexpr int SVD_CT = TTG_SVD_CT;
constexpr int SVD_MAX_SWEEPS = 60;

template <class T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One-sided Jacobi sweeps over the column pairs of M (p x q), rotations
// accumulated in V (q x q).  Cooperative launch: a round of disjoint pairs
// (round-robin ordering) per grid barrier, one CTA per pair whose four warps
// split the rows (so all four FP64 pipes of an SM work on it).  T = float
// gives the cheap pre-sweeps of large matrices, T = double the polish.
template <class T>
__global__ void __launch_bounds__(SVD_CT) svd_sweep_kernel(int p, int q, T* M, T* V,
                                                           int* counters, int* status, int init_v,
                                                           T tol, T tol_count, int max_sweeps) {
  cg::grid_group grid = cg::this_grid();
  __shared__ T red[3][SVD_CT / 32];
  __shared__ T csn[2];
  __shared__ int act;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int K = (q + 1) & ~1;
  const int npairs = K / 2;
  // V = I, unless the pre-sweeps already supplied the rotation
  if (!init_v)
    for (i64 e = blockIdx.x * (i64)SVD_CT + tid; e < (i64)q * q; e += (i64)gridDim.x * SVD_CT)
      V[e] = (e % q == e / q) ? T(1) : T(0);
  if (blockIdx.x == 0 && tid == 0) { counters[0] = 0; counters[1] = 0; }
  grid.sync();
  int sweep = 0;
  for (sweep = 0; sweep < max_sweeps; ++sweep) {
    int* cnt = counters + (sweep & 1);
    for (int r = 0; r < K - 1; ++r) {
      for (int pi = blockIdx.x; pi < npairs; pi += gridDim.x) {
        int a, b;
        rr_pair(K, r, pi, a, b);
        if (a >= q || b >= q) continue;
        T* ca = M + (i64)p * a;
        T* cb = M + (i64)p * b;
        T al = 0, be = 0, ga = 0;
        for (int i = tid; i < p; i += SVD_CT) {
          const T x = ca[i], y = cb[i];
          al = fma(x, x, al); be = fma(y, y, be); ga = fma(x, y, ga);
        }
        al = warp_sum_t(al); be = warp_sum_t(be); ga = warp_sum_t(ga);
        if (lane == 0) { red[0][warp] = al; red[1][warp] = be; red[2][warp] = ga; }
        __syncthreads();
        if (tid == 0) {
          T A = 0, Bv = 0, G = 0;
          for (int w = 0; w < SVD_CT / 32; ++w) { A += red[0][w]; Bv += red[1][w]; G += red[2][w]; }
          // |G| > tol sqrt(A Bv), compared in squares (no square root)
          const T g2 = G * G, ab = A * Bv;
          int go = (G != T(0)) && (g2 > tol * tol * ab);
          if (go) {
            // The angle is taken in FP32 (GB300 runs FP64 square roots and
            // divides as long dependent chains on a narrow pipe, and this is
            // the serial part of every round); c and s are formed in T from
            // that t, c = 1/sqrt(1 + t^2), s = c t, so the rotation is
            // orthogonal to T's precision whatever t is.  A t off by FP32
            // rounding leaves an off-diagonal ~1e-7 of G, which the next
            // sweep removes like any other; the stopping test is unchanged.
            const T zeta_t = (Bv - A) / (T(2) * G);
            const float z = (float)zeta_t, az = fabsf(z);
            // |zeta| beyond FP32's comfortable range: t = 1/(2 zeta) in T
            const T t = az < 1e18f ? (T)copysignf(1.f / (az + sqrtf(1.f + z * z)), z)
                                   : T(0.5) / zeta_t;
            const T c = rsqrt(T(1) + t * t);
            csn[0] = c;
            csn[1] = c * t;
            // rotations whose cosine is within the rounding noise of a dot
            // product of length p are applied but do not keep the sweeps going
            if (g2 > tol_count * tol_count * ab) atomicAdd(cnt, 1);
          }
          act = go;
        }
        __syncthreads();
        if (act) {
          const T c = csn[0], sn = csn[1];
          for (int i = tid; i < p; i += SVD_CT) {
            const T x = ca[i], y = cb[i];
            ca[i] = c * x - sn * y;
            cb[i] = sn * x + c * y;
          }
          T* va = V + (i64)q * a;
          T* vb = V + (i64)q * b;
          for (int i = tid; i < q; i += SVD_CT) {
            const T x = va[i], y = vb[i];
            va[i] = c * x - sn * y;
            vb[i] = sn * x + c * y;
          }
        }
        __syncthreads();
      }
      grid.sync();
    }
    int done = (*((volatile int*)cnt) == 0);
    grid.sync();
    if (blockIdx.x == 0 && tid == 0) counters[(sweep + 1) & 1] = 0;
    grid.sync();
    if (done) break;
  }
  if (blockIdx.x == 0 && tid == 0 && status) *status = sweep;
}

__global__ void d2f_kernel(i64 n, const double* __restrict__ a, float* __restrict__ b) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x)
    b[e] = (float)a[e];
}
__global__ void f2d_kernel(i64 n, const float* __restrict__ a, double* __restrict__ b) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x)
    b[e] = (double)a[e];
}

template <class T>
static int svd_coop_blocks() {
  static const int max_coop = [] {
    int dev = 0, nsm = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, svd_sweep_kernel<T>, SVD_CT, 0) !=
            cudaSuccess)
      return 0;
    return nsm * per;
  }();
  TTG_REQUIRE(max_coop > 0, "svd: occupancy query failed");
  return max_coop;
}

template <class T>
static void svd_sweeps(int p, int q, T* M, T* V, int* counters, int* status, int init_v, T tol,
                       T tol_count, int max_sweeps, cudaStream_t s) {
  int blocks = std::max(1, std::min((q + 1) / 2, svd_coop_blocks<T>()));
  void* args[] = {&p, &q, &M, &V, &counters, &status, &init_v, &tol, &tol_count, &max_sweeps};
  TTG_CUDA(cudaLaunchCooperativeKernel((void*)svd_sweep_kernel<T>, dim3(blocks), dim3(SVD_CT),
                                       args, 0, s));
  ++g_launches;
}

// FP32 pre-sweeps of the one-sided Jacobi SVD, one CTA with M (p x q) and the
// accumulated rotation V (q x q) in shared memory.  FP32 runs at 64 times
// the FP64 rate of a GB300 SM, so the sweeps that take the columns from
// arbitrary to nearly orthogonal are cheap here; the FP64 sweeps that follow
// (svd_rotate_kernel, started from V) only polish.  V is written as FP64.
constexpr int SVD32_NT = 1024;
constexpr int SVD32_MAX_SWEEPS = 20;
constexpr size_t SVD32_SMEM = 227 * 1024 - 1024;

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(SVD32_NT) svd_pre32_kernel(int p, int q, const double* __restrict__ M,
                                                             double* __restrict__ Vout, int* status) {
  extern __shared__ float sm32[];
  float* A = sm32;                       // p x q
  float* W = sm32 + (size_t)p * q;       // q x q
  __shared__ int rot;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = SVD32_NT >> 5;
  for (int e = tid; e < p * q; e += SVD32_NT) A[e] = (float)M[e];
  for (int e = tid; e < q * q; e += SVD32_NT) W[e] = (e % q == e / q) ? 1.f : 0.f;
  const int K = (q + 1) & ~1;
  const int npairs = K / 2;
  const float tol = sqrtf((float)p) * FLT_EPSILON;
  int sweep = 0;
  for (sweep = 0; sweep < SVD32_MAX_SWEEPS; ++sweep) {
    if (tid == 0) rot = 0;
    __syncthreads();
    for (int r = 0; r < K - 1; ++r) {
      for (int pi = warp; pi < npairs; pi += nwarp) {
        int a, b;
        rr_pair(K, r, pi, a, b);
        if (a >= q || b >= q) continue;
        float* ca = A + (size_t)p * a;
        float* cb = A + (size_t)p * b;
        float al = 0.f, be = 0.f, ga = 0.f;
        for (int i = lane; i < p; i += 32) {
          const float x = ca[i], y = cb[i];
          al = fmaf(x, x, al); be = fmaf(y, y, be); ga = fmaf(x, y, ga);
        }
        al = warp_sumf(al); be = warp_sumf(be); ga = warp_sumf(ga);
        if (ga == 0.f || !(fabsf(ga) > tol * sqrtf(al * be))) continue;
        const float zeta = (be - al) / (2.f * ga);
        const float t = (zeta >= 0.f ? 1.f : -1.f) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
        const float c = 1.f / sqrtf(1.f + t * t);
        const float sn = c * t;
        for (int i = lane; i < p; i += 32) {
          const float x = ca[i], y = cb[i];
          ca[i] = c * x - sn * y;
          cb[i] = sn * x + c * y;
        }
        float* wa = W + (size_t)q * a;
        float* wb = W + (size_t)q * b;
        for (int i = lane; i < q; i += 32) {
          const float x = wa[i], y = wb[i];
          wa[i] = c * x - sn * y;
          wb[i] = sn * x + c * y;
        }
        if (lane == 0) atomicAdd(&rot, 1);
      }
      __syncthreads();
    }
    const int done = rot == 0;
    __syncthreads();
    if (done) break;
  }
  for (int e = tid; e < q * q; e += SVD32_NT) Vout[e] = (double)W[e];
  if (tid == 0 && status) *status = sweep;
}

// Z = 1.5 I - 0.5 Y (one Newton-Schulz step toward the orthogonal factor)
__global__ void ns_coef_kernel(int q, const double* __restrict__ Y, double* __restrict__ Z) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < q * q; e += gridDim.x * blockDim.x)
    Z[e] = (e % q == e / q ? 1.5 : 0.0) - 0.5 * Y[e];
}

// sigma_j = ||M_j||, rank sort descending, write U (normalised), sigma, Vt
__global__ void svd_finish_kernel(int p, int q, const double* M, const double* V, double* U,
                                  double* sigma, double* Vt, double* nrm, int* rank) {
  // phase 1 (all blocks): column norms, one warp per column
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int j = gw; j < q; j += nw) {
    double s = 0.0;
    for (int i = lane; i < p; i += 32) { double x = M[i + (i64)p * j]; s = fma(x, x, s); }
    s = warp_sum(s);
    if (lane == 0) nrm[j] = sqrt(s);
  }
}

__global__ void svd_rank_kernel(int q, const double* nrm, int* rank) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < q; j += gridDim.x * blockDim.x) {
    double v = nrm[j];
    int rk = 0;
    for (int t = 0; t < q; ++t) rk += (nrm[t] > v) || (nrm[t] == v && t < j);
    rank[j] = rk;
  }
}

__global__ void svd_gather_kernel(int p, int q, const double* M, const double* V,
                                  const double* nrm, const int* rank, double* U,
                                  double* sigma, double* Vt) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)p * q;
       e += (i64)gridDim.x * blockDim.x) {
    int i = (int)(e % p), j = (int)(e / p);
    double s = nrm[j];
    U[i + (i64)p * rank[j]] = s > 0 ? M[e] / s : (i == j ? 1.0 : 0.0);
  }
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)q * q;
       e += (i64)gridDim.x * blockDim.x) {
    int i = (int)(e % q), j = (int)(e / q);
    // Vt row rank[j] = V column j
    Vt[rank[j] + (i64)q * i] = V[e];
  }
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < q; j += gridDim.x * blockDim.x)
    sigma[rank[j]] = nrm[j];
}

// ---------------------------------------------------------------------------
// QR-preconditioned one-sided Jacobi (Drmac and Veselic, "New fast and
// accurate Jacobi SVD algorithm", SIAM J. Matrix Anal. Appl. 29, 2008).
// Plain one-sided Jacobi on the truncation blocks of the sweeps, whose
// singular values fall over fifteen decades, needs 25-35 sweeps; on the
// transposed triangular factor of a QR of the column-sorted matrix it needs
// 6-8.  So for M (p x q, p >= q):
//   M P = Q R   (columns sorted by decreasing norm, blocked Householder QR:
//                one-CTA panels of QRP_NB columns, trailing update by FP64
//                GEMMs over the whole GPU with the compact WY form)
//   R^T = Ux S J^T   (one-sided Jacobi on the q x q matrix R^T)
//   M = (Q J) S (P Ux)^T.
// ---------------------------------------------------------------------------
constexpr int QRP_NB = 32;
constexpr int QRP_NT = 1024;

// Householder QR of one panel in place: rows 0..m-1 from the panel's
// diagonal down, columns 0..w-1 (leading dimension lda).  R goes above the
// diagonal, the reflector vectors below it (unit diagonal implied), tau[c];
// T (w x w, leading dimension ldt) is the triangular factor of the block
// reflector H_0 H_1 ... H_{w-1} = I - Y T Y^T (forward, columnwise).
__global__ void __launch_bounds__(QRP_NT) qr_panel_kernel(int m, int w, double* A, i64 lda,
                                                          double* tau, double* T, int ldt) {
  __shared__ double red[33];
  __shared__ double s_beta, s_tau, s_scale;
  __shared__ double zt[QRP_NB];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nwarp = QRP_NT / 32;
  for (int c = 0; c < w; ++c) {
    double* col = A + lda * c;
    double t = 0.0;
    for (int i = c + 1 + tid; i < m; i += QRP_NT) t = fma(col[i], col[i], t);
    const double xn2 = block_sum<QRP_NT>(t, red);
    if (tid == 0) {
      const double alpha = col[c];
      if (xn2 == 0.0) {
        s_tau = 0.0; s_beta = alpha; s_scale = 0.0;
      } else {
        const double beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
        s_tau = (beta - alpha) / beta;
        s_beta = beta;
        s_scale = 1.0 / (alpha - beta);
      }
      tau[c] = s_tau;
    }
    __syncthreads();
    const double tc = s_tau, sc = s_scale;
    if (tc != 0.0)
      for (int i = c + 1 + tid; i < m; i += QRP_NT) col[i] *= sc;
    __syncthreads();
    if (tid == 0) col[c] = s_beta;
    __syncthreads();
    // H_c = I - tau v v^T on columns c+1..w-1, one warp per column
    if (tc != 0.0) {
      for (int cc = c + 1 + wid; cc < w; cc += nwarp) {
        double* a = A + lda * cc;
        double d = lane == 0 ? a[c] : 0.0;
        for (int i = c + 1 + lane; i < m; i += 32) d = fma(col[i], a[i], d);
        d = warp_sum(d) * tc;
        if (lane == 0) a[c] -= d;
        for (int i = c + 1 + lane; i < m; i += 32) a[i] = fma(-d, col[i], a[i]);
      }
    }
    __syncthreads();
  }
  // T: T[i, i] = tau_i, T[0:i, i] = -tau_i T[0:i, 0:i] (Y[:, 0:i]^T y_i)
  for (int e = tid; e < ldt * w; e += QRP_NT) T[e] = 0.0;
  __syncthreads();
  for (int i = 0; i < w; ++i) {
    for (int j = wid; j < i; j += nwarp) {
      const double* yj = A + lda * j;
      const double* yi = A + lda * i;
      double z = lane == 0 ? yj[i] : 0.0;          // y_i(i) = 1
      for (int r = i + 1 + lane; r < m; r += 32) z = fma(yj[r], yi[r], z);
      z = warp_sum(z);
      if (lane == 0) zt[j] = -tau[i] * z;
    }
    __syncthreads();
    if (tid < i) {
      double v = 0.0;
      for (int k = tid; k < i; ++k) v = fma(T[tid + (i64)ldt * k], zt[k], v);
      T[tid + (i64)ldt * i] = v;
    }
    if (tid == 0) T[i + (i64)ldt * i] = tau[i];
    __syncthreads();
  }
}

// The same panel factorization spread over a cooperative grid for tall
// panels (one CTA holds FP64 at two FMAs per clock, so a 2048 x 32 panel is
// FP64-bound on it): CTA b owns rows [b*chunk, (b+1)*chunk).  Per column,
// the partial sums of squares and then the partial dot products with the
// later columns go to per-column slots of part; after each grid barrier every
// CTA adds the G partials in the same order, so all compute the same
// reflector.  T comes from the panel's Gram matrix Y^T Y (partial sums per
// CTA, added by CTA 0, which then runs the recurrence).
constexpr int QRC_NT = 256;
constexpr int QRC_GMAX = 32;
__global__ void __launch_bounds__(QRC_NT) qr_panel_coop_kernel(int m, int w, double* A, i64 lda,
                                                               double* tau, double* T, int ldt,
                                                               double* part) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double red[33];
  __shared__ double zt[QRP_NB];
  __shared__ double gram[QRP_NB * QRP_NB];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nwarp = QRC_NT / 32;
  const int G = gridDim.x, b = blockIdx.x;
  const int chunk = (m + G - 1) / G;
  const int lo = min(m, b * chunk), hi = min(m, lo + chunk);
  double* pn = part;                                 // [w][G]: sums of squares
  double* pd = part + (size_t)QRP_NB * QRC_GMAX;     // [w][G][w]: dots
  double* pg = pd + (size_t)QRP_NB * QRC_GMAX * QRP_NB;   // [G][w*w]: Gram
  // partial sums of squares of column c below row c over the own rows
  auto norm_part = [&](int c) {
    const double* col = A + lda * c;
    double t = 0.0;
    for (int i = max(lo, c + 1) + tid; i < hi; i += QRC_NT) t = fma(col[i], col[i], t);
    t = block_sum<QRC_NT>(t, red);
    if (tid == 0) pn[(size_t)c * QRC_GMAX + b] = t;
  };
  norm_part(0);
  for (int c = 0; c < w; ++c) {
    double* col = A + lda * c;
    grid.sync();   // column c final below the diagonal, its norm partials written
    // row c may belong to another CTA: read it from L2 (this CTA's L1 may hold
    // the line from a neighbouring own row); its owner overwrites it only
    // after the next barrier
    const double alpha = __ldcg(col + c);
    double xn2 = 0.0;
    for (int q = 0; q < G; ++q) xn2 += __ldcg(pn + (size_t)c * QRC_GMAX + q);
    double tc = 0.0, sc = 0.0, beta = alpha;
    if (xn2 != 0.0) {
      beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
      tc = (beta - alpha) / beta;
      sc = 1.0 / (alpha - beta);
    }
    if (b == 0 && tid == 0) tau[c] = tc;
    if (tc != 0.0)
      for (int i = max(lo, c + 1) + tid; i < hi; i += QRC_NT) col[i] *= sc;
    __syncthreads();
    // partial dots v^T a_cc over the own rows (the owner of row c adds a_cc(c))
    for (int cc = c + 1 + wid; cc < w; cc += nwarp) {
      const double* a = A + lda * cc;
      double d = (lane == 0 && c >= lo && c < hi) ? a[c] : 0.0;
      for (int i = max(lo, c + 1) + lane; i < hi; i += 32) d = fma(col[i], a[i], d);
      d = warp_sum(d);
      if (lane == 0) pd[((size_t)c * QRC_GMAX + b) * QRP_NB + cc] = d;
    }
    grid.sync();   // dots complete; every CTA has read alpha
    if (c >= lo && c < hi && tid == 0) col[c] = beta;
    if (tc != 0.0) {
      for (int cc = c + 1 + wid; cc < w; cc += nwarp) {
        double d = 0.0;
        for (int q = 0; q < G; ++q) d += __ldcg(pd + ((size_t)c * QRC_GMAX + q) * QRP_NB + cc);
        d *= tc;
        double* a = A + lda * cc;
        if (lane == 0 && c >= lo && c < hi) a[c] -= d;
        for (int i = max(lo, c + 1) + lane; i < hi; i += 32) a[i] = fma(-d, col[i], a[i]);
      }
    }
    __syncthreads();
    if (c + 1 < w) norm_part(c + 1);
  }
  // Gram of Y (unit diagonal, zeros above) over the own rows
  for (int e = tid; e < w * w; e += QRC_NT) {
    const int i = e % w, j = e / w;
    double g = 0.0;
    if (i <= j) {
      for (int r = max(lo, j); r < hi; ++r) {
        const double yi = r == i ? 1.0 : (r > i ? A[r + lda * i] : 0.0);
        const double yj = r == j ? 1.0 : A[r + lda * j];
        g = fma(yi, yj, g);
      }
    }
    pg[(size_t)b * QRP_NB * QRP_NB + e] = g;
  }
  grid.sync();
  if (b != 0) return;
  for (int e = tid; e < w * w; e += QRC_NT) {
    double g = 0.0;
    for (int q = 0; q < G; ++q) g += __ldcg(pg + (size_t)q * QRP_NB * QRP_NB + e);
    gram[e] = g;
  }
  for (int e = tid; e < ldt * w; e += QRC_NT) T[e] = 0.0;
  __syncthreads();
  // T[0:i, i] = -tau_i T[0:i, 0:i] (Y[:, 0:i]^T y_i), Y^T y_i = gram[0:i, i]
  for (int i = 0; i < w; ++i) {
    if (tid < i) zt[tid] = -tau[i] * gram[tid + w * i];
    __syncthreads();
    if (tid < i) {
      double v = 0.0;
      for (int k = tid; k < i; ++k) v = fma(T[tid + (i64)ldt * k], zt[k], v);
      T[tid + (i64)ldt * i] = v;
    }
    if (tid == 0) T[i + (i64)ldt * i] = tau[i];
    __syncthreads();
  }
}

// Y (m x w) with the unit diagonal and zeros above it, from a factored panel
__global__ void qr_make_y_kernel(int m, int w, const double* __restrict__ A, i64 lda,
                                 double* __restrict__ Y) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)m * w; e += (i64)gridDim.x * blockDim.x) {
    const int r = (int)(e % m), c = (int)(e / m);
    Y[e] = r > c ? A[r + lda * c] : (r == c ? 1.0 : 0.0);
  }
}
// A[:, rank[j]] = M[:, j]
__global__ void permute_cols_kernel(int p, int q, const double* __restrict__ M,
                                    const int* __restrict__ rank, double* __restrict__ A) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)p * q; e += (i64)gridDim.x * blockDim.x) {
    const int i = (int)(e % p), j = (int)(e / p);
    A[i + (i64)p * rank[j]] = M[e];
  }
}
// X (q x q) = R^T, R the upper triangle of A's leading q x q block
__global__ void rt_kernel(int q, const double* __restrict__ A, i64 lda, double* __restrict__ X) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)q * q; e += (i64)gridDim.x * blockDim.x) {
    const int i = (int)(e % q), j = (int)(e / q);
    X[e] = j <= i ? A[j + lda * i] : 0.0;
  }
}
// C (p x q) = [Vtx^T; 0]
__global__ void qr_c0n_kernel(int p, int q, const double* __restrict__ Ux, double* __restrict__ C) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)p * q; e += (i64)gridDim.x * blockDim.x) {
    const int i = (int)(e % p), k = (int)(e / p);
    C[e] = i < q ? Ux[i + (i64)q * k] : 0.0;
  }
}
__global__ void qr_vt_kernel(int q, const double* __restrict__ Ux, const int* __restrict__ perm,
                             double* __restrict__ Vt) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)q * q; e += (i64)gridDim.x * blockDim.x) {
    const int k = (int)(e % q), j = (int)(e / q);
    Vt[e] = Ux[perm[j] + (i64)q * k];
  }
}

// doubles of the QR-preconditioned path's own workspace
static size_t svd_qr_work(size_t p, size_t q) {
  const size_t npan = (q + QRP_NB - 1) / QRP_NB;
  const size_t coop = QRP_NB * QRC_GMAX + QRP_NB * QRC_GMAX * QRP_NB + QRC_GMAX * QRP_NB * QRP_NB;
  // first QR (A, X, Ux, Vtx, Tf, Yp, G1, G2, tau, perm, coop partials), then
  // the second QR's R2^T, Q2 V2, T factors and tau
  return p * q + 3 * q * q + npan * QRP_NB * QRP_NB + p * QRP_NB + 2 * QRP_NB * q + 2 * q + 256 +
         coop + 64 + 2 * q * q + npan * QRP_NB * QRP_NB + q + 64;
}

size_t svd_scratch(int p, int q) {
  // working copy of M (max(p,q) x min(p,q)), V (min^2), norms, ranks, counters, Ut,
  // for the FP32 pre-sweeps two min^2 and one max x min temporaries, and the
  // workspace of the QR-preconditioned path
  size_t pp = std::max(p, q), qq = std::min(p, q);
  return (pp * qq + qq * qq + 2 * qq + 64) * sizeof(double) + pp * qq * sizeof(double) +
         (2 * qq * qq + pp * qq) * sizeof(double) + svd_qr_work(pp, qq) * sizeof(double);
}

static inline int gbl(i64 n) { return (int)std::max<i64>(1, std::min<i64>(4096, (n + 255) / 256)); }

static void svd_tall(int p, int q, double* Mw, double* U, double* sigma, double* Vt,
                     double* V, double* nrm, int* rank, int* counters, int* status,
                     double* tmp, cudaStream_t s, double* qrwork = nullptr);

// The QR-preconditioned path (q >= SVD_QR_MIN_Q):
//   M P = Q1 R1        columns sorted by norm, blocked Householder QR
//   R1^T = Q2 R2       for q >= SVD_QR2_MIN_Q a second QR, of R1^T
//   R2^T = U2 S V2^T   one-sided Jacobi on R2^T (rotations accumulated in V2)
// so M = (Q1 U2) S (P Q2 V2)^T; without the second QR (Q2 = I, R2 = R1)
// the Jacobi runs on R1^T itself and M = (Q1 V2') S (P U2')^T with the roles
// of the factors exchanged.  The second QR leaves R2^T closer to orthogonal
// columns: on graded blocks (singular values 1 to 1e-13) the sweeps drop
// from 9-10 to about 6; measured on GB300 that pays from q ~ 200 (2048 x 512:
// 59.2 -> 53.8 ms) but not at q = 128 (320 x 128: 7.6 -> 7.3 ms, and the
// d=20 solve, whose blocks are mostly narrower, slower by its ~30 extra
// launches per SVD).
constexpr int SVD_QR2_MIN_Q = 192;

static void svd_tall_qr(int p, int q, double* Mw, double* U, double* sigma, double* Vt,
                        double* V, double* nrm, int* rank, int* counters, int* status,
                        double* tmp, double* work, cudaStream_t s) {
  const int npan = ceil_div(q, QRP_NB);
  double* A = work;                                     // p x q
  double* X = A + (size_t)p * q;                        // q x q: R1^T, then its QR
  double* Ux = X + (size_t)q * q;                       // q x q
  double* Vtx = Ux + (size_t)q * q;                     // q x q
  double* Tf = Vtx + (size_t)q * q;                     // NB x NB per panel (first QR)
  double* Yp = Tf + (size_t)npan * QRP_NB * QRP_NB;     // p x NB
  double* G1 = Yp + (size_t)p * QRP_NB;                 // NB x q
  double* G2 = G1 + (size_t)QRP_NB * q;                 // NB x q
  double* tau = G2 + (size_t)QRP_NB * q;                // q
  int* perm = (int*)(tau + q);                          // q ints
  double* qpart = tau + 2 * (size_t)q + 64;             // cooperative panel partials
  const size_t coop = (size_t)QRP_NB * QRC_GMAX + (size_t)QRP_NB * QRC_GMAX * QRP_NB +
                      (size_t)QRC_GMAX * QRP_NB * QRP_NB;
  double* X2 = qpart + coop;                            // q x q: R2^T, Jacobi
  double* W = X2 + (size_t)q * q;                       // q x q: Q2 V2
  double* Tf2 = W + (size_t)q * q;                      // NB x NB per panel (second QR)
  double* tau2 = Tf2 + (size_t)npan * QRP_NB * QRP_NB;  // q
  auto gemm = [&](int M, int N, int K, const double* Am, i64 sAm, i64 sAk, const double* Bm,
                  i64 sBk, i64 sBn, double* C, i64 sCm, i64 sCn, double alpha, double beta) {
    GemmF64 g;
    g.M = M; g.N = N; g.K = K;
    g.A = Am; g.sAm = sAm; g.sAk = sAk;
    g.B = Bm; g.sBk = sBk; g.sBn = sBn;
    g.C = C; g.sCm = sCm; g.sCn = sCn;
    g.alpha = alpha; g.beta = beta;
    gemm_f64(g, s);
  };
  // blocked Householder QR of F (rows x q, leading dimension rows) in place:
  // reflectors below the diagonal, R on and above it, panel T factors in Tk
  auto qr_factor = [&](int rows, double* F, double* Tfac, double* tv) {
    for (int k = 0; k < npan; ++k) {
      const int j0 = k * QRP_NB, w = std::min(QRP_NB, q - j0), m = rows - j0;
      double* Ap = F + j0 + (i64)rows * j0;
      double* Tk = Tfac + (size_t)k * QRP_NB * QRP_NB;
      // panels of 1024+ rows on a grid of CTAs (rows split, two grid
      // barriers per column); narrower ones in one CTA (grids from 256 rows,
      // one CTA per 32 or 64 rows, measured no faster on GB300: 7.8 against
      // 7.55 ms for the 320 x 128 truncation)
      if (m >= 1024) {
        static const int coop_max = [] {
          int dev = 0, nsm = 0, per = 0;
          cudaGetDevice(&dev);
          cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, qr_panel_coop_kernel, QRC_NT, 0);
          return std::max(1, nsm * per);
        }();
        int G = std::min(std::min(QRC_GMAX, std::max(1, m / 128)), coop_max);
        int mm = m, ww = w, ldt = QRP_NB;
        i64 ld = rows;
        double* tk = tv + j0;
        void* args[] = {&mm, &ww, &Ap, &ld, &tk, &Tk, &ldt, &qpart};
        TTG_CUDA(cudaLaunchCooperativeKernel((const void*)qr_panel_coop_kernel, dim3(G),
                                             dim3(QRC_NT), args, 0, s));
        ++g_launches;
      } else {
        qr_panel_kernel<<<1, QRP_NT, 0, s>>>(m, w, Ap, rows, tv + j0, Tk, QRP_NB);
        TTG_CHECK_LAUNCH();
      }
      const int n2 = q - j0 - w;
      if (n2 > 0) {
        qr_make_y_kernel<<<gbl((i64)m * w), 256, 0, s>>>(m, w, Ap, rows, Yp);
        TTG_CHECK_LAUNCH();
        double* A2 = Ap + (i64)rows * w;
        gemm(w, n2, m, Yp, m, 1, A2, 1, rows, G1, 1, w, 1.0, 0.0);     // G1 = Y^T A2
        gemm(w, n2, w, Tk, QRP_NB, 1, G1, 1, w, G2, 1, w, 1.0, 0.0);   // G2 = T^T G1
        gemm(m, n2, w, Yp, 1, m, G2, 1, w, A2, 1, rows, -1.0, 1.0);    // A2 -= Y G2
      }
    }
  };
  // C (rows x q, leading dimension rows) = Q C, Q the product of F's block
  // reflectors, applied in reverse order
  auto qr_apply = [&](int rows, const double* F, const double* Tfac, double* C) {
    for (int k = npan - 1; k >= 0; --k) {
      const int j0 = k * QRP_NB, w = std::min(QRP_NB, q - j0), m = rows - j0;
      const double* Ap = F + j0 + (i64)rows * j0;
      const double* Tk = Tfac + (size_t)k * QRP_NB * QRP_NB;
      qr_make_y_kernel<<<gbl((i64)m * w), 256, 0, s>>>(m, w, Ap, rows, Yp);
      TTG_CHECK_LAUNCH();
      double* Cs = C + j0;
      gemm(w, q, m, Yp, m, 1, Cs, 1, rows, G1, 1, w, 1.0, 0.0);        // G1 = Y^T C
      gemm(w, q, w, Tk, 1, QRP_NB, G1, 1, w, G2, 1, w, 1.0, 0.0);      // G2 = T G1
      gemm(m, q, w, Yp, 1, m, G2, 1, w, Cs, 1, rows, -1.0, 1.0);      // C -= Y G2
    }
  };
  // column norms, descending order (ties by index), permuted copy
  int nb = std::max(1, std::min(1024, ceil_div((i64)q * 32, 256)));
  svd_finish_kernel<<<nb, 256, 0, s>>>(p, q, Mw, nullptr, nullptr, nullptr, nullptr, nrm, perm);
  TTG_CHECK_LAUNCH();
  svd_rank_kernel<<<ceil_div(q, 256), 256, 0, s>>>(q, nrm, perm);
  TTG_CHECK_LAUNCH();
  permute_cols_kernel<<<gbl((i64)p * q), 256, 0, s>>>(p, q, Mw, perm, A);
  TTG_CHECK_LAUNCH();
  qr_factor(p, A, Tf, tau);                             // M P = Q1 R1
  (void)tmp;
  const bool qr2 = q >= SVD_QR2_MIN_Q;
  if (qr2) {
    rt_kernel<<<gbl((i64)q * q), 256, 0, s>>>(q, A, p, X);   // X = R1^T
    TTG_CHECK_LAUNCH();
    qr_factor(q, X, Tf2, tau2);                                // R1^T = Q2 R2
    rt_kernel<<<gbl((i64)q * q), 256, 0, s>>>(q, X, q, X2);  // X2 = R2^T
  } else {
    rt_kernel<<<gbl((i64)q * q), 256, 0, s>>>(q, A, p, X2);  // X2 = R1^T
  }
  TTG_CHECK_LAUNCH();
  // one-sided Jacobi on R2^T, FP64 sweeps over the grid from the identity
  // (FP32 pre-sweeps do not pay here: the preconditioned matrix converges in
  // a few FP64 sweeps, and FP32 cannot resolve its small columns)
  svd_sweeps<double>(q, q, X2, V, counters, status, 0, sqrt((double)q) * DBL_EPSILON,
                     (double)q * DBL_EPSILON, SVD_MAX_SWEEPS, s);
  svd_finish_kernel<<<nb, 256, 0, s>>>(q, q, X2, V, nullptr, nullptr, nullptr, nrm, rank);
  TTG_CHECK_LAUNCH();
  svd_rank_kernel<<<ceil_div(q, 256), 256, 0, s>>>(q, nrm, rank);
  TTG_CHECK_LAUNCH();
  // Ux = U2 (sorted), sigma, Vtx = V2^T (sorted rows)
  svd_gather_kernel<<<gbl((i64)q * q), 256, 0, s>>>(q, q, X2, V, nrm, rank, Ux, sigma, Vtx);
  TTG_CHECK_LAUNCH();
  if (qr2) {
    // U = Q1 [U2; 0]; W = Q2 V2, Vt = (P W)^T
    qr_c0n_kernel<<<gbl((i64)p * q), 256, 0, s>>>(p, q, Ux, U);
    TTG_CHECK_LAUNCH();
    qr_apply(p, A, Tf, U);
    transpose_f64(q, q, Vtx, W, s);
    qr_apply(q, X, Tf2, W);
    qr_vt_kernel<<<gbl((i64)q * q), 256, 0, s>>>(q, W, perm, Vt);
  } else {
    // R1 = V2 S U2^T: U = Q1 [V2; 0], Vt = (P U2)^T
    transpose_f64(q, q, Vtx, W, s);
    qr_c0n_kernel<<<gbl((i64)p * q), 256, 0, s>>>(p, q, W, U);
    TTG_CHECK_LAUNCH();
    qr_apply(p, A, Tf, U);
    qr_vt_kernel<<<gbl((i64)q * q), 256, 0, s>>>(q, Ux, perm, Vt);
  }
  TTG_CHECK_LAUNCH();
}

constexpr int SVD_QR_MIN_Q = 16;   // narrower blocks keep the plain sweeps

static void svd_tall(int p, int q, double* Mw, double* U, double* sigma, double* Vt,
                     double* V, double* nrm, int* rank, int* counters, int* status,
                     double* tmp, cudaStream_t s, double* qrwork) {
  // Mw (p x q, p >= q) is overwritten.  tmp: 2 q^2 + p q doubles.
  if (qrwork && q >= SVD_QR_MIN_Q) {
    svd_tall_qr(p, q, Mw, U, sigma, Vt, V, nrm, rank, counters, status, tmp, qrwork, s);
    return;
  }
  int init_v = 0;
  double* Y = tmp;
  double* Z = tmp + (size_t)q * q;
  double* W = tmp + 2 * (size_t)q * q;
  const size_t smem32 = ((size_t)p * q + (size_t)q * q) * sizeof(float);
  if (q >= 8) {
    if (smem32 <= SVD32_SMEM) {
      // FP32 pre-sweeps in one CTA's shared memory
      static const cudaError_t attr_rc = cudaFuncSetAttribute(
          svd_pre32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SVD32_SMEM);
      TTG_CUDA(attr_rc);
      svd_pre32_kernel<<<1, SVD32_NT, smem32, s>>>(p, q, Mw, V, status);
      TTG_CHECK_LAUNCH();
    } else {
      // FP32 pre-sweeps over the whole grid: M32 in W's space, V32 in Y's
      float* M32 = (float*)W;
      float* V32 = (float*)Y;
      d2f_kernel<<<(int)std::min<i64>(4096, ((i64)p * q + 255) / 256), 256, 0, s>>>((i64)p * q, Mw, M32);
      TTG_CHECK_LAUNCH();
      svd_sweeps<float>(p, q, M32, V32, counters, status, 0, sqrtf((float)p) * FLT_EPSILON,
                        (float)p * FLT_EPSILON, 30, s);
      f2d_kernel<<<(int)std::min<i64>(4096, ((i64)q * q + 255) / 256), 256, 0, s>>>((i64)q * q, V32, V);
      TTG_CHECK_LAUNCH();
    }
    // make V orthogonal to FP64 precision: V <- V (1.5 I - 0.5 V^T V), twice
    for (int it = 0; it < 2; ++it) {
      GemmF64 g;   // Y = V^T V
      g.M = q; g.N = q; g.K = q;
      g.A = V; g.sAm = q; g.sAk = 1;
      g.B = V; g.sBk = 1; g.sBn = q;
      g.C = Y; g.sCm = 1; g.sCn = q;
      gemm_f64(g, s);
      ns_coef_kernel<<<ceil_div((i64)q * q, 256), 256, 0, s>>>(q, Y, Z);
      TTG_CHECK_LAUNCH();
      GemmF64 h;   // W = V Z, then V = W
      h.M = q; h.N = q; h.K = q;
      h.A = V; h.sAm = 1; h.sAk = q;
      h.B = Z; h.sBk = 1; h.sBn = q;
      h.C = W; h.sCm = 1; h.sCn = q;
      gemm_f64(h, s);
      TTG_CUDA(cudaMemcpyAsync(V, W, sizeof(double) * q * q, cudaMemcpyDeviceToDevice, s));
    }
    GemmF64 m;   // W = Mw V (p x q), then Mw = W
    m.M = p; m.N = q; m.K = q;
    m.A = Mw; m.sAm = 1; m.sAk = p;
    m.B = V; m.sBk = 1; m.sBn = q;
    m.C = W; m.sCm = 1; m.sCn = p;
    gemm_f64(m, s);
    TTG_CUDA(cudaMemcpyAsync(Mw, W, sizeof(double) * p * q, cudaMemcpyDeviceToDevice, s));
    init_v = 1;
  }
  svd_sweeps<double>(p, q, Mw, V, counters, status, init_v, sqrt((double)p) * DBL_EPSILON,
                     (double)p * DBL_EPSILON, SVD_MAX_SWEEPS, s);
  int nb = std::max(1, std::min(1024, ceil_div((i64)q * 32, 256)));
  svd_finish_kernel<<<nb, 256, 0, s>>>(p, q, Mw, V, U, sigma, Vt, nrm, rank);
  TTG_CHECK_LAUNCH();
  svd_rank_kernel<<<ceil_div(q, 256), 256, 0, s>>>(q, nrm, rank);
  TTG_CHECK_LAUNCH();
  int gb = (int)std::min<i64>(4096, ((i64)p * q + 255) / 256);
  svd_gather_kernel<<<gb, 256, 0, s>>>(p, q, Mw, V, nrm, rank, U, sigma, Vt);
  TTG_CHECK_LAUNCH();
}

// Thin SVD of M (p x q, column-major):  M = U diag(sigma) Vt
//   U (p x r), sigma (r), Vt (r x q), r = min(p, q)
void svd_jacobi(int p, int q, const double* M, double* U, double* sigma, double* Vt,
                double* scratch, int* status, cudaStream_t s) {
  if (p <= 0 || q <= 0) return;
  int r = std::min(p, q);
  double* Mw = scratch;                                   // max x min
  double* V = Mw + (size_t)std::max(p, q) * r;            // r x r
  double* nrm = V + (size_t)r * r;                        // r
  int* rank = (int*)(nrm + r);                            // r ints (<= r doubles)
  int* counters = (int*)(nrm + 2 * r);                    // 2 ints
  double* T = nrm + 2 * r + 64;                           // max x min (for p < q)
  double* tmp = T + (size_t)std::max(p, q) * r;           // 2 min^2 + max x min
  double* qrw = tmp + 2 * (size_t)r * r + (size_t)std::max(p, q) * r;   // svd_qr_work
  if (p >= q) {
    TTG_CUDA(cudaMemcpyAsync(Mw, M, sizeof(double) * (size_t)p * q, cudaMemcpyDeviceToDevice, s));
    svd_tall(p, q, Mw, U, sigma, Vt, V, nrm, rank, counters, status, tmp, s, qrw);
  } else {
    // M^T = V S U^T: run on the q x p transpose, then U_M = Vt_T^T, Vt_M = U_T^T
    transpose_f64(p, q, M, Mw, s);                        // Mw: q x p
    double* UT = T;                                       // q x p   (left vectors of M^T)
    double* VtT = U;                                      // p x p   written into U's storage
    svd_tall(q, p, Mw, UT, sigma, VtT, V, nrm, rank, counters, status, tmp, s, qrw);
    // U (p x p) = VtT^T ; VtT currently occupies U: transpose through Mw
    TTG_CUDA(cudaMemcpyAsync(Mw, VtT, sizeof(double) * (size_t)p * p, cudaMemcpyDeviceToDevice, s));
    transpose_f64(p, p, Mw, U, s);
    // Vt (p x q) = UT^T
    transpose_f64(q, p, UT, Vt, s);
  }
}

// ---------------------------------------------------------------------------
// Householder QR, one CTA, LAPACK reflector convention (real and complex)
// ---------------------------------------------------------------------------
template <class T> struct CT;
template <> struct CT<double> {
  static __device__ double conj(double a) { return a; }
  static __device__ double abs2(double a) { return a * a; }
  static __device__ double re(double a) { return a; }
  static __device__ double im(double) { return 0.0; }
  static __device__ double mk(double r, double) { return r; }
  static __device__ double mul(double a, double b) { return a * b; }
  static __device__ double sub(double a, double b) { return a - b; }
  static __device__ double add(double a, double b) { return a + b; }
  static __device__ double scal(double a, double s) { return a * s; }
};
template <> struct CT<double2> {
  static __device__ double2 conj(double2 a) { return make_double2(a.x, -a.y); }
  static __device__ double abs2(double2 a) { return a.x * a.x + a.y * a.y; }
  static __device__ double re(double2 a) { return a.x; }
  static __device__ double im(double2 a) { return a.y; }
  static __device__ double2 mk(double r, double i) { return make_double2(r, i); }
  static __device__ double2 mul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
  }
  static __device__ double2 sub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
  static __device__ double2 add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
  static __device__ double2 scal(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
};

__device__ __forceinline__ double2 warp_sum2(double2 v) {
  v.x = warp_sum(v.x);
  v.y = warp_sum(v.y);
  return v;
}
__device__ __forceinline__ double warp_sum2(double v) { return warp_sum(v); }

constexpr int QR_NT = 1024;

// complex reciprocal 1/a
__device__ __forceinline__ double2 crecip(double2 a) {
  double d = a.x * a.x + a.y * a.y;
  return make_double2(a.x / d, -a.y / d);
}
__device__ __forceinline__ double crecip(double a) { return 1.0 / a; }

// SM: the matrix is staged in shared memory (small cores: the column sweeps
// then wait on shared rather than global memory latency), same arithmetic.
template <class T, bool SM>
__global__ void __launch_bounds__(QR_NT) qr_kernel(int n, int m, T* Ag, T* R, T* tau) {
  using C = CT<T>;
  __shared__ double red[33];
  __shared__ T s_tau, s_beta;
  extern __shared__ __align__(16) unsigned char qr_dyn[];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int nwarp = QR_NT / 32;
  const int r = min(n, m);
  T* A = Ag;
  if constexpr (SM) {
    A = reinterpret_cast<T*>(qr_dyn);
    for (i64 e = tid; e < (i64)n * m; e += QR_NT) A[e] = Ag[e];
    __syncthreads();
  }
  for (int j = 0; j < r; ++j) {
    T* col = A + (i64)n * j;
    double t = 0.0;
    for (int i = j + 1 + tid; i < n; i += QR_NT) t += C::abs2(col[i]);
    double xnorm2 = block_sum<QR_NT>(t, red);
    if (tid == 0) {
      T alpha = col[j];
      double alphr = C::re(alpha), alphi = C::im(alpha);
      if (xnorm2 == 0.0 && alphi == 0.0) {
        s_tau = C::mk(0.0, 0.0);
        s_beta = alpha;
      } else {
        double nrm = sqrt(alphr * alphr + alphi * alphi + xnorm2);
        double beta = alphr >= 0 ? -nrm : nrm;
        s_tau = C::mk((beta - alphr) / beta, -alphi / beta);
        s_beta = C::mk(beta, 0.0);
      }
      tau[j] = s_tau;
    }
    __syncthreads();
    T tj = s_tau;
    T alpha = col[j];
    if (!(C::re(tj) == 0.0 && C::im(tj) == 0.0)) {
      T sc = crecip(C::sub(alpha, s_beta));
      for (int i = j + 1 + tid; i < n; i += QR_NT) col[i] = C::mul(col[i], sc);
    }
    __syncthreads();
    if (tid == 0) col[j] = s_beta;
    __syncthreads();
    // apply H^H = I - conj(tau) v v^H to A[j:, j+1:m]   (zgeqr2: zlarf with conjg(tau))
    T ctau = C::conj(tj);
    if (!(C::re(tj) == 0.0 && C::im(tj) == 0.0)) {
      for (int c = j + 1 + wid; c < m; c += nwarp) {
        T* cc = A + (i64)n * c;
        T w = lane == 0 ? cc[j] : C::mk(0.0, 0.0);
        for (int i = j + 1 + lane; i < n; i += 32) w = C::add(w, C::mul(C::conj(col[i]), cc[i]));
        w = warp_sum2(w);
        T f = C::mul(ctau, w);
        if (lane == 0) cc[j] = C::sub(cc[j], f);
        for (int i = j + 1 + lane; i < n; i += 32) cc[i] = C::sub(cc[i], C::mul(col[i], f));
      }
    }
    __syncthreads();
  }
  // R (r x m): upper triangle
  for (i64 e = tid; e < (i64)r * m; e += QR_NT) {
    int i = (int)(e % r), c = (int)(e / r);
    R[e] = (i <= c) ? A[i + (i64)n * c] : C::mk(0.0, 0.0);
  }
  __syncthreads();
  // form Q in place (dorg2r / zung2r), columns 0..r-1
  for (int j = r - 1; j >= 0; --j) {
    T* col = A + (i64)n * j;
    T tj = tau[j];
    if (j < r - 1) {
      // apply H(j) = I - tau v v^H to A[j:, j+1:r] from the left, v(j) = 1
      for (int c = j + 1 + wid; c < r; c += nwarp) {
        T* cc = A + (i64)n * c;
        T w = lane == 0 ? cc[j] : C::mk(0.0, 0.0);
        for (int i = j + 1 + lane; i < n; i += 32) w = C::add(w, C::mul(C::conj(col[i]), cc[i]));
        w = warp_sum2(w);
        T f = C::mul(tj, w);
        if (lane == 0) cc[j] = C::sub(cc[j], f);
        for (int i = j + 1 + lane; i < n; i += 32) cc[i] = C::sub(cc[i], C::mul(col[i], f));
      }
    }
    __syncthreads();
    T mt = C::sub(C::mk(0.0, 0.0), tj);
    for (int i = j + 1 + tid; i < n; i += QR_NT) col[i] = C::mul(col[i], mt);
    if (tid == 0) col[j] = C::sub(C::mk(1.0, 0.0), tj);
    for (int i = tid; i < j; i += QR_NT) col[i] = C::mk(0.0, 0.0);
    __syncthreads();
  }
  if constexpr (SM) {
    __syncthreads();
    for (i64 e = tid; e < (i64)n * m; e += QR_NT) Ag[e] = A[e];
  }
}

constexpr size_t QR_SMEM_MAX = 200 * 1024;
template <class T>
static void qr_launch(int n, int m, T* A, T* R, T* tau, cudaStream_t s) {
  const size_t bytes = (size_t)n * m * sizeof(T);
  if (bytes <= QR_SMEM_MAX) {
    static const bool attr_ok = cudaFuncSetAttribute(qr_kernel<T, true>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)QR_SMEM_MAX) == cudaSuccess;
    if (attr_ok) {
      qr_kernel<T, true><<<1, QR_NT, bytes, s>>>(n, m, A, R, tau);
      TTG_CHECK_LAUNCH();
      return;
    }
    (void)cudaGetLastError();
  }
  qr_kernel<T, false><<<1, QR_NT, 0, s>>>(n, m, A, R, tau);
  TTG_CHECK_LAUNCH();
}

void qr_householder(int n, int m, double* A, double* R, double* tau, cudaStream_t s) {
  if (n <= 0 || m <= 0) return;
  qr_launch<double>(n, m, A, R, tau, s);
}
void qr_householder_z(int n, int m, double2* A, double2* R, double2* tau, cudaStream_t s) {
  if (n <= 0 || m <= 0) return;
  qr_launch<double2>(n, m, A, R, tau, s);
}

}  // namespace ttg

namespace ttg {

// ---------------------------------------------------------------------------
// Lowest eigenpairs of a dense symmetric matrix through the Jacobi SVD: with
// c = ||H||_F, H + c I is positive semidefinite, so its singular vectors are
// its eigenvectors and its singular values are lambda + c.  The one-sided
// Jacobi SVD above (FP32 pre-sweeps + FP64 polish) is much faster on GB300
// than the cyclic two-sided FP64 Jacobi; the shift adds an absolute error of
// order eps ||H||, the backward error of any dense symmetric eigensolver.
// ---------------------------------------------------------------------------
namespace {
__global__ void fro_shift_kernel(int N, double* H, double* cval) {
  __shared__ double red[32];
  double acc = 0.0;
  for (i64 e = threadIdx.x; e < (i64)N * N; e += blockDim.x) acc = fma(H[e], H[e], acc);
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    red[0] = sqrt(t) > 0.0 ? sqrt(t) : 1.0;
    *cval = red[0];
  }
  __syncthreads();
  const double c = red[0];
  for (int i = threadIdx.x; i < N; i += blockDim.x) H[i + (i64)N * i] += c;
}
// w[j] = S[N-1-j] - c, V[:, j] = row N-1-j of Vt (j < k)
__global__ void lowest_pairs_kernel(int N, int k, const double* S, const double* Vt,
                                    const double* cval, double* w, double* V) {
  const double c = *cval;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < (i64)N * k; e += (i64)gridDim.x * blockDim.x) {
    const int r = (int)(e % N), j = (int)(e / N);
    V[e] = Vt[(N - 1 - j) + (i64)N * r];
    if (r == 0) w[j] = S[N - 1 - j] - c;
  }
}
}  // namespace

size_t syev_lowest_scratch(int N) {
  return svd_scratch(N, N) + (2 * (size_t)N * N + N + 64) * sizeof(double);
}

void syev_lowest_svd(int N, int k, double* H, double* w, double* V, double* scratch, int* status,
                     cudaStream_t s) {
  double* U = scratch;
  double* Sv = U + (size_t)N * N;
  double* Vt = Sv + N;
  double* cval = Vt + (size_t)N * N;
  double* svscr = cval + 64;
  fro_shift_kernel<<<1, 1024, 0, s>>>(N, H, cval);
  TTG_CHECK_LAUNCH();
  svd_jacobi(N, N, H, U, Sv, Vt, svscr, status, s);
  lowest_pairs_kernel<<<ceil_div((i64)N * k, 256), 256, 0, s>>>(N, k, Sv, Vt, cval, w, V);
  TTG_CHECK_LAUNCH();
}

}  // namespace ttg
