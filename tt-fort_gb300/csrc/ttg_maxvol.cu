// maxvol row selection on the device (maxvol0_d, maxvol.f90:27-119; the
// start-from-scratch path of maxvol_d, :197-288).
//
//   1. lu_top_kernel (one CTA): LU with partial pivoting of a copy of the tall
//      m x n matrix (dgetrf), then the inverse of the leading n x n block of
//      the pivoted matrix from its factors without pivoting (dgetri with the
//      identity pivot vector: inv(U), then X L = inv(U)), and the row set p
//      that the interchanges move to the top.
//   2. Z = A * inv(A(p,:)) with the FP64 GEMM.
//   3. maxvol_iter_kernel (cooperative): each iteration finds, per column,
//      the first row of largest |z| (idamax) and the first column of the
//      largest of those (maxloc); it stops below 1 + tol or when the row is
//      already selected, else swaps the row into p and applies the rank-1
//      update, forcing the new row to e_j.  Rows are split over the CTAs;
//      three grid barriers per iteration.
// Indices are 0-based (the reference's are 1-based).
#include "ttg_common.cuh"
#include <cooperative_groups.h>
#include <algorithm>

namespace cg = cooperative_groups;

namespace ttg {
namespace {

constexpr int LU_NT = 1024;
constexpr int MV_NT = 256;
constexpr int MV_MAX_ROWS = 2048;   // rows one CTA of the iteration kernel owns

// (value, index) maximum: larger value wins, equal values keep the lower index
__device__ __forceinline__ void better(double& v, long long& i, double v2, long long i2) {
  if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
}
__device__ __forceinline__ void warp_best(double& v, long long& i) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double v2 = __shfl_xor_sync(0xffffffffu, v, o);
    long long i2 = __shfl_xor_sync(0xffffffffu, i, o);
    better(v, i, v2, i2);
  }
}
__device__ void block_best(double& v, long long& i, double* sv, long long* si) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  warp_best(v, i);
  __syncthreads();
  if (lane == 0) { sv[w] = v; si[w] = i; }
  __syncthreads();
  if (w == 0) {
    v = lane < nw ? sv[lane] : -1.0;
    i = lane < nw ? si[lane] : (1ll << 62);
    warp_best(v, i);
    if (lane == 0) { sv[0] = v; si[0] = i; }
  }
  __syncthreads();
  v = sv[0];
  i = si[0];
}

// W (m x n, ld m) is factored in place; B (n x n) receives inv(L_n U_n);
// per (m ints) is scratch; p (n) receives the selected rows; status 0 ok,
// 1 = exactly singular leading block (the reference stops on info != 0).
__global__ void __launch_bounds__(LU_NT) lu_top_kernel(i64 m, int n, double* W, double* B,
                                                        long long* per, long long* p,
                                                        int* status) {
  __shared__ double sv[32];
  __shared__ long long si[32];
  __shared__ long long piv_s[1];
  const int tid = threadIdx.x;
  if (tid == 0) *status = 0;
  for (i64 r = tid; r < m; r += LU_NT) per[r] = r;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    double v = -1.0;
    long long idx = 1ll << 62;
    for (i64 r = k + tid; r < m; r += LU_NT) better(v, idx, fabs(W[r + m * k]), r);
    block_best(v, idx, sv, si);
    if (v == 0.0) {
      if (tid == 0) *status = 1;
      return;
    }
    if (tid == 0) {
      piv_s[0] = idx;
      const long long t = per[k];   // per(k) <-> per(piv(k))
      per[k] = per[idx];
      per[idx] = t;
    }
    __syncthreads();
    const i64 pr = piv_s[0];
    if (pr != k)
      for (int j = tid; j < n; j += LU_NT) {
        const double t = W[k + m * j];
        W[k + m * j] = W[pr + m * j];
        W[pr + m * j] = t;
      }
    __syncthreads();
    const double rp = 1.0 / W[k + m * k];
    for (i64 r = k + 1 + tid; r < m; r += LU_NT) W[r + m * k] *= rp;
    __syncthreads();
    // trailing update W(k+1:, k+1:) -= W(k+1:, k) W(k, k+1:)
    const i64 rows = m - k - 1;
    const int cols = n - k - 1;
    for (i64 e = tid; e < rows * cols; e += LU_NT) {
      const i64 r = k + 1 + e % rows;
      const int j = k + 1 + (int)(e / rows);
      W[r + m * j] = fma(-W[r + m * k], W[k + m * j], W[r + m * j]);
    }
    __syncthreads();
  }
  // B = inv(U) (upper), column by column: B(j,j) = 1/U(j,j),
  // B(i,j) = -B(j,j) * sum_{k=i..j-1} B(i,k) U(k,j)
  for (int e = tid; e < n * n; e += LU_NT) B[e] = 0.0;
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    if (tid == 0) B[j + n * j] = 1.0 / W[j + m * j];
    __syncthreads();
    const double bjj = B[j + n * j];
    for (int i = tid; i < j; i += LU_NT) {
      double t = 0.0;
      for (int k = i; k < j; ++k) t = fma(B[i + n * k], W[k + m * j], t);
      B[i + n * j] = -bjj * t;
    }
    __syncthreads();
  }
  // X L = inv(U): for j = n-1 .. 0, X(:, j) -= sum_{k>j} X(:, k) L(k, j)
  for (int j = n - 2; j >= 0; --j) {
    for (int i = tid; i < n; i += LU_NT) {
      double t = B[i + n * j];
      for (int k = j + 1; k < n; ++k) t = fma(-B[i + n * k], W[k + m * j], t);
      B[i + n * j] = t;
    }
    __syncthreads();
  }
  for (int j = tid; j < n; j += LU_NT) p[j] = per[j];
}

struct IterArgs {
  i64 m;
  int n;
  double* Z;
  long long* p;
  double* pv;          // partial maxima (nblocks x n)
  long long* pi;       // their rows
  double tol;
  int maxiter;
  int* status;         // [0] iterations, [1] error
};

__global__ void __launch_bounds__(MV_NT) maxvol_iter_kernel(IterArgs a) {
  cg::grid_group grid = cg::this_grid();
  extern __shared__ double sh[];   // n (row difference) + rows (pivot column)
  __shared__ double sv[32];
  __shared__ long long si[32];
  __shared__ int sdone;
  __shared__ long long sij[3];     // i*, j*, ip
  const i64 m = a.m;
  const int n = a.n;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = MV_NT >> 5;
  const i64 per_cta = (m + gridDim.x - 1) / gridDim.x;
  const i64 r0 = (i64)blockIdx.x * per_cta;
  const i64 r1 = r0 + per_cta < m ? r0 + per_cta : (m > r0 ? m : r0);
  double* vrow = sh;
  double* ucol = sh + n;
  int it = 0;
  for (it = 1; it <= a.maxiter; ++it) {
    // (a) per column: the first row of largest |z| among this CTA's rows
    for (int j = w; j < n; j += nw) {
      double v = -1.0;
      long long idx = 1ll << 62;
      for (i64 r = r0 + lane; r < r1; r += 32) better(v, idx, fabs(a.Z[r + m * j]), r);
      warp_best(v, idx);
      if (lane == 0) {
        a.pv[(i64)blockIdx.x * n + j] = v;
        a.pi[(i64)blockIdx.x * n + j] = idx;
      }
    }
    grid.sync();
    // (b) every CTA reduces the same partials: per column over CTAs, then
    // the first column of largest maximum
    double bv = -1.0;
    long long bj = 1ll << 62, bi = 0;
    for (int j = w; j < n; j += nw) {
      double v = -1.0;
      long long idx = 1ll << 62;
      for (int c = lane; c < (int)gridDim.x; c += 32)
        better(v, idx, a.pv[(i64)c * n + j], a.pi[(i64)c * n + j]);
      warp_best(v, idx);
      // columns compete on (value, column index)
      long long jj = j;
      if (v > bv || (v == bv && jj < bj)) { bv = v; bj = jj; bi = idx; }
    }
    // combine the warps' best columns (lane 0 of each warp holds it)
    if (lane == 0) { sv[w] = bv; si[w] = bj; }
    __syncthreads();
    if (tid == 0) {
      double v = -1.0;
      long long j = 1ll << 62;
      for (int q = 0; q < nw; ++q)
        if (sv[q] > v || (sv[q] == v && si[q] < j)) { v = sv[q]; j = si[q]; }
      sij[1] = j;
    }
    __syncthreads();
    // the winning warp's lane 0 knows the row of the winning column
    if (lane == 0 && bj == sij[1]) sij[0] = bi;
    __syncthreads();
    const i64 is = sij[0];
    const int js = (int)sij[1];
    if (tid == 0) {
      const double amax = fabs(a.Z[is + m * js]);
      sdone = (amax < 1.0 + a.tol || a.p[js] == is) ? 1 : 0;
      sij[2] = a.p[js];
    }
    __syncthreads();
    if (sdone) break;
    const i64 ip = sij[2];
    const double zinv = 1.0 / a.Z[is + m * js];
    for (int j = tid; j < n; j += MV_NT) vrow[j] = zinv * (a.Z[ip + m * j] - a.Z[is + m * j]);
    for (i64 r = r0 + tid; r < r1; r += MV_NT) ucol[r - r0] = a.Z[r + m * js];
    grid.sync();   // everyone has read rows ip and i* and its pivot column
    if (blockIdx.x == 0 && tid == 0) a.p[js] = is;
    const i64 rows = r1 - r0;
    for (i64 e = tid; e < rows * n; e += MV_NT) {
      const i64 r = r0 + e % rows;
      const int j = (int)(e / rows);
      a.Z[r + m * j] = fma(ucol[r - r0], vrow[j], a.Z[r + m * j]);
    }
    __syncthreads();
    if (is >= r0 && is < r1)
      for (int j = tid; j < n; j += MV_NT) a.Z[is + m * j] = (j == js) ? 1.0 : 0.0;
    grid.sync();
  }
  if (blockIdx.x == 0 && tid == 0) a.status[0] = it < a.maxiter ? it : a.maxiter;
}

}  // namespace

}  // namespace ttg

using namespace ttg;

extern "C" int ttg_dmaxvol(ttg_ctx* c, ttg_int m, ttg_int n, const double* A, ttg_int* p,
                           double* Z, double tol, ttg_int maxiters) {
  if (!c) return TTG_ERR_ARG;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    TTG_REQUIRE(m > 0 && n > 0 && m >= n, "maxvol: need a tall matrix (m >= n > 0)");
    TTG_REQUIRE(A && p, "maxvol: null pointer");
    TTG_REQUIRE(n <= 4096 && m < (1ll << 40), "maxvol: matrix too large");
    TTG_REQUIRE(tol >= 0.0, "maxvol: tol must be non-negative");
    const int maxit = maxiters > 0 ? (int)std::min<ttg_int>(maxiters, 1 << 30) : 1024;
    cudaStream_t s = c->stream;
    // cooperative grid for the iterations
    static const int max_coop = [] {
      int dev = 0, nsm = 0, per = 0;
      if (cudaGetDevice(&dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, maxvol_iter_kernel, MV_NT,
                                                        (MV_MAX_ROWS + 4096) * sizeof(double)) !=
              cudaSuccess)
        return 0;
      return nsm * std::max(per, 1);
    }();
    TTG_REQUIRE(max_coop > 0, "maxvol: occupancy query failed");
    int blocks = (int)std::min<i64>(std::min(max_coop, 152), std::max<i64>(1, ceil_div(m, (i64)64)));
    blocks = std::max(blocks, (int)std::min<i64>(max_coop, ceil_div(m, (i64)MV_MAX_ROWS)));
    TTG_REQUIRE(ceil_div(m, (i64)blocks) <= MV_MAX_ROWS, "maxvol: too many rows for one grid");
    const i64 per_cta = ceil_div(m, (i64)blocks);
    c->ws.reset();
    const size_t need = sizeof(double) * ((size_t)m * n * 2 + (size_t)n * n + (size_t)blocks * n) +
                        sizeof(long long) * ((size_t)m + (size_t)blocks * n) + 4096;
    c->ws.reserve(need);
    double* W = c->ws.takeT<double>((size_t)m * n);
    double* B = c->ws.takeT<double>((size_t)n * n);
    double* Zw = Z ? Z : c->ws.takeT<double>((size_t)m * n);
    double* pv = c->ws.takeT<double>((size_t)blocks * n);
    long long* per = c->ws.takeT<long long>((size_t)m);
    long long* pi = c->ws.takeT<long long>((size_t)blocks * n);
    int* status = c->ws.takeT<int>(4);
    TTG_CUDA(cudaMemcpyAsync(W, A, sizeof(double) * m * n, cudaMemcpyDeviceToDevice, s));
    lu_top_kernel<<<1, LU_NT, 0, s>>>(m, (int)n, W, B, per, (long long*)p, status);
    TTG_CHECK_LAUNCH();
    int hst[2] = {0, 0};
    TTG_CUDA(cudaMemcpyAsync(hst, status, sizeof(int), cudaMemcpyDeviceToHost, s));
    TTG_CUDA(cudaStreamSynchronize(s));
    if (hst[0]) throw Error{TTG_ERR_ARG, "maxvol: the pivoted leading block is singular"};
    {  // Z = A * B
      GemmF64 g;
      g.M = (int)m; g.N = (int)n; g.K = (int)n;
      g.A = A; g.sAm = 1; g.sAk = m;
      g.B = B; g.sBk = 1; g.sBn = n;
      g.C = Zw; g.sCm = 1; g.sCn = m;
      gemm_f64(g, s);
    }
    IterArgs ia{m, (int)n, Zw, (long long*)p, pv, pi, tol, maxit, status};
    void* args[] = {&ia};
    const size_t smem = sizeof(double) * ((size_t)n + (size_t)per_cta);
    if (smem > 48 * 1024)
      TTG_CUDA(cudaFuncSetAttribute(maxvol_iter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
    TTG_CUDA(cudaLaunchCooperativeKernel((void*)maxvol_iter_kernel, dim3(blocks), dim3(MV_NT), args,
                                         smem, s));
    ++g_launches;
    TTG_CUDA(cudaStreamSynchronize(s));
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}
