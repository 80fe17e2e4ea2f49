// Expokit ZGEXPV / ZGPADM and the Higham-Tisseur block 1-norm estimate on the
// device (the KSL time stepper's local exponentials, tt_ksl.f90:567-625).
//
// ZGEXPV (expm/expokit.f:2403-2793) is restated with the same step logic:
// Arnoldi with modified Gram-Schmidt (one CTA per Krylov step, the matvec in
// between), happy breakdown below 1e-7, the (m+2) x (m+2) Pade exponential of
// degree 6 with scaling and squaring (ZGPADM, expokit.f:767-940) in one CTA,
// the local error estimate from the last two entries of its first column,
// rejection and the delta = 1.2 / gamma = 0.9 step rule with step sizes
// rounded to two significant digits.  The vectors never leave the device; the
// host reads the few scalars that steer the step control.
//
// The 1-norm estimate restates ZLACN1 (expm/zlacn1.f) as driven by
// znormest_higham (expm/normest.f90:52-94): t = 4 columns, ITMAX = 5, the
// first column all ones, the others on the unit circle from a splitmix64
// stream (LAPACK's ZLARNV is not part of the reference; the oracle uses the
// same stream), the top-t selection breaking ties by the lower index.
#include "ttg_expokit.cuh"
#include <cooperative_groups.h>
#include <algorithm>
#include <cfloat>
#include <cmath>

namespace cg = cooperative_groups;

namespace ttg {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double cabsd(double2 a) { return hypot(a.x, a.y); }
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  // Smith's algorithm
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, den = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  }
  double r = b.x / b.y, den = b.x * r + b.y;
  return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sum (all threads get the result); red has >= 33 slots
__device__ double bsum(double v, double* red) {
  v = wsum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
    t = wsum(t);
    if (lane == 0) red[32] = t;
  }
  __syncthreads();
  return red[32];
}

size_t ExpWork::bytes(i64 nmax, int m) {
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  return al(sizeof(double2) * nmax * (m + 1)) + al(sizeof(double2) * nmax) +
         2 * al(sizeof(double2) * nmax * 4) + al(sizeof(double2) * (m + 2) * (m + 2)) +
         al(sizeof(double2) * (m + 2)) + al(sizeof(double) * 64) + al(sizeof(int) * 64) +
         al(sizeof(double2) * 64 * (m + 2)) + 4096;
}

void ExpWork::bind(void* mem, i64 nmax_, int m_, double* pinned) {
  nmax = nmax_;
  m = m_;
  hbuf = pinned;
  char* p = (char*)mem;
  auto take = [&](size_t b) {
    void* r = p;
    p += (b + 255) & ~size_t(255);
    return r;
  };
  V = (double2*)take(sizeof(double2) * nmax * (m + 1));
  tmp = (double2*)take(sizeof(double2) * nmax);
  X = (double2*)take(sizeof(double2) * nmax * 4);
  Y = (double2*)take(sizeof(double2) * nmax * 4);
  H = (double2*)take(sizeof(double2) * (m + 2) * (m + 2));
  E = (double2*)take(sizeof(double2) * (m + 2));
  red = (double*)take(sizeof(double) * 64);
  ired = (int*)take(sizeof(int) * 64);
  part = (double2*)take(sizeof(double2) * 64 * (m + 2));
}

// ---------------------------------------------------------------------------
// norm estimate kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 unit_random(unsigned long long k) {
  unsigned long long z = k * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  const double u = (double)(z >> 11) * 0x1.0p-53;
  const double ang = 2.0 * 3.141592653589793 * u;
  double sn, cs;
  sincos(ang, &sn, &cs);
  return make_double2(cs, sn);
}

__global__ void ne_init_kernel(i64 n, int t, unsigned long long counter, double2* X) {
  const double sc = 1.0 / (double)n;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n * t; e += (i64)gridDim.x * blockDim.x) {
    const i64 i = e % n;
    const int j = (int)(e / n);
    double2 v = j == 0 ? make_double2(1.0, 0.0)
                       : unit_random(counter + (unsigned long long)(j - 1) * n + i + 1);
    X[e] = cscale(v, sc);
  }
}

// one CTA per column: out[j] = sum_i |X(i, j)|
__global__ void ne_colsum_kernel(i64 n, const double2* X, double* out) {
  __shared__ double red[33];
  const int j = blockIdx.x;
  double acc = 0.0;
  for (i64 i = threadIdx.x; i < n; i += blockDim.x) acc += cabsd(X[i + n * j]);
  acc = bsum(acc, red);
  if (threadIdx.x == 0) out[j] = acc;
}

__global__ void ne_sign_kernel(i64 total, const double2* X, double2* S) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
    const double a = cabsd(X[e]);
    S[e] = a > DBL_MIN ? make_double2(X[e].x / a, X[e].y / a) : make_double2(1.0, 0.0);
  }
}

// h(i) = max_j |X(i,j)|; top-t rows by (h desc, index asc); out: ind[0..t),
// red[0] = h of the top row, red[1] = h(ibest).  One CTA of TOPK_NT threads.
constexpr int TOPK_NT = 256;
__global__ void __launch_bounds__(TOPK_NT) ne_topk_kernel(i64 n, int t, const double2* X, int ibest,
                                                          int* ind, double* red_out) {
  __shared__ double cv[TOPK_NT * 4];
  __shared__ long long ci[TOPK_NT * 4];
  __shared__ double bv[32];
  __shared__ long long bi[32];
  __shared__ int bs[32];
  const int tid = threadIdx.x;
  double lv[4];
  long long li[4];
  for (int q = 0; q < 4; ++q) { lv[q] = -1.0; li[q] = -1; }
  for (i64 i = tid; i < n; i += blockDim.x) {
    double h = 0.0;
    for (int j = 0; j < t; ++j) h = fmax(h, cabsd(X[i + n * j]));
    if (i == ibest) red_out[1] = h;
    // insert (h, i) into the local sorted list (desc h, asc index)
    for (int q = 0; q < t; ++q) {
      if (h > lv[q] || (h == lv[q] && (li[q] < 0 || i < li[q]))) {
        for (int r = t - 1; r > q; --r) { lv[r] = lv[r - 1]; li[r] = li[r - 1]; }
        lv[q] = h;
        li[q] = i;
        break;
      }
    }
  }
  for (int q = 0; q < 4; ++q) { cv[tid * 4 + q] = lv[q]; ci[tid * 4 + q] = li[q]; }
  __syncthreads();
  // t rounds of a block-wide arg-max over the candidates
  for (int r = 0; r < t; ++r) {
    double best = -2.0;
    long long bidx = -1;
    int bslot = -1;
    for (int q = tid; q < TOPK_NT * 4; q += blockDim.x) {
      double v = cv[q];
      long long ii = ci[q];
      if (ii < 0) continue;
      if (v > best || (v == best && ii < bidx)) { best = v; bidx = ii; bslot = q; }
    }
    // warp reduce
    for (int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_xor_sync(0xffffffffu, best, o);
      long long oi = __shfl_xor_sync(0xffffffffu, bidx, o);
      int os = __shfl_xor_sync(0xffffffffu, bslot, o);
      if (oi >= 0 && (ov > best || (ov == best && (bidx < 0 || oi < bidx)))) {
        best = ov; bidx = oi; bslot = os;
      }
    }
    if ((tid & 31) == 0) { bv[tid >> 5] = best; bi[tid >> 5] = bidx; bs[tid >> 5] = bslot; }
    __syncthreads();
    if (tid == 0) {
      double b = -2.0;
      long long ix = -1;
      int sl = -1;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        if (bi[w] >= 0 && (bv[w] > b || (bv[w] == b && (ix < 0 || bi[w] < ix)))) {
          b = bv[w]; ix = bi[w]; sl = bs[w];
        }
      }
      ind[r] = (int)ix;
      if (r == 0) red_out[0] = b;
      if (sl >= 0) ci[sl] = -1;   // remove it from the candidates
    }
    __syncthreads();
  }
}

__global__ void ne_unit_kernel(i64 n, int t, const int* ind, double2* X) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n * t; e += (i64)gridDim.x * blockDim.x) {
    const i64 i = e % n;
    const int j = (int)(e / n);
    X[e] = (i == ind[j]) ? make_double2(1.0, 0.0) : make_double2(0.0, 0.0);
  }
}

static int eblocks(i64 total) { return (int)std::max<i64>(1, std::min<i64>(4096, (total + 255) / 256)); }

double znormest_dev(ExpWork& w, i64 n, int t0, const ZMatvecFn& mv, const ZMatvecFn* transp,
                    unsigned long long& counter, cudaStream_t s, ExpStats* st) {
  const int t = (int)std::min<i64>(n, t0);
  const int itmax = 5;
  double* h = w.hbuf;
  auto sync = [&]() {
    TTG_CUDA(cudaStreamSynchronize(s));
    if (st) st->syncs++;
  };
  ne_init_kernel<<<eblocks(n * t), 256, 0, s>>>(n, t, counter, w.X);
  TTG_CHECK_LAUNCH();
  counter += (unsigned long long)n * (t - 1);
  mv(w.X, w.Y, t);
  std::swap(w.X, w.Y);
  double estold = 0.0;
  int ibest = 0;
  int ind[8];
  for (int j = 0; j < t; ++j) ind[j] = j;
  for (int it = 1;; ++it) {
    if (it == 1 && n == 1) {
      TTG_CUDA(cudaMemcpyAsync(h, w.X, sizeof(double2), cudaMemcpyDeviceToHost, s));
      sync();
      return std::hypot(h[0], h[1]);
    }
    ne_colsum_kernel<<<t, 256, 0, s>>>(n, w.X, w.red);
    TTG_CHECK_LAUNCH();
    TTG_CUDA(cudaMemcpyAsync(h, w.red, sizeof(double) * t, cudaMemcpyDeviceToHost, s));
    sync();
    int itemp = 0;
    double est = 0.0;
    for (int j = 0; j < t; ++j)
      if (h[j] > est) { est = h[j]; itemp = j; }
    if (est > estold || it == 2) ibest = ind[itemp];
    if (est <= estold && it >= 2) return estold;
    estold = est;
    if (it > itmax) return est;
    ne_sign_kernel<<<eblocks(n * t), 256, 0, s>>>(n * t, w.X, w.Y);
    TTG_CHECK_LAUNCH();
    if (transp) {
      (*transp)(w.Y, w.X, t);
    } else {
      std::swap(w.X, w.Y);
    }
    ne_topk_kernel<<<1, TOPK_NT, 0, s>>>(n, t, w.X, ibest, w.ired, w.red);
    TTG_CHECK_LAUNCH();
    TTG_CUDA(cudaMemcpyAsync(h, w.red, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
    TTG_CUDA(cudaMemcpyAsync(h + 8, w.ired, sizeof(int) * t, cudaMemcpyDeviceToHost, s));
    sync();
    if (it >= 2 && h[0] == h[1]) return est;
    if (it >= 2 && t > 1 && (i64)(it - 1) * t > n) return est;
    const int* hi = (const int*)(h + 8);
    for (int j = 0; j < t; ++j) ind[j] = hi[j];
    ne_unit_kernel<<<eblocks(n * t), 256, 0, s>>>(n, t, w.ired, w.X);
    TTG_CHECK_LAUNCH();
    mv(w.X, w.Y, t);
    std::swap(w.X, w.Y);
  }
}

// ---------------------------------------------------------------------------
// Krylov step kernels
// ---------------------------------------------------------------------------
// v = a * src (complex vector, real scale from device or host)
__global__ void zscale_kernel(i64 n, const double2* src, double2* dst, const double* sdev, double shost) {
  const double sc = sdev ? 1.0 / sdev[0] : shost;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    dst[i] = cscale(src[i], sc);
}

// out[0] = ||x||_2 (one CTA)
__global__ void znrm2_kernel(i64 n, const double2* x, double* out) {
  __shared__ double red[33];
  double acc = 0.0;
  for (i64 i = threadIdx.x; i < n; i += blockDim.x) acc += cabs2(x[i]);
  acc = bsum(acc, red);
  if (threadIdx.x == 0) out[0] = sqrt(acc);
}

// Modified Gram-Schmidt of column j+1 of V against columns 0..j (one CTA).
// flag[0] = mbrkdwn (0 while no breakdown): once set, later steps do nothing.
__global__ void mgs_kernel(i64 n, int j, int mh, double2* V, double2* H, int* flag,
                           double break_tol) {
  __shared__ double red[33];
  if (flag[0] != 0) return;
  double2* p = V + n * (j + 1);
  for (int i = 0; i <= j; ++i) {
    const double2* vi = V + n * i;
    double ar = 0.0, ai = 0.0;
    for (i64 k = threadIdx.x; k < n; k += blockDim.x) {
      // conj(vi) * p
      ar += vi[k].x * p[k].x + vi[k].y * p[k].y;
      ai += vi[k].x * p[k].y - vi[k].y * p[k].x;
    }
    ar = bsum(ar, red);
    ai = bsum(ai, red);
    const double2 hij = make_double2(ar, ai);
    for (i64 k = threadIdx.x; k < n; k += blockDim.x) p[k] = csub(p[k], cmul(hij, vi[k]));
    if (threadIdx.x == 0) H[i + (i64)mh * j] = hij;
    __syncthreads();
  }
  double acc = 0.0;
  for (i64 k = threadIdx.x; k < n; k += blockDim.x) acc += cabs2(p[k]);
  const double nrm = sqrt(bsum(acc, red));
  if (nrm <= break_tol) {
    if (threadIdx.x == 0) flag[0] = j + 1;
    return;
  }
  if (threadIdx.x == 0) H[(j + 1) + (i64)mh * j] = make_double2(nrm, 0.0);
  const double inv = 1.0 / nrm;
  for (i64 k = threadIdx.x; k < n; k += blockDim.x) p[k] = cscale(p[k], inv);
}

// The same step in one warp, for small vectors (S-step problems): warp
// shuffles only, no block barriers.
__global__ void mgs_warp_kernel(i64 n, int j, int mh, double2* V, double2* H, int* flag,
                                double break_tol) {
  if (flag[0] != 0) return;
  double2* p = V + n * (j + 1);
  const int lane = threadIdx.x;
  for (int i = 0; i <= j; ++i) {
    const double2* vi = V + n * i;
    double ar = 0.0, ai = 0.0;
    for (i64 k = lane; k < n; k += 32) {
      const double2 a = vi[k], c = p[k];
      ar += a.x * c.x + a.y * c.y;
      ai += a.x * c.y - a.y * c.x;
    }
    const double2 hij = make_double2(wsum(ar), wsum(ai));
    for (i64 k = lane; k < n; k += 32) p[k] = csub(p[k], cmul(hij, vi[k]));
    if (lane == 0) H[i + (i64)mh * j] = hij;
    __syncwarp();
  }
  double acc = 0.0;
  for (i64 k = lane; k < n; k += 32) acc += cabs2(p[k]);
  const double nrm = sqrt(wsum(acc));
  if (nrm <= break_tol) {
    if (lane == 0) flag[0] = j + 1;
    return;
  }
  if (lane == 0) H[(j + 1) + (i64)mh * j] = make_double2(nrm, 0.0);
  const double inv = 1.0 / nrm;
  for (i64 k = lane; k < n; k += 32) p[k] = cscale(p[k], inv);
}

// The same modified Gram-Schmidt step spread over the CTAs of a cooperative
// grid: FP64 runs at two FMAs per clock per SM on GB300, so one CTA would
// leave the step FP64-bound on a single SM.  Each CTA owns a contiguous slice
// of the vector; per column the slices' partial dot products go to their own
// slots of part (round r uses part[r * gridDim.x ...]), and after a grid
// barrier every CTA sums them in the same order.
constexpr int MGS_NT = 128;
__global__ void __launch_bounds__(MGS_NT) mgs_coop_kernel(i64 n, int j, int mh, double2* V,
                                                          double2* H, int* flag, double break_tol,
                                                          double2* part) {
  __shared__ double red[33];
  __shared__ double2 tot;
  cg::grid_group grid = cg::this_grid();
  if (flag[0] != 0) return;   // uniform: flag changes only after the last barrier
  const int G = gridDim.x, b = blockIdx.x;
  const i64 chunk = (n + G - 1) / G;
  const i64 lo = std::min<i64>(n, chunk * b), hi = std::min<i64>(n, lo + chunk);
  double2* p = V + n * (j + 1);
  auto reduce_slots = [&](int r) {
    // every CTA sums the G partials of round r in index order
    if (threadIdx.x < 32) {
      double ax = 0.0, ay = 0.0;
      for (int q = threadIdx.x; q < G; q += 32) {
        const double2 v = __ldcg(part + (i64)r * G + q);
        ax += v.x;
        ay += v.y;
      }
      ax = wsum(ax);
      ay = wsum(ay);
      if (threadIdx.x == 0) tot = make_double2(ax, ay);
    }
    __syncthreads();
    return tot;
  };
  for (int i = 0; i <= j; ++i) {
    const double2* vi = V + n * i;
    double ar = 0.0, ai = 0.0;
    for (i64 k = lo + threadIdx.x; k < hi; k += blockDim.x) {
      const double2 a = vi[k], c = p[k];
      ar += a.x * c.x + a.y * c.y;
      ai += a.x * c.y - a.y * c.x;
    }
    ar = bsum(ar, red);
    ai = bsum(ai, red);
    if (threadIdx.x == 0) part[(i64)i * G + b] = make_double2(ar, ai);
    grid.sync();
    const double2 hij = reduce_slots(i);
    for (i64 k = lo + threadIdx.x; k < hi; k += blockDim.x) p[k] = csub(p[k], cmul(hij, vi[k]));
    if (b == 0 && threadIdx.x == 0) H[i + (i64)mh * j] = hij;
    __syncthreads();
  }
  double acc = 0.0;
  for (i64 k = lo + threadIdx.x; k < hi; k += blockDim.x) acc += cabs2(p[k]);
  acc = bsum(acc, red);
  if (threadIdx.x == 0) part[(i64)(j + 1) * G + b] = make_double2(acc, 0.0);
  grid.sync();
  const double nrm = sqrt(reduce_slots(j + 1).x);
  if (nrm <= break_tol) {
    if (b == 0 && threadIdx.x == 0) flag[0] = j + 1;
    return;
  }
  if (b == 0 && threadIdx.x == 0) H[(j + 1) + (i64)mh * j] = make_double2(nrm, 0.0);
  const double inv = 1.0 / nrm;
  for (i64 k = lo + threadIdx.x; k < hi; k += blockDim.x) p[k] = cscale(p[k], inv);
}

static void mgs_step(ExpWork& w, i64 n, int j, int mh, double break_tol, cudaStream_t s) {
  static const int G_MAX = [] {
    int dev = 0, per = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, mgs_coop_kernel, MGS_NT, 0);
    return std::max(1, std::min(64, per * sms));
  }();
  const int G = (int)std::max<i64>(1, std::min<i64>(G_MAX, (n + 2 * MGS_NT - 1) / (2 * MGS_NT)));
  if (n <= 1024) {
    mgs_warp_kernel<<<1, 32, 0, s>>>(n, j, mh, w.V, w.H, w.ired, break_tol);
    TTG_CHECK_LAUNCH();
    return;
  }
  if (G == 1) {
    mgs_kernel<<<1, 1024, 0, s>>>(n, j, mh, w.V, w.H, w.ired, break_tol);
    TTG_CHECK_LAUNCH();
    return;
  }
  double2* part = w.part;
  void* args[] = {&n, &j, &mh, &w.V, &w.H, &w.ired, &break_tol, &part};
  TTG_CUDA(cudaLaunchCooperativeKernel((const void*)mgs_coop_kernel, dim3(G), dim3(MGS_NT), args, 0, s));
  g_launches++;
}

// exp(t H[:mx,:mx]) (H with leading dimension mh), degree-ideg Pade with
// scaling and squaring as ZGPADM (expokit.f:767-940); writes the first
// column to E.  Runs on the host: the matrix is at most 16 x 16, its result
// steers the step control there, and serial FP64 code is what a CPU core
// does best (one thread on the device pays the full FP64 pipe per warp).
constexpr int PADE_MAX = 16;
namespace {
struct Z {
  double x, y;
};
inline Z zmul(Z a, Z b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
inline Z zadd(Z a, Z b) { return {a.x + b.x, a.y + b.y}; }
inline Z zsub(Z a, Z b) { return {a.x - b.x, a.y - b.y}; }
inline Z zsc(Z a, double s) { return {a.x * s, a.y * s}; }
inline Z zdiv(Z a, Z b) {
  if (std::fabs(b.x) >= std::fabs(b.y)) {
    const double r = b.y / b.x, den = b.x + b.y * r;
    return {(a.x + a.y * r) / den, (a.y - a.x * r) / den};
  }
  const double r = b.x / b.y, den = b.x * r + b.y;
  return {(a.x * r + a.y) / den, (a.y * r - a.x) / den};
}
using ZM = Z[PADE_MAX][PADE_MAX];
inline void zmm(int mx, const ZM& A, const ZM& B, ZM& C, double sc) {
  for (int i = 0; i < mx; ++i)
    for (int j = 0; j < mx; ++j) {
      Z acc{0.0, 0.0};
      for (int k = 0; k < mx; ++k) acc = zadd(acc, zmul(A[i][k], B[k][j]));
      C[i][j] = zsc(acc, sc);
    }
}
}  // namespace

static void zgpadm_host(int ideg, int mx, double t, const double* Hh, int mh, double* Eout) {
  TTG_REQUIRE(mx >= 1 && mx <= PADE_MAX, "zgpadm: matrix too large");
  static thread_local ZM H, H2, P, Q, F, G;
  for (int i = 0; i < mx; ++i)
    for (int j = 0; j < mx; ++j) H[i][j] = {Hh[2 * (i + mh * j)], Hh[2 * (i + mh * j) + 1]};
  double hn = 0.0;
  for (int i = 0; i < mx; ++i) {
    double r = 0.0;
    for (int j = 0; j < mx; ++j) r += std::hypot(H[i][j].x, H[i][j].y);
    hn = std::max(hn, r);
  }
  hn = std::fabs(t * hn);
  TTG_REQUIRE(hn > 0.0, "zgpadm: null H in input");
  const int ns = std::max(0, (int)(std::log(hn) / std::log(2.0)) + 2);
  const double scale = t / (double)(1ll << ns), scale2 = scale * scale;
  double coef[PADE_MAX + 1];
  coef[0] = 1.0;
  {
    const int i1 = ideg + 1, j1 = 2 * ideg + 1;
    for (int k = 1; k <= ideg; ++k) coef[k] = coef[k - 1] * (double)(i1 - k) / (double)(k * (j1 - k));
  }
  zmm(mx, H, H, H2, scale2);
  for (int i = 0; i < mx; ++i)
    for (int j = 0; j < mx; ++j) {
      P[i][j] = {i == j ? coef[ideg - 1] : 0.0, 0.0};
      Q[i][j] = {i == j ? coef[ideg] : 0.0, 0.0};
    }
  // Horner: alternately Q <- Q H2 + c I, P <- P H2 + c I
  int iodd = 1;
  for (int k = ideg - 1; k > 0; --k) {
    ZM& U = iodd ? Q : P;
    zmm(mx, U, H2, F, 1.0);
    for (int i = 0; i < mx; ++i)
      for (int j = 0; j < mx; ++j) U[i][j] = i == j ? Z{F[i][j].x + coef[k - 1], F[i][j].y} : F[i][j];
    iodd = 1 - iodd;
  }
  {
    ZM& U = iodd ? Q : P;
    zmm(mx, U, H, F, scale);
    for (int i = 0; i < mx; ++i)
      for (int j = 0; j < mx; ++j) U[i][j] = F[i][j];
  }
  // Q <- Q - P; solve Q E = P (LU with partial pivoting, |re|+|im| pivots)
  for (int i = 0; i < mx; ++i)
    for (int j = 0; j < mx; ++j) Q[i][j] = zsub(Q[i][j], P[i][j]);
  int piv[PADE_MAX];
  for (int k = 0; k < mx; ++k) {
    int p = k;
    double best = std::fabs(Q[k][k].x) + std::fabs(Q[k][k].y);
    for (int i = k + 1; i < mx; ++i) {
      const double v = std::fabs(Q[i][k].x) + std::fabs(Q[i][k].y);
      if (v > best) { best = v; p = i; }
    }
    piv[k] = p;
    TTG_REQUIRE(best != 0.0, "zgpadm: the Pade denominator is singular");
    if (p != k)
      for (int j = 0; j < mx; ++j) std::swap(Q[k][j], Q[p][j]);
    for (int i = k + 1; i < mx; ++i) {
      Q[i][k] = zdiv(Q[i][k], Q[k][k]);
      for (int j = k + 1; j < mx; ++j) Q[i][j] = zsub(Q[i][j], zmul(Q[i][k], Q[k][j]));
    }
  }
  for (int c = 0; c < mx; ++c) {
    for (int k = 0; k < mx; ++k)
      if (piv[k] != k) std::swap(P[k][c], P[piv[k]][c]);
    for (int i = 0; i < mx; ++i)
      for (int k = 0; k < i; ++k) P[i][c] = zsub(P[i][c], zmul(Q[i][k], P[k][c]));
    for (int i = mx - 1; i >= 0; --i) {
      Z v = P[i][c];
      for (int k = i + 1; k < mx; ++k) v = zsub(v, zmul(Q[i][k], P[k][c]));
      P[i][c] = zdiv(v, Q[i][i]);
    }
  }
  // E = 2 E + I
  for (int i = 0; i < mx; ++i)
    for (int j = 0; j < mx; ++j) P[i][j] = i == j ? Z{2.0 * P[i][j].x + 1.0, 2.0 * P[i][j].y}
                                                  : zsc(P[i][j], 2.0);
  if (ns == 0 && iodd) {
    for (int i = 0; i < mx; ++i) { Eout[2 * i] = -P[i][0].x; Eout[2 * i + 1] = -P[i][0].y; }
    return;
  }
  ZM* cur = &P;
  ZM* nxt = &G;
  for (int k = 0; k < ns; ++k) {
    zmm(mx, *cur, *cur, *nxt, 1.0);
    std::swap(cur, nxt);
  }
  for (int i = 0; i < mx; ++i) { Eout[2 * i] = (*cur)[i][0].x; Eout[2 * i + 1] = (*cur)[i][0].y; }
}

// out = beta * V[:, :mx] E[:mx]   (complex gemv)
__global__ void zgemv_kernel(i64 n, int mx, const double2* V, const double2* E, double beta,
                             double2* out) {
  __shared__ double2 Es[PADE_MAX];
  if (threadIdx.x < mx) Es[threadIdx.x] = E[threadIdx.x];
  __syncthreads();
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int k = 0; k < mx; ++k) acc = cadd(acc, cmul(V[i + n * k], Es[k]));
    out[i] = cscale(acc, beta);
  }
}

__global__ void hset_kernel(double2* H, int mh, int m) {
  for (int e = threadIdx.x; e < mh * mh; e += blockDim.x) H[e] = make_double2(0.0, 0.0);
  __syncthreads();
  if (threadIdx.x == 0) H[(m + 1) + mh * m] = make_double2(1.0, 0.0);
}

static inline int fnint(double x) { return x >= 0 ? (int)std::floor(x + 0.5) : -(int)std::floor(-x + 0.5); }
static inline double round2(double x) {
  const double p1 = std::pow(10.0, fnint(std::log10(x) - std::sqrt(0.1)) - 1);
  return std::trunc(x / p1 + 0.55) * p1;
}

// ZGEXPV (expokit.f:2403-2793) on a normalised start vector v (device).
static void zgexpv_dev(ExpWork& w, i64 n, int m, double t, const double2* v, double2* out,
                       double tol, double anorm, const ZMatvecFn& mv, cudaStream_t s,
                       ExpStats* st) {
  const int ideg = 6, mxstep = st && st->mxstep > 0 ? st->mxstep : 500;
  const double delta = 1.2, gamma = 0.9, break_tol = 1.0e-7;
  const double eps = DBL_EPSILON;
  TTG_REQUIRE(m + 2 <= PADE_MAX, "zgexpv: Krylov order too large");
  if (tol <= eps) tol = std::sqrt(eps);
  const double sgn = t >= 0 ? 1.0 : -1.0;
  const double t_out = std::fabs(t);
  const int mh = m + 2;
  double* h = w.hbuf;
  auto sync = [&]() {
    TTG_CUDA(cudaStreamSynchronize(s));
    if (st) st->syncs++;
  };
  const int eb = eblocks(n);
  TTG_CUDA(cudaMemcpyAsync(out, v, sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
  znrm2_kernel<<<1, 1024, 0, s>>>(n, out, w.red);
  TTG_CHECK_LAUNCH();
  TTG_CUDA(cudaMemcpyAsync(h, w.red, sizeof(double), cudaMemcpyDeviceToHost, s));
  sync();
  double beta = h[0];
  double xm = 1.0 / m;
  double p2 = tol * std::pow((m + 1) / 2.72, m + 1) * std::sqrt(2.0 * 3.14 * (m + 1));
  double t_new = round2((1.0 / anorm) * std::pow(p2 / (4.0 * beta * anorm), xm));
  double t_now = 0.0;
  int nstep = 0;
  while (t_now < t_out) {
    ++nstep;
    double t_step = std::min(t_out - t_now, t_new);
    zscale_kernel<<<eb, 256, 0, s>>>(n, out, w.V, nullptr, 1.0 / beta);
    TTG_CHECK_LAUNCH();
    hset_kernel<<<1, 256, 0, s>>>(w.H, mh, m);
    TTG_CHECK_LAUNCH();
    TTG_CUDA(cudaMemsetAsync(w.ired, 0, sizeof(int), s));
    for (int j = 0; j < m; ++j) {
      mv(w.V + n * j, w.V + n * (j + 1), 1);
      mgs_step(w, n, j, mh, break_tol, s);
    }
    if (st) st->nmult += m;
    mv(w.V + n * m, w.tmp, 1);
    znrm2_kernel<<<1, 1024, 0, s>>>(n, w.tmp, w.red);
    TTG_CHECK_LAUNCH();
    // one read-back per Krylov step: ||A v_{m+1}||, the breakdown flag and H
    double* hH = h + 16;
    double* hE = h + 16 + 2 * PADE_MAX * PADE_MAX;
    TTG_CUDA(cudaMemcpyAsync(h, w.red, sizeof(double), cudaMemcpyDeviceToHost, s));
    TTG_CUDA(cudaMemcpyAsync(h + 1, w.ired, sizeof(int), cudaMemcpyDeviceToHost, s));
    TTG_CUDA(cudaMemcpyAsync(hH, w.H, sizeof(double2) * mh * mh, cudaMemcpyDeviceToHost, s));
    sync();
    const int brk = *(const int*)(h + 1);
    int k1 = 2, mbrkdwn = m;
    double avnorm = h[0];
    if (brk != 0) {
      k1 = 0;
      mbrkdwn = brk;
      t_step = t_out - t_now;
    } else if (st) {
      st->nmult += 1;
    }
    // H(m+2, m+1) = 1 was set by hset_kernel; the breakdown left later
    // columns untouched, as in the reference.
    double err_loc = tol;
    while (true) {
      const int mx = mbrkdwn + k1;
      zgpadm_host(ideg, mx, sgn * t_step, hH, mh, hE);
      if (k1 == 0) {
        err_loc = tol;
      } else {
        const double p1 = std::hypot(hE[2 * m], hE[2 * m + 1]) * beta;
        const double q2 = std::hypot(hE[2 * (m + 1)], hE[2 * (m + 1) + 1]) * beta * avnorm;
        if (p1 > 10.0 * q2) {
          err_loc = q2;
          xm = 1.0 / m;
        } else if (p1 > q2) {
          err_loc = (p1 * q2) / (p1 - q2);
          xm = 1.0 / m;
        } else {
          err_loc = p1;
          xm = 1.0 / (m - 1);
        }
      }
      if (k1 != 0 && err_loc > delta * t_step * tol) {
        t_step = round2(gamma * t_step * std::pow(t_step * tol / err_loc, xm));
        if (st) st->nreject++;
        continue;
      }
      break;
    }
    const int mx = mbrkdwn + std::max(0, k1 - 1);
    // hE is rewritten only after the next sync, when this copy has run
    TTG_CUDA(cudaMemcpyAsync(w.E, hE, sizeof(double2) * mx, cudaMemcpyHostToDevice, s));
    zgemv_kernel<<<eb, 256, 0, s>>>(n, mx, w.V, w.E, beta, out);
    TTG_CHECK_LAUNCH();
    znrm2_kernel<<<1, 1024, 0, s>>>(n, out, w.red);
    TTG_CHECK_LAUNCH();
    TTG_CUDA(cudaMemcpyAsync(h, w.red, sizeof(double), cudaMemcpyDeviceToHost, s));
    sync();
    beta = h[0];
    t_new = round2(gamma * t_step * std::pow(t_step * tol / err_loc, xm));
    t_now += t_step;
    if (nstep >= mxstep) break;
  }
  if (st) st->nstep += nstep;
  if (t_now < t_out) {
    // stopped at mxstep short of t: Expokit's iflag = 1, which zexp_mv prints
    // and tolerates (explib.f90:108-111)
    if (st) ++st->capped;
    if (st && st->strict)
      throw Error{TTG_ERR_NOCONV, "zexp_mv: Krylov exponential reached the step cap (" +
                                      std::to_string(mxstep) + " steps) before t"};
  }
}

__global__ void z1x1_kernel(const double2* v, const double2* a, double tau, double2* out) {
  // out = v * exp(a * tau)
  const double2 z = make_double2(a[0].x * tau, a[0].y * tau);
  double sn, cs;
  sincos(z.y, &sn, &cs);
  const double ex = exp(z.x);
  out[0] = cmul(v[0], make_double2(ex * cs, ex * sn));
}

__global__ void zone_kernel(double2* x) { x[0] = make_double2(1.0, 0.0); }

void zexp_mv_dev(ExpWork& w, i64 n, int m, double tau, const double2* v, double2* out, double tol,
                 double anorm, const ZMatvecFn& mv, cudaStream_t s, ExpStats* st) {
  const int m1 = (int)std::min<i64>(m, n);
  if (m1 == 1) {
    // zexp_mv, explib.f90:96-98: the 1x1 operator is its matvec of 1
    zone_kernel<<<1, 1, 0, s>>>(w.tmp);
    TTG_CHECK_LAUNCH();
    mv(w.tmp, w.tmp + 1, 1);
    z1x1_kernel<<<1, 1, 0, s>>>(v, w.tmp + 1, tau, out);
    TTG_CHECK_LAUNCH();
    return;
  }
  znrm2_kernel<<<1, 1024, 0, s>>>(n, v, w.red);
  TTG_CHECK_LAUNCH();
  TTG_CUDA(cudaMemcpyAsync(w.hbuf, w.red, sizeof(double), cudaMemcpyDeviceToHost, s));
  TTG_CUDA(cudaStreamSynchronize(s));
  const double nrm = w.hbuf[0];
  if (!(nrm > 0.0)) {
    TTG_CUDA(cudaMemsetAsync(out, 0, sizeof(double2) * n, s));
    return;
  }
  // vtmp = v / nrm (held in the last Krylov column, overwritten later)
  double2* vt = w.V + n * m;
  zscale_kernel<<<eblocks(n), 256, 0, s>>>(n, v, vt, nullptr, 1.0 / nrm);
  TTG_CHECK_LAUNCH();
  zgexpv_dev(w, n, m1, tau, vt, out, tol, anorm, mv, s, st);
  zscale_kernel<<<eblocks(n), 256, 0, s>>>(n, out, out, nullptr, nrm);
  TTG_CHECK_LAUNCH();
}

}  // namespace ttg
