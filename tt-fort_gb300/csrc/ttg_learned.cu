// Learned pointwise preconditioner for the local eigensolver.
//
// No counterpart in the reference: PRIMME's applyPreconditioner hook exists
// but tt_eigb leaves it unset (primme/primme.h:144-145, tt_eigb.f90:252-283),
// so the reference expands its Davidson basis with plain residuals.  Here a
// ReLU multilayer perceptron (default widths 3-512-512-512-1, FP32) maps
// per-entry features of the local problem to a correction h of the classical
// Davidson preconditioner:
//
//   q_i   = clip(s / (D_i - theta), +-100)     D = diag of the local operator,
//                                              s = max_i |D_i - theta|
//   t_i   = q_i (1 + h_i) r_i / s              (r itself where not finite)
//   feats = [(D_i - theta)/s, r_i sqrt(N)/||r||, q_i/100]
//
// With the last layer zero the network is exactly the classical diagonal
// preconditioner.  Training data are recorded by the sweeps themselves (the
// start Ritz block of every local problem and its converged block); the loss
// of one column is 1 - cos^2 between the expansion and the ideal correction,
// both projected off the start block, so it measures what Davidson can use.
// Training runs on the GPU with this file's forward/backward kernels, the
// FP32 GEMM of ttg_gemm.cu and Adam; the FP64 Davidson residual test remains
// the judge of every eigenpair.
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

constexpr int NFEAT = 3;
constexpr double QCLIP = 100.0;

inline int eb(i64 n) { return (int)std::max<i64>(1, std::min<i64>(8192, (n + 255) / 256)); }

// D(b1, j, b2) = sum_{a1,a2} Phi1(b1,b1,a1) A(a1,j,j,a2) Phi2(b2,a2,b2)
__global__ void local_diag_kernel(i64 rx1, i64 n, i64 rx2, int ra1, int ra2,
                                  const double* __restrict__ phi1, const double* __restrict__ A,
                                  const double* __restrict__ phi2, double* __restrict__ D) {
  const i64 N = rx1 * n * rx2;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < N; e += (i64)gridDim.x * blockDim.x) {
    const i64 b1 = e % rx1, j = (e / rx1) % n, b2 = e / (rx1 * n);
    double acc = 0.0;
    for (int a2 = 0; a2 < ra2; ++a2) {
      const double p2 = phi2[b2 + rx2 * (a2 + (i64)ra2 * b2)];
      double t = 0.0;
      for (int a1 = 0; a1 < ra1; ++a1)
        t = fma(phi1[b1 + rx1 * (b1 + rx1 * a1)], A[a1 + ra1 * (j + n * (j + n * a2))], t);
      acc = fma(t, p2, acc);
    }
    D[e] = acc;
  }
}

// per column q: s_q = max_i |D_i - theta_q| (1 if zero), rn_q = ||R_q|| (1 if zero)
__global__ void col_stats_kernel(i64 N, const double* __restrict__ D, const double* __restrict__ theta,
                                 const double* __restrict__ R, double* __restrict__ sv,
                                 double* __restrict__ rn) {
  __shared__ double smax[32], ssum[32];
  const int q = blockIdx.x;
  const double th = theta[q];
  double mx = 0.0, sm = 0.0;
  for (i64 i = threadIdx.x; i < N; i += blockDim.x) {
    mx = fmax(mx, fabs(D[i] - th));
    const double r = R[i + N * q];
    sm = fma(r, r, sm);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    sm += __shfl_xor_sync(0xffffffffu, sm, o);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { smax[w] = mx; ssum[w] = sm; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double m2 = 0.0, s2 = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { m2 = fmax(m2, smax[k]); s2 += ssum[k]; }
    sv[q] = m2 > 0.0 ? m2 : 1.0;
    rn[q] = s2 > 0.0 ? sqrt(s2) : 1.0;
  }
}

// features (P x 3 row-major, point p = i + N q) and the classical term base
__global__ void features_kernel(i64 N, int t, const double* __restrict__ D,
                                const double* __restrict__ theta, const double* __restrict__ R,
                                const double* __restrict__ sv, const double* __restrict__ rn,
                                float* __restrict__ F, double* __restrict__ base) {
  const double sq = sqrt((double)N);
  for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < N * t; p += (i64)gridDim.x * blockDim.x) {
    const int q = (int)(p / N);
    const i64 i = p % N;
    const double s = sv[q], dd = D[i] - theta[q], r = R[p];
    double qc = dd != 0.0 ? s / dd : QCLIP;
    qc = fmin(QCLIP, fmax(-QCLIP, qc));
    F[p * NFEAT + 0] = (float)(dd / s);
    F[p * NFEAT + 1] = (float)(r * sq / rn[q]);
    F[p * NFEAT + 2] = (float)(qc / QCLIP);
    base[p] = qc * r / s;
  }
}

__global__ void bias_act_kernel(i64 P, int n, float* __restrict__ Z, const float* __restrict__ b,
                                int relu) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < P * n; e += (i64)gridDim.x * blockDim.x) {
    float v = Z[e] + b[e % n];
    Z[e] = relu ? fmaxf(v, 0.f) : v;
  }
}

// t = base (1 + h), r where that is not finite
__global__ void prec_apply_kernel(i64 P, const double* __restrict__ base, const float* __restrict__ h,
                                  double* __restrict__ T) {
  for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < P; p += (i64)gridDim.x * blockDim.x) {
    const double v = base[p] * (1.0 + (double)h[p]);
    if (isfinite(v)) T[p] = v;
  }
}

__global__ void expand_kernel(i64 P, const double* __restrict__ base, const float* __restrict__ h,
                              double* __restrict__ u) {
  for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < P; p += (i64)gridDim.x * blockDim.x)
    u[p] = base[p] * (1.0 + (double)h[p]);
}

// per column: d[3q] = u.u, d[3q+1] = v.v, d[3q+2] = u.v  (one block per column)
__global__ void dot3_kernel(i64 N, const double* __restrict__ u, const double* __restrict__ v,
                            double* __restrict__ d) {
  __shared__ double sh[3][32];
  const int q = blockIdx.x;
  double a = 0.0, b = 0.0, c = 0.0;
  for (i64 i = threadIdx.x; i < N; i += blockDim.x) {
    const double x = u[i + N * q], y = v[i + N * q];
    a = fma(x, x, a); b = fma(y, y, b); c = fma(x, y, c);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { sh[0][w] = a; sh[1][w] = b; sh[2][w] = c; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0, y = 0, z = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { x += sh[0][k]; y += sh[1][k]; z += sh[2][k]; }
    d[3 * q] = x; d[3 * q + 1] = y; d[3 * q + 2] = z;
  }
}

// loss = mean_q (1 - uv^2/(uu vv)); g = dloss/du = -(2 uv/(uu vv t)) (v - (uv/uu) u)
__global__ void cos_grad_kernel(i64 N, int t, const double* __restrict__ u,
                                const double* __restrict__ v, const double* __restrict__ d,
                                double* __restrict__ g, double* __restrict__ loss) {
  for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < N * t; p += (i64)gridDim.x * blockDim.x) {
    const int q = (int)(p / N);
    const double uu = d[3 * q], vv = d[3 * q + 1], uv = d[3 * q + 2];
    double gv = 0.0;
    if (uu > 0.0 && vv > 0.0) gv = -(2.0 * uv / (uu * vv * t)) * (v[p] - (uv / uu) * u[p]);
    g[p] = gv;
    if (p == 0) {
      double L = 0.0;
      for (int k = 0; k < t; ++k) {
        const double a = d[3 * k], b = d[3 * k + 1], c = d[3 * k + 2];
        L += (a > 0.0 && b > 0.0) ? 1.0 - c * c / (a * b) : 0.0;
      }
      *loss = L / t;
    }
  }
}

// dh = g * base (float)
__global__ void head_grad_kernel(i64 P, const double* __restrict__ g, const double* __restrict__ base,
                                 float* __restrict__ dh) {
  for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < P; p += (i64)gridDim.x * blockDim.x)
    dh[p] = (float)(g[p] * base[p]);
}

__global__ void relu_mask_kernel(i64 n, float* __restrict__ dz, const float* __restrict__ a) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x)
    if (!(a[e] > 0.f)) dz[e] = 0.f;
}

// db[j] = sum_p dz[p, j]
__global__ void colsum_kernel(i64 P, int n, const float* __restrict__ dz, float* __restrict__ db) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const i64 p0 = (i64)blockIdx.y * 1024, p1 = std::min<i64>(P, p0 + 1024);
  float acc = 0.f;
  for (i64 p = p0; p < p1; ++p) acc += dz[p * n + j];
  atomicAdd(&db[j], acc);
}

__global__ void adam_kernel(i64 n, float* __restrict__ w, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, float lr, float b1,
                            float b2, float c1, float c2, float eps) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x) {
    const float gg = g[e];
    const float mm = b1 * m[e] + (1.f - b1) * gg;
    const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
    m[e] = mm;
    v[e] = vv;
    w[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  }
}

}  // namespace
}  // namespace ttg

// ---------------------------------------------------------------------------
// the network
// ---------------------------------------------------------------------------
struct ttg_mlp {
  ttg_ctx* ctx = nullptr;
  std::vector<int> dims;               // [NFEAT, width..., 1]
  std::vector<size_t> woff, boff;      // parameter offsets (floats)
  size_t nparams = 0;
  float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  long long adam_t = 0;
  // grow-only work buffers
  void* work = nullptr;
  size_t work_cap = 0;
  double last_loss = 0.0;
  // layer products: 1 = BF16 on the tensor cores (tcgen05, FP32 accumulate),
  // 0 = FP32 on the CUDA cores
  int bf16 = 1;
  void* tcws = nullptr;     // bf16 operand tiles and K-split partials (grow-only)
  size_t tcws_cap = 0;
  int* tcerr = nullptr;     // bounded-wait flag of the tensor-core products
};

namespace ttg {
namespace {

struct MlpWork {
  float* F;        // P x NFEAT
  double* base;    // P
  float* act;      // all layer outputs, P x dims[l+1] each
  float* dz;       // P x maxw
  float* dz2;      // P x maxw
  double* u;       // P
  double* gu;      // P
  double* C;       // 64 x 64 projection coefficients
  double* dots;    // 3 * 64
  double* loss;    // 1
  double* sv;      // 64
  double* rn;      // 64
};

size_t act_floats(const ttg_mlp* M, i64 P) {
  size_t a = 0;
  for (size_t l = 1; l < M->dims.size(); ++l) a += (size_t)P * M->dims[l];
  return a;
}
int max_width(const ttg_mlp* M) { return *std::max_element(M->dims.begin(), M->dims.end()); }

MlpWork mlp_work(ttg_mlp* M, i64 P, cudaStream_t s) {
  const size_t al = 256;
  auto up = [&](size_t b) { return (b + al - 1) / al * al; };
  const size_t mw = (size_t)max_width(M);
  size_t bytes = up(P * NFEAT * 4) + up(P * 8) + up(act_floats(M, P) * 4) + 2 * up(P * mw * 4) +
                 2 * up(P * 8) + up(64 * 64 * 8) + up(3 * 64 * 8) + up(8) + 2 * up(64 * 8);
  if (bytes > M->work_cap) {
    if (M->work) { cudaStreamSynchronize(s); cudaFree(M->work); M->work = nullptr; }
    TTG_CUDA(cudaMalloc(&M->work, bytes));
    M->work_cap = bytes;
  }
  char* p = (char*)M->work;
  MlpWork w;
  w.F = (float*)p; p += up(P * NFEAT * 4);
  w.base = (double*)p; p += up(P * 8);
  w.act = (float*)p; p += up(act_floats(M, P) * 4);
  w.dz = (float*)p; p += up(P * mw * 4);
  w.dz2 = (float*)p; p += up(P * mw * 4);
  w.u = (double*)p; p += up(P * 8);
  w.gu = (double*)p; p += up(P * 8);
  w.C = (double*)p; p += up(64 * 64 * 8);
  w.dots = (double*)p; p += up(3 * 64 * 8);
  w.loss = (double*)p; p += up(8);
  w.sv = (double*)p; p += up(64 * 8);
  w.rn = (double*)p; p += up(64 * 8);
  return w;
}

// c[m*scm + n*scn] = sum_k a[m*sam + k*sak] b[n*sbn + k*sbk] (FP32 in and
// out), on the tensor cores in BF16 or on the CUDA cores in FP32
void mlp_gemm(ttg_mlp* M, int Mm, int N, int K, const float* a, i64 sam, i64 sak, const float* b,
              i64 sbn, i64 sbk, float* c, i64 scm, i64 scn, cudaStream_t s) {
  if (M->bf16) {
    const size_t need = bf16_gemm_ws(Mm, N, K);
    if (need > M->tcws_cap) {
      if (M->tcws) { cudaStreamSynchronize(s); cudaFree(M->tcws); M->tcws = nullptr; }
      M->tcws_cap = 0;
      TTG_CUDA(cudaMalloc(&M->tcws, need));
      M->tcws_cap = need;
    }
    bf16_gemm(Mm, N, K, a, sam, sak, b, sbn, sbk, c, scm, scn, M->tcws, M->tcerr, s);
    return;
  }
  GemmF32 g;
  g.M = Mm; g.N = N; g.K = K;
  g.A = a; g.sAm = sam; g.sAk = sak;
  g.B = b; g.sBk = sbk; g.sBn = sbn;
  g.C = c; g.sCm = scm; g.sCn = scn;
  gemm_f32(g, s);
}

// forward over P points (features in F), layer outputs stored in act; returns h
const float* mlp_forward(ttg_mlp* M, i64 P, const float* F, float* act, cudaStream_t s) {
  const int L = (int)M->dims.size() - 1;
  const float* in = F;
  float* out = act;
  for (int l = 0; l < L; ++l) {
    const int k = M->dims[l], n = M->dims[l + 1];
    // out (P x n) = in (P x k) W (k x n), row-major; computed as
    // out^T[n_, p] = sum_k W[k, n_] in[p, k] so that the contiguous index of
    // the output (n_) lies on the tensor-core M side (coalesced stores)
    mlp_gemm(M, n, (int)P, k, M->w + M->woff[l], 1, n, in, k, 1, out, 1, n, s);
    bias_act_kernel<<<eb(P * n), 256, 0, s>>>(P, n, out, M->w + M->boff[l], l < L - 1);
    TTG_CHECK_LAUNCH();
    in = out;
    out += (size_t)P * n;
  }
  return in;
}

// backward from dh (P) into M->g (overwritten)
void mlp_backward(ttg_mlp* M, i64 P, const float* F, const float* act, float* dz, float* dz2,
                  cudaStream_t s) {
  const int L = (int)M->dims.size() - 1;
  // ain[l] = input of layer l: F for l = 0, the stored output of layer l-1 otherwise
  std::vector<const float*> ain(L);
  ain[0] = F;
  {
    const float* blk = act;
    for (int l = 1; l < L; ++l) { ain[l] = blk; blk += (size_t)P * M->dims[l]; }
  }
  TTG_CUDA(cudaMemsetAsync(M->g, 0, M->nparams * sizeof(float), s));
  float* cur = dz;     // gradient of layer l's pre-activation output (P x dims[l+1])
  float* nxt = dz2;
  for (int l = L - 1; l >= 0; --l) {
    const int k = M->dims[l], n = M->dims[l + 1];
    // dW (k x n) = in^T (k x P) cur (P x n): dW[kk, n_] = sum_p cur[p, n_] in[p, kk]
    mlp_gemm(M, n, k, (int)P, cur, 1, n, ain[l], 1, k, M->g + M->woff[l], 1, n, s);
    {
      dim3 grid((unsigned)ceil_div(n, 128), (unsigned)ceil_div(P, (i64)1024));
      colsum_kernel<<<grid, 128, 0, s>>>(P, n, cur, M->g + M->boff[l]);
      TTG_CHECK_LAUNCH();
    }
    if (l > 0) {
      // nxt (P x k) = cur (P x n) W^T (n x k): nxt^T[kk, p] = sum_n_ W[kk, n_] cur[p, n_]
      mlp_gemm(M, k, (int)P, n, M->w + M->woff[l], n, 1, cur, n, 1, nxt, 1, k, s);
      relu_mask_kernel<<<eb(P * k), 256, 0, s>>>(P * k, nxt, ain[l]);
      TTG_CHECK_LAUNCH();
      std::swap(cur, nxt);
    }
  }
}

// features of t residual columns R (N x t) with Ritz values theta (device)
void features(const double* D, i64 N, int t, const double* theta, const double* R, MlpWork& w,
              cudaStream_t s) {
  col_stats_kernel<<<t, 256, 0, s>>>(N, D, theta, R, w.sv, w.rn);
  TTG_CHECK_LAUNCH();
  features_kernel<<<eb(N * t), 256, 0, s>>>(N, t, D, theta, R, w.sv, w.rn, w.F, w.base);
  TTG_CHECK_LAUNCH();
}

// loss and gradient of one recorded problem (all device pointers):
// X (N x B) start Ritz block, R residuals, V ideal corrections projected off X
double problem_loss_grad(ttg_mlp* M, i64 N, int B, const double* D, const double* theta,
                         const double* X, const double* R, const double* V, cudaStream_t s,
                         bool want_loss) {
  const i64 P = N * B;
  MlpWork w = mlp_work(M, P, s);
  features(D, N, B, theta, R, w, s);
  const float* h = mlp_forward(M, P, w.F, w.act, s);
  expand_kernel<<<eb(P), 256, 0, s>>>(P, w.base, h, w.u);
  TTG_CHECK_LAUNCH();
  // u -= X (X^T u)
  gemm_tn_small(B, B, N, X, N, w.u, N, w.C, B, 1.0, 0.0, s);
  gemm_nn_small(N, B, B, X, N, w.C, B, w.u, N, -1.0, 1.0, s);
  dot3_kernel<<<B, 256, 0, s>>>(N, w.u, V, w.dots);
  TTG_CHECK_LAUNCH();
  cos_grad_kernel<<<eb(P), 256, 0, s>>>(N, B, w.u, V, w.dots, w.gu, w.loss);
  TTG_CHECK_LAUNCH();
  // the gradient with respect to the unprojected expansion: project again
  gemm_tn_small(B, B, N, X, N, w.gu, N, w.C, B, 1.0, 0.0, s);
  gemm_nn_small(N, B, B, X, N, w.C, B, w.gu, N, -1.0, 1.0, s);
  // dh into the last layer's gradient slot (P x 1)
  head_grad_kernel<<<eb(P), 256, 0, s>>>(P, w.gu, w.base, w.dz);
  TTG_CHECK_LAUNCH();
  mlp_backward(M, P, w.F, w.act, w.dz, w.dz2, s);
  double loss = 0.0;
  if (want_loss) {
    TTG_CUDA(cudaMemcpyAsync(&loss, w.loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    TTG_CUDA(cudaStreamSynchronize(s));
  }
  return loss;
}

void adam(ttg_mlp* M, float lr, cudaStream_t s) {
  M->adam_t += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)M->adam_t), c2 = 1.f - std::pow(b2, (float)M->adam_t);
  adam_kernel<<<eb(M->nparams), 256, 0, s>>>(M->nparams, M->w, M->g, M->m, M->v, lr, b1, b2, c1,
                                             c2, 1e-8f);
  TTG_CHECK_LAUNCH();
}

}  // namespace

// the Davidson preconditioner of one local problem (plain method)
PrecFn make_learned_prec(ttg_mlp* M, const LocalDims& L, const double* phi1, const double* A,
                         const double* phi2, double* D, cudaStream_t s) {
  local_diag_kernel<<<eb(L.xsize()), 256, 0, s>>>(L.rx1, L.m, L.rx2, (int)L.ra1, (int)L.ra2, phi1,
                                                 A, phi2, D);
  TTG_CHECK_LAUNCH();
  const i64 N = L.xsize();
  return [M, N, D, s](double* T, int t, const double*, int, const double* theta) {
    const i64 P = N * t;
    MlpWork w = mlp_work(M, P, s);
    features(D, N, t, theta, T, w, s);
    const float* h = mlp_forward(M, P, w.F, w.act, s);
    prec_apply_kernel<<<eb(P), 256, 0, s>>>(P, w.base, h, T);
    TTG_CHECK_LAUNCH();
  };
}

}  // namespace ttg

// ---------------------------------------------------------------------------
// recording training problems from the sweeps
// ---------------------------------------------------------------------------
namespace ttg {
namespace {

__global__ void ritz_residual_kernel(i64 N, int B, const double* __restrict__ AX,
                                     const double* __restrict__ X, const double* __restrict__ th,
                                     double* __restrict__ R) {
  for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < N * B; p += (i64)gridDim.x * blockDim.x)
    R[p] = AX[p] - th[p / N] * X[p];
}
__global__ void sub_kernel(i64 n, const double* __restrict__ a, double* __restrict__ y) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x)
    y[e] -= a[e];
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
};

}  // namespace

// Records one local problem: the start Ritz block of X0, its residuals, the
// diagonal of the operator and the converged block Xs rotated onto it.
void learned_record(ttg_ctx* ctx, const LocalDims& L, const double* phi1, const double* A,
                    const double* phi2, const double* X0, const double* Xs, int B,
                    const MatvecFn& mv, cudaStream_t s) {
  const i64 N = L.xsize();
  const size_t nb = (size_t)N * B;
  const size_t svs = svd_scratch(B, B) / sizeof(double) + 1;
  const size_t total = 6 * nb + N + 16 * (size_t)B * B + svs + 64;
  DevBuf buf;
  TTG_CUDA(cudaMalloc(&buf.p, total * sizeof(double)));
  double* V = (double*)buf.p;
  double* W = V + nb;
  double* Xr = W + nb;
  double* AXr = Xr + nb;
  double* R = AXr + nb;
  double* Y = R + nb;
  double* D = Y + nb;
  double* Rq = D + N;
  double* tau = Rq + (size_t)B * B;
  double* H = tau + (size_t)B * B;
  double* S = H + (size_t)B * B;
  double* th = S + (size_t)B * B;
  double* Mx = th + (size_t)B * B;
  double* U = Mx + (size_t)B * B;
  double* sg = U + (size_t)B * B;
  double* Vt = sg + (size_t)B * B;
  double* Q = Vt + (size_t)B * B;
  double* Cc = Q + (size_t)B * B;
  double* scr = Cc + (size_t)B * B;
  int* st = (int*)(scr + svs);
  TTG_CUDA(cudaMemcpyAsync(V, X0, nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
  qr_householder((int)N, B, V, Rq, tau, s);
  mv(V, W, B);
  gemm_tn_small(B, B, N, V, N, W, N, H, B, 1.0, 0.0, s);
  syev_jacobi(B, H, B, th, S, B, st, s);
  gemm_nn_small(N, B, B, V, N, S, B, Xr, N, 1.0, 0.0, s);
  gemm_nn_small(N, B, B, W, N, S, B, AXr, N, 1.0, 0.0, s);
  ritz_residual_kernel<<<eb(nb), 256, 0, s>>>(N, B, AXr, Xr, th, R);
  TTG_CHECK_LAUNCH();
  // Q = U Vt from the SVD of Xs^T Xr; Y = Xs Q - Xr, projected off Xr
  gemm_tn_small(B, B, N, Xs, N, Xr, N, Mx, B, 1.0, 0.0, s);
  svd_jacobi(B, B, Mx, U, sg, Vt, scr, st, s);
  {
    GemmF64 g;
    g.M = B; g.N = B; g.K = B;
    g.A = U; g.sAm = 1; g.sAk = B;
    g.B = Vt; g.sBk = 1; g.sBn = B;
    g.C = Q; g.sCm = 1; g.sCn = B;
    gemm_f64(g, s);
  }
  gemm_nn_small(N, B, B, Xs, N, Q, B, Y, N, 1.0, 0.0, s);
  sub_kernel<<<eb(nb), 256, 0, s>>>(nb, Xr, Y);
  TTG_CHECK_LAUNCH();
  gemm_tn_small(B, B, N, Xr, N, Y, N, Cc, B, 1.0, 0.0, s);
  gemm_nn_small(N, B, B, Xr, N, Cc, B, Y, N, -1.0, 1.0, s);
  local_diag_kernel<<<eb(N), 256, 0, s>>>(L.rx1, L.m, L.rx2, (int)L.ra1, (int)L.ra2, phi1, A, phi2, D);
  TTG_CHECK_LAUNCH();
  LearnedRecord rec;
  rec.N = N;
  rec.B = B;
  rec.D.resize(N); rec.theta.resize(B); rec.X.resize(nb); rec.R.resize(nb); rec.V.resize(nb);
  TTG_CUDA(cudaMemcpyAsync(rec.D.data(), D, N * sizeof(double), cudaMemcpyDeviceToHost, s));
  TTG_CUDA(cudaMemcpyAsync(rec.theta.data(), th, B * sizeof(double), cudaMemcpyDeviceToHost, s));
  TTG_CUDA(cudaMemcpyAsync(rec.X.data(), Xr, nb * sizeof(double), cudaMemcpyDeviceToHost, s));
  TTG_CUDA(cudaMemcpyAsync(rec.R.data(), R, nb * sizeof(double), cudaMemcpyDeviceToHost, s));
  TTG_CUDA(cudaMemcpyAsync(rec.V.data(), Y, nb * sizeof(double), cudaMemcpyDeviceToHost, s));
  TTG_CUDA(cudaStreamSynchronize(s));
  ctx->records.push_back(std::move(rec));
}

}  // namespace ttg

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace ttg;

extern "C" int ttg_mlp_create(ttg_ctx* c, ttg_int width, ttg_int depth, ttg_int seed, ttg_mlp** out) {
  if (!c || !out) return TTG_ERR_ARG;
  *out = nullptr;
  ttg_mlp* M = nullptr;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    TTG_REQUIRE(width >= 1 && width <= 4096 && depth >= 1 && depth <= 8, "mlp: bad width or depth");
    M = new ttg_mlp();
    M->ctx = c;
    M->dims.push_back(NFEAT);
    for (int l = 0; l < depth; ++l) M->dims.push_back((int)width);
    M->dims.push_back(1);
    size_t off = 0, nw = 0;
    for (size_t l = 0; l + 1 < M->dims.size(); ++l) {
      M->woff.push_back(off);
      off += (size_t)M->dims[l] * M->dims[l + 1];
      nw += (size_t)M->dims[l] * M->dims[l + 1];
      M->boff.push_back(off);
      off += M->dims[l + 1];
    }
    M->nparams = off;
    TTG_CUDA(cudaMalloc(&M->w, 4 * off * sizeof(float) + 256));
    M->g = M->w + off; M->m = M->g + off; M->v = M->m + off;
    M->tcerr = (int*)(M->v + off);
    TTG_CUDA(cudaMemset(M->w, 0, 4 * off * sizeof(float) + 256));
    // He-normal weights from the shared splitmix64 stream, zero biases, and a
    // zero output layer: the untrained network is the classical preconditioner
    std::vector<double> z(nw);
    sm_normals((unsigned long long)seed, (i64)nw, z.data());
    std::vector<float> h(off, 0.f);
    size_t zi = 0;
    for (size_t l = 0; l + 1 < M->dims.size(); ++l) {
      const size_t cnt = (size_t)M->dims[l] * M->dims[l + 1];
      const double sc = std::sqrt(2.0 / M->dims[l]);
      const bool last = l + 2 == M->dims.size();
      for (size_t e = 0; e < cnt; ++e) h[M->woff[l] + e] = last ? 0.f : (float)(z[zi + e] * sc);
      zi += cnt;
    }
    TTG_CUDA(cudaMemcpy(M->w, h.data(), off * sizeof(float), cudaMemcpyHostToDevice));
    *out = M;
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    if (M) { if (M->w) cudaFree(M->w); delete M; }
    return e.code;
  }
  return TTG_OK;
}

extern "C" int ttg_mlp_destroy(ttg_mlp* M) {
  if (!M) return TTG_ERR_ARG;
  cudaSetDevice(M->ctx->device);
  cudaStreamSynchronize(M->ctx->stream);
  if (M->ctx->learned == M) { M->ctx->learned = nullptr; M->ctx->learned_mode = 0; }
  if (M->w) cudaFree(M->w);
  if (M->work) cudaFree(M->work);
  if (M->tcws) cudaFree(M->tcws);
  delete M;
  return TTG_OK;
}

extern "C" int ttg_mlp_set_precision(ttg_mlp* M, int bf16) {
  if (!M) return TTG_ERR_ARG;
  M->bf16 = bf16 ? 1 : 0;
  return TTG_OK;
}

extern "C" int ttg_mlp_check(ttg_mlp* M) {
  if (!M) return TTG_ERR_ARG;
  try {
    TTG_CUDA(cudaSetDevice(M->ctx->device));
    int h = 0;
    TTG_CUDA(cudaMemcpyAsync(&h, M->tcerr, sizeof(int), cudaMemcpyDeviceToHost, M->ctx->stream));
    TTG_CUDA(cudaStreamSynchronize(M->ctx->stream));
    if (h) throw Error{TTG_ERR_CUDA, "mlp: tensor-core product gave up waiting (mbarrier)"};
  } catch (const ttg::Error& e) {
    M->ctx->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}

extern "C" ttg_int ttg_mlp_nparams(const ttg_mlp* M) { return M ? (ttg_int)M->nparams : -1; }

static int mlp_copy(ttg_mlp* M, float* host, const float* dev_src, float* dev_dst, ttg_int n) {
  if (!M || !host || n != (ttg_int)M->nparams) return TTG_ERR_ARG;
  ttg_ctx* c = M->ctx;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    TTG_CUDA(cudaStreamSynchronize(c->stream));
    if (dev_src) TTG_CUDA(cudaMemcpy(host, dev_src, n * sizeof(float), cudaMemcpyDeviceToHost));
    else TTG_CUDA(cudaMemcpy(dev_dst, host, n * sizeof(float), cudaMemcpyHostToDevice));
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}
extern "C" int ttg_mlp_get_params(ttg_mlp* M, float* host, ttg_int n) {
  return M ? mlp_copy(M, host, M->w, nullptr, n) : TTG_ERR_ARG;
}
extern "C" int ttg_mlp_set_params(ttg_mlp* M, const float* host, ttg_int n) {
  return M ? mlp_copy(M, const_cast<float*>(host), nullptr, M->w, n) : TTG_ERR_ARG;
}
extern "C" int ttg_mlp_get_grads(ttg_mlp* M, float* host, ttg_int n) {
  return M ? mlp_copy(M, host, M->g, nullptr, n) : TTG_ERR_ARG;
}

extern "C" int ttg_mlp_forward(ttg_mlp* M, ttg_int P, const float* F, float* h) {
  if (!M || !F || !h || P <= 0) return TTG_ERR_ARG;
  ttg_ctx* c = M->ctx;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    MlpWork w = mlp_work(M, P, c->stream);
    const float* out = mlp_forward(M, P, F, w.act, c->stream);
    TTG_CUDA(cudaMemcpyAsync(h, out, P * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}

extern "C" int ttg_mlp_loss_grad(ttg_mlp* M, ttg_int N, ttg_int B, const double* D,
                                 const double* theta, const double* X, const double* R,
                                 const double* V, double* loss) {
  if (!M || !D || !theta || !X || !R || !V || N <= 0 || B <= 0 || B > 64) return TTG_ERR_ARG;
  ttg_ctx* c = M->ctx;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    const double L = problem_loss_grad(M, N, (int)B, D, theta, X, R, V, c->stream, true);
    if (loss) *loss = L;
    M->last_loss = L;
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}

extern "C" int ttg_mlp_adam_step(ttg_mlp* M, double lr) {
  if (!M || !(lr > 0)) return TTG_ERR_ARG;
  ttg_ctx* c = M->ctx;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    adam(M, (float)lr, c->stream);
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}

extern "C" int ttg_set_learned(ttg_ctx* c, ttg_mlp* M, int mode) {
  if (!c || mode < 0 || mode > 3 || ((mode & 1) && !M)) return TTG_ERR_ARG;
  c->learned = M;
  c->learned_mode = mode;
  return TTG_OK;
}

extern "C" int ttg_record_count(const ttg_ctx* c, ttg_int* nprob, ttg_int* npoints) {
  if (!c) return TTG_ERR_ARG;
  ttg_int np = 0;
  for (const auto& r : c->records) np += r.N * r.B;
  if (nprob) *nprob = (ttg_int)c->records.size();
  if (npoints) *npoints = np;
  return TTG_OK;
}

extern "C" int ttg_record_clear(ttg_ctx* c) {
  if (!c) return TTG_ERR_ARG;
  c->records.clear();
  return TTG_OK;
}

// Adam over the recorded problems of `rec` (one problem per step, picked by a
// splitmix64 stream); loss_first / loss_last = mean loss over every recorded
// problem before and after.  When training did not lower the mean loss the
// parameters before training are restored (the classical preconditioner
// judges the network).
extern "C" int ttg_mlp_train_recorded(ttg_mlp* M, const ttg_ctx* rec, ttg_int steps, double lr,
                                      ttg_int seed, double* loss_first, double* loss_last) {
  if (!M || !rec || steps < 0 || !(lr > 0)) return TTG_ERR_ARG;
  ttg_ctx* c = M->ctx;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    TTG_REQUIRE(!rec->records.empty(), "mlp: no recorded problems");
    cudaStream_t s = c->stream;
    i64 nmax = 0;
    int bmax = 0;
    for (const auto& r : rec->records) { nmax = std::max(nmax, r.N); bmax = std::max(bmax, r.B); }
    TTG_REQUIRE(bmax <= 64, "mlp: block too wide");
    DevBuf buf;
    const size_t nb = (size_t)nmax * bmax;
    TTG_CUDA(cudaMalloc(&buf.p, (3 * nb + nmax + 64) * sizeof(double)));
    double* X = (double*)buf.p;
    double* R = X + nb;
    double* V = R + nb;
    double* D = V + nb;
    double* th = D + nmax;
    auto upload = [&](const LearnedRecord& r) {
      const size_t n = (size_t)r.N * r.B;
      TTG_CUDA(cudaMemcpyAsync(X, r.X.data(), n * 8, cudaMemcpyHostToDevice, s));
      TTG_CUDA(cudaMemcpyAsync(R, r.R.data(), n * 8, cudaMemcpyHostToDevice, s));
      TTG_CUDA(cudaMemcpyAsync(V, r.V.data(), n * 8, cudaMemcpyHostToDevice, s));
      TTG_CUDA(cudaMemcpyAsync(D, r.D.data(), r.N * 8, cudaMemcpyHostToDevice, s));
      TTG_CUDA(cudaMemcpyAsync(th, r.theta.data(), r.B * 8, cudaMemcpyHostToDevice, s));
    };
    auto mean_loss = [&]() {
      double acc = 0.0;
      for (const auto& r : rec->records) {
        upload(r);
        acc += problem_loss_grad(M, r.N, r.B, D, th, X, R, V, s, true);
      }
      return acc / rec->records.size();
    };
    std::vector<float> w0(M->nparams);
    TTG_CUDA(cudaStreamSynchronize(s));
    TTG_CUDA(cudaMemcpy(w0.data(), M->w, M->nparams * sizeof(float), cudaMemcpyDeviceToHost));
    const double l0 = mean_loss();
    unsigned long long st = (unsigned long long)seed * 0x9E3779B97F4A7C15ull + 1;
    for (ttg_int it = 0; it < steps; ++it) {
      st += 0x9E3779B97F4A7C15ull;
      unsigned long long z = st;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      z ^= z >> 31;
      const LearnedRecord& r = rec->records[z % rec->records.size()];
      upload(r);
      problem_loss_grad(M, r.N, r.B, D, th, X, R, V, s, false);
      adam(M, (float)lr, s);
    }
    const double l1 = mean_loss();
    if (!(l1 < l0)) {
      TTG_CUDA(cudaStreamSynchronize(s));
      TTG_CUDA(cudaMemcpy(M->w, w0.data(), M->nparams * sizeof(float), cudaMemcpyHostToDevice));
    }
    if (loss_first) *loss_first = l0;
    if (loss_last) *loss_last = l1;
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}
