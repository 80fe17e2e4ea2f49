// Block-Jacobi preconditioners of the local AMEn system: djac_gen
// (tt_linalg.f90:363-494) and djac_apply (tt_linalg.f90:497-531), the
// prec = 'c' | 'l' | 'r' options of tt_amen_solve (tt_adapt_als.f90:746-779).
//
// Each keeps part of the local operator
//   B[(c1,i,c2),(b1,j,b2)] = sum Phi1[c1,b1,a1] A[a1,i,j,a2] Phi2[b2,a2,c2]
// and inverts it block by block:
//   'c'  diagonals of Phi1 and Phi2: an n x n block per (b1, b2), stored
//        (n, n, rx2, rx1);
//   'l'  all of Phi1, diagonal of Phi2: an (rx1 n)^2 block per b2 with rows
//        (c1, i) and columns (b1, j), stored (rx1 n, rx1 n, rx2);
//   'r'  diagonal of Phi1, all of Phi2: an (n rx2)^2 block per b1 with rows
//        (i, c2) and columns (j, b2), stored (n rx2, n rx2, rx1).
// The blocks are assembled with the reference's GEMM order (FP64 GEMMs and
// the same dtransp / dperm1324 index maps, without the copies), then inverted
// by LU with partial pivoting against the identity (dgesv), one CTA per block:
// in shared memory up to k = 112, in a global work array above.  Applying
// the preconditioner is one batched block matrix-vector product.
#include "ttg_common.cuh"

namespace ttg {
namespace {

constexpr int INV_NT = 256;
constexpr int INV_SMEM_K = 112;   // 2 k^2 doubles <= 200 KB

// d1[b + rx1 a1] = Phi1[b, b, a1];  d2[b + rx2 a2] = Phi2[b, a2, b]
__global__ void jac_diags_kernel(i64 rx1, i64 ra1, i64 rx2, i64 ra2, const double* __restrict__ phi1,
                                 const double* __restrict__ phi2, double* __restrict__ d1,
                                 double* __restrict__ d2) {
  const i64 n1 = rx1 * ra1, n2 = rx2 * ra2;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n1 + n2; e += (i64)gridDim.x * blockDim.x) {
    if (e < n1) {
      const i64 b = e % rx1, a = e / rx1;
      d1[e] = phi1[b + rx1 * (b + rx1 * a)];
    } else {
      const i64 f = e - n1, b = f % rx2, a = f / rx2;
      d2[f] = phi2[b + rx2 * (a + ra2 * b)];
    }
  }
}

// B(n1, n3, n2, n4) = A(n1, n2, n3, n4)   (dperm1324, tt_linalg.f90:101-120)
__global__ void jac_perm1324_kernel(i64 n1, i64 n2, i64 n3, i64 n4, const double* __restrict__ A,
                                    double* __restrict__ B) {
  const i64 tot = n1 * n2 * n3 * n4;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    const i64 i1 = e % n1, i2 = (e / n1) % n2, i3 = (e / (n1 * n2)) % n3, i4 = e / (n1 * n2 * n3);
    B[i1 + n1 * (i3 + n3 * (i2 + n2 * i4))] = A[e];
  }
}

// Inverse of each k x k block of M (column-major, back to back) into Minv:
// LU with partial pivoting (the first row of largest |.| as idamax), row
// interchanges over whole rows as dgetf2, then L U X = P I column by column.
// SM: LU and X in shared memory; else LU in work (k^2 per block), X in Minv.
template <bool SM>
__global__ void __launch_bounds__(INV_NT) inv_blocks_kernel(int k, const double* __restrict__ M,
                                                             double* __restrict__ Minv,
                                                             double* __restrict__ work) {
  extern __shared__ __align__(16) double inv_dyn[];
  __shared__ double rv[INV_NT / 32];
  __shared__ int ri[INV_NT / 32];
  __shared__ int s_piv;
  const i64 kk = (i64)k * k;
  const i64 b = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  double* LU = SM ? inv_dyn : work + b * kk;
  double* X = SM ? inv_dyn + kk : Minv + b * kk;
  for (i64 e = tid; e < kk; e += INV_NT) {
    LU[e] = M[b * kk + e];
    X[e] = (e % k == e / k) ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int p = 0; p < k; ++p) {
    // pivot: first row r >= p of largest |LU[r, p]|
    double best = -1.0;
    int bi = k;
    for (int r = p + tid; r < k; r += INV_NT) {
      const double v = fabs(LU[r + (i64)k * p]);
      if (v > best) { best = v; bi = r; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) { rv[wid] = best; ri[wid] = bi; }
    __syncthreads();
    if (tid == 0) {
      double bb = rv[0];
      int ii = ri[0];
      for (int w = 1; w < INV_NT / 32; ++w)
        if (rv[w] > bb || (rv[w] == bb && ri[w] < ii)) { bb = rv[w]; ii = ri[w]; }
      s_piv = ii < k ? ii : p;
    }
    __syncthreads();
    const int piv = s_piv;
    if (piv != p) {
      for (int c = tid; c < k; c += INV_NT) {
        const double t = LU[p + (i64)k * c];
        LU[p + (i64)k * c] = LU[piv + (i64)k * c];
        LU[piv + (i64)k * c] = t;
        const double u = X[p + (i64)k * c];
        X[p + (i64)k * c] = X[piv + (i64)k * c];
        X[piv + (i64)k * c] = u;
      }
      __syncthreads();
    }
    const double d = LU[p + (i64)k * p];
    for (int r = p + 1 + tid; r < k; r += INV_NT) LU[r + (i64)k * p] /= d;
    __syncthreads();
    const int w = k - p - 1;
    for (i64 e = tid; e < (i64)w * w; e += INV_NT) {
      const int r = p + 1 + (int)(e % w), c = p + 1 + (int)(e / w);
      LU[r + (i64)k * c] -= LU[r + (i64)k * p] * LU[p + (i64)k * c];
    }
    __syncthreads();
  }
  // forward (unit L) and backward (U) substitution, one column of X per thread
  for (int c = tid; c < k; c += INV_NT) {
    double* x = X + (i64)k * c;
    for (int i = 1; i < k; ++i) {
      double v = x[i];
      for (int j = 0; j < i; ++j) v -= LU[i + (i64)k * j] * x[j];
      x[i] = v;
    }
    for (int i = k - 1; i >= 0; --i) {
      double v = x[i];
      for (int j = i + 1; j < k; ++j) v -= LU[i + (i64)k * j] * x[j];
      x[i] = v / LU[i + (i64)k * i];
    }
  }
  if (SM) {
    __syncthreads();
    for (i64 e = tid; e < kk; e += INV_NT) Minv[b * kk + e] = X[e];
  }
}

// y_v[base(b) + st r] = sum_c J_b[r, c] x_v[base(b) + st c], base(b) =
// (b / q) s1 + (b % q) s2; one thread per (r, b, v).
__global__ void jac_apply_kernel(int k, i64 nb, const double* __restrict__ J, i64 q, i64 s1, i64 s2,
                                 i64 st, const double* __restrict__ x, double* __restrict__ y,
                                 int nvec, i64 vstride) {
  const i64 tot = (i64)k * nb * nvec;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    const int r = (int)(e % k);
    const i64 b = (e / k) % nb, v = e / (k * nb);
    const i64 base = (b / q) * s1 + (b % q) * s2 + v * vstride;
    const double* Jb = J + b * (i64)k * k + r;
    double acc = 0.0;
    for (int c = 0; c < k; ++c) acc = fma(Jb[(i64)k * c], x[base + st * c], acc);
    y[base + st * r] = acc;
  }
}

inline int ebj(i64 n) { return (int)std::max<i64>(1, std::min<i64>(8192, (n + 255) / 256)); }

struct JacShape {
  i64 k;     // block size
  i64 nb;    // number of blocks
};

JacShape jac_shape(char p, i64 rx1, i64 n, i64 rx2) {
  switch (p) {
    case 'c': return {n, rx1 * rx2};
    case 'l': return {rx1 * n, rx2};
    default: return {n * rx2, rx1};
  }
}

}  // namespace

char jac_type(char p) {
  if (p == 'c' || p == 'C') return 'c';
  if (p == 'l' || p == 'L') return 'l';
  if (p == 'r' || p == 'R') return 'r';
  return 0;
}

constexpr i64 JAC_K_MAX = 4096;

i64 jac_size(char p, i64 rx1, i64 n, i64 rx2) {
  const JacShape sh = jac_shape(jac_type(p), rx1, n, rx2);
  return sh.k * sh.k * sh.nb;
}

// scratch doubles of jac_gen_f64: d1, d2, Phi2^T, T, W, W2 (and the LU work
// array when the blocks do not fit in shared memory)
i64 jac_gen_scratch(char p, i64 rx1, i64 n, i64 rx2, i64 ra1, i64 ra2) {
  p = jac_type(p);
  const JacShape sh = jac_shape(p, rx1, n, rx2);
  const i64 W = sh.k * sh.k * sh.nb;
  const i64 T = (p == 'l' ? rx1 * rx1 : rx1) * n * n * ra2;
  const i64 small = rx1 * ra1 + rx2 * ra2 + rx2 * rx2 * ra2 + 64;
  return small + T + W + std::max(W, T) + (sh.k > INV_SMEM_K ? W : 0) + 6 * 32;
}

void jac_gen_f64(char p, i64 rx1, i64 n, i64 rx2, i64 ra1, i64 ra2, const double* phi1,
                 const double* A, const double* phi2, double* jacs, double* scr, cudaStream_t s) {
  p = jac_type(p);
  TTG_REQUIRE(p, "djac_gen: prec must be 'c', 'l' or 'r'");
  const JacShape sh = jac_shape(p, rx1, n, rx2);
  TTG_REQUIRE(sh.k <= JAC_K_MAX, "djac_gen: preconditioner block larger than 4096");
  auto al = [](i64 c) { return (c + 31) & ~i64(31); };
  double* d1 = scr;
  double* d2 = d1 + al(rx1 * ra1);
  double* p2t = d2 + al(rx2 * ra2);
  double* T = p2t + al(rx2 * rx2 * ra2);
  double* W = T + al((p == 'l' ? rx1 * rx1 : rx1) * n * n * ra2);
  const i64 Wn = sh.k * sh.k * sh.nb;
  double* W2 = W + al(Wn);   // also the dperm1324 output of T ('l')
  double* LUw = W2 + al(std::max(Wn, (p == 'l' ? rx1 * rx1 : rx1) * n * n * ra2));
  auto gemm = [&](int M, int N, int K, const double* Am, i64 sAm, i64 sAk, const double* Bm,
                  i64 sBk, i64 sBn, double* C, i64 sCm, i64 sCn) {
    GemmF64 g;
    g.M = M; g.N = N; g.K = K;
    g.A = Am; g.sAm = sAm; g.sAk = sAk;
    g.B = Bm; g.sBk = sBk; g.sBn = sBn;
    g.C = C; g.sCm = sCm; g.sCn = sCn;
    gemm_f64(g, s);
  };
  jac_diags_kernel<<<ebj(rx1 * ra1 + rx2 * ra2), 256, 0, s>>>(rx1, ra1, rx2, ra2, phi1, phi2, d1, d2);
  TTG_CHECK_LAUNCH();
  const double* blocks = nullptr;
  if (p == 'c') {
    // T[b1, (i,j,a2)] = sum_a1 d1[b1,a1] A[a1,(i,j,a2)]
    gemm((int)rx1, (int)(n * n * ra2), (int)ra1, d1, 1, rx1, A, 1, ra1, T, 1, rx1);
    // W[(b1,i,j), b2] = sum_a2 T[(b1,i,j), a2] d2[b2, a2]
    gemm((int)(rx1 * n * n), (int)rx2, (int)ra2, T, 1, rx1 * n * n, d2, rx2, 1, W, 1, rx1 * n * n);
    // blocks [(i,j,b2), b1]
    transpose_f64(rx1, n * n * rx2, W, W2, s);
    blocks = W2;
  } else if (p == 'l') {
    // T[(c1,b1), (i,j,a2)] = sum_a1 Phi1[c1,b1,a1] A[a1,(i,j,a2)]
    gemm((int)(rx1 * rx1), (int)(n * n * ra2), (int)ra1, phi1, 1, rx1 * rx1, A, 1, ra1, T, 1,
         rx1 * rx1);
    // [c1, i, b1, (j,a2)]
    jac_perm1324_kernel<<<ebj(rx1 * rx1 * n * n * ra2), 256, 0, s>>>(rx1, rx1, n, n * ra2, T, W2);
    TTG_CHECK_LAUNCH();
    // W[(c1,i,b1,j), b2] = sum_a2 W2[(c1,i,b1,j), a2] d2[b2, a2]
    const i64 kk = rx1 * n * rx1 * n;
    gemm((int)kk, (int)rx2, (int)ra2, W2, 1, kk, d2, rx2, 1, W, 1, kk);
    blocks = W;
  } else {
    // Phi2^T: [c2, (b2,a2)]
    transpose_f64(rx2 * ra2, rx2, phi2, p2t, s);
    gemm((int)rx1, (int)(n * n * ra2), (int)ra1, d1, 1, rx1, A, 1, ra1, T, 1, rx1);
    // W[(b1,i,j), (c2,b2)] = sum_a2 T[(b1,i,j), a2] Phi2[b2, a2, c2]
    gemm((int)(rx1 * n * n), (int)(rx2 * rx2), (int)ra2, T, 1, rx1 * n * n, p2t, rx2 * rx2, 1, W,
         1, rx1 * n * n);
    // [(b1,i), c2, j, b2], then [(i,c2,j,b2), b1]
    jac_perm1324_kernel<<<ebj(rx1 * n * n * rx2 * rx2), 256, 0, s>>>(rx1 * n, n, rx2, rx2, W, W2);
    TTG_CHECK_LAUNCH();
    transpose_f64(rx1, n * rx2 * n * rx2, W2, W, s);
    blocks = W;
  }
  TTG_REQUIRE(sh.nb < (1ll << 31), "djac_gen: too many blocks");
  if (sh.k <= INV_SMEM_K) {
    const size_t bytes = 2 * (size_t)sh.k * sh.k * sizeof(double);
    static const bool attr_ok = cudaFuncSetAttribute(inv_blocks_kernel<true>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)(2 * INV_SMEM_K * INV_SMEM_K * sizeof(double))) ==
                                cudaSuccess;
    TTG_REQUIRE(attr_ok, "djac_gen: shared memory attribute refused");
    inv_blocks_kernel<true><<<(unsigned)sh.nb, INV_NT, bytes, s>>>((int)sh.k, blocks, jacs, nullptr);
  } else {
    inv_blocks_kernel<false><<<(unsigned)sh.nb, INV_NT, 0, s>>>((int)sh.k, blocks, jacs, LUw);
  }
  TTG_CHECK_LAUNCH();
}

void jac_apply_f64(char p, i64 rx1, i64 n, i64 rx2, const double* jacs, const double* x,
                   double* y, int nvec, cudaStream_t s) {
  p = jac_type(p);
  TTG_REQUIRE(p, "djac_apply: prec must be 'c', 'l' or 'r'");
  TTG_REQUIRE(x != y, "djac_apply: x and y must not overlap");
  const JacShape sh = jac_shape(p, rx1, n, rx2);
  TTG_REQUIRE(sh.k <= JAC_K_MAX, "djac_apply: preconditioner block larger than 4096");
  const i64 N = rx1 * n * rx2;
  i64 q, s1, s2, st;
  if (p == 'c') {          // block b2 + rx2 b1: x[b1 + rx1 (j + n b2)]
    q = rx2; s1 = 1; s2 = rx1 * n; st = rx1;
  } else if (p == 'l') {   // block b2: x[(b1,j) + rx1 n b2]
    q = 1; s1 = rx1 * n; s2 = 0; st = 1;
  } else {                 // block b1: x[b1 + rx1 (j + n b2)]
    q = 1; s1 = 1; s2 = 0; st = rx1;
  }
  jac_apply_kernel<<<ebj(sh.k * sh.nb * nvec), 256, 0, s>>>((int)sh.k, sh.nb, jacs, q, s1, s2, st,
                                                                   x, y, nvec, N);
  TTG_CHECK_LAUNCH();
}

}  // namespace ttg

using namespace ttg;

extern "C" ttg_int ttg_djac_size(char ptype, ttg_int rx1, ttg_int n, ttg_int rx2) {
  if (!jac_type(ptype) || rx1 <= 0 || n <= 0 || rx2 <= 0) return 0;
  return jac_size(ptype, rx1, n, rx2);
}

extern "C" int ttg_djac_gen(ttg_ctx* c, char ptype, ttg_int rx1, ttg_int n, ttg_int rx2,
                            ttg_int ra1, ttg_int ra2, const double* phi1, const double* A,
                            const double* phi2, double* jacs) {
  if (!c) return TTG_ERR_ARG;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    TTG_REQUIRE(jac_type(ptype), "djac_gen: prec must be 'c', 'l' or 'r'");
    TTG_REQUIRE(rx1 > 0 && n > 0 && rx2 > 0 && ra1 > 0 && ra2 > 0, "all sizes must be positive");
    TTG_REQUIRE(phi1 && A && phi2 && jacs, "null pointer");
    const size_t bytes = (size_t)jac_gen_scratch(ptype, rx1, n, rx2, ra1, ra2) * sizeof(double);
    c->ws.reset();
    c->ws.reserve(bytes);
    double* scr = (double*)c->ws.take(bytes);
    jac_gen_f64(ptype, rx1, n, rx2, ra1, ra2, phi1, A, phi2, jacs, scr, c->stream);
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}

extern "C" int ttg_djac_apply(ttg_ctx* c, char ptype, ttg_int rx1, ttg_int n, ttg_int rx2,
                              const double* jacs, const double* x, double* y) {
  if (!c) return TTG_ERR_ARG;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    TTG_REQUIRE(jac_type(ptype), "djac_apply: prec must be 'c', 'l' or 'r'");
    TTG_REQUIRE(rx1 > 0 && n > 0 && rx2 > 0, "all sizes must be positive");
    TTG_REQUIRE(jacs && x && y, "null pointer");
    const double* src = x;
    if (x == y) {   // the reference allows y == x (through its work array)
      const size_t bytes = (size_t)(rx1 * n * rx2) * sizeof(double);
      c->ws.reset();
      c->ws.reserve(bytes);
      double* tmp = (double*)c->ws.take(bytes);
      TTG_CUDA(cudaMemcpyAsync(tmp, x, bytes, cudaMemcpyDeviceToDevice, c->stream));
      src = tmp;
    }
    jac_apply_f64(ptype, rx1, n, rx2, jacs, src, y, 1, c->stream);
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}
