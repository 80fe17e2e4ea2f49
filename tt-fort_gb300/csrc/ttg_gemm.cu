// FP64 / complex128 strided batched GEMM for the plain (FP64) sweep path.
//
// One kernel template covers every dgemm/zgemm call site of the reference's
// hot path (ttals.f90:20,24,29,161-169,215-223; tt_eigb.f90:208,348,384;
// tt_ksl.f90:586,614; PRIMME's tall-skinny V'W / V*S products).  Operands are
// addressed through explicit (row, column) strides, so the reference's
// dtransp/ztransp passes (ttals.f90:22,26) fold into the index arithmetic
// instead of running as separate kernels.  A K-split mode serves the
// tall-skinny reductions (K = local problem size, M,N <= 128): the K-chunks of
// one output tile run as the CTAs of one thread block cluster and their
// partial tiles are added in rank order through distributed shared memory, so
// results are bit-reproducible (no atomics).
//
// Tiles: 256 threads, BK = 16, register-prefetched global loads, shared
// memory staged epilogue so that stores are coalesced along whichever output
// stride is unit.
#include "ttg_common.cuh"

namespace ttg {
namespace {

template <class T> struct Ops;
template <> struct Ops<float> {
  static __device__ __forceinline__ float zero() { return 0.f; }
  static __device__ __forceinline__ float fma(float a, float b, float c) { return fmaf(a, b, c); }
  static __device__ __forceinline__ float conj(float a) { return a; }
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
  static __device__ __forceinline__ float add(float a, float b) { return a + b; }
  static __device__ __forceinline__ bool is_zero(float a) { return a == 0.f; }
};
template <> struct Ops<double> {
  static __device__ __forceinline__ double zero() { return 0.0; }
  static __device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
  static __device__ __forceinline__ double conj(double a) { return a; }
  static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __device__ __forceinline__ bool is_zero(double a) { return a == 0.0; }
};
template <> struct Ops<double2> {
  static __device__ __forceinline__ double2 zero() { return make_double2(0.0, 0.0); }
  static __device__ __forceinline__ double2 fma(double2 a, double2 b, double2 c) {
    c.x = ::fma(a.x, b.x, c.x);
    c.x = ::fma(-a.y, b.y, c.x);
    c.y = ::fma(a.x, b.y, c.y);
    c.y = ::fma(a.y, b.x, c.y);
    return c;
  }
  static __device__ __forceinline__ double2 conj(double2 a) { return make_double2(a.x, -a.y); }
  static __device__ __forceinline__ double2 mul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
  }
  static __device__ __forceinline__ double2 add(double2 a, double2 b) {
    return make_double2(a.x + b.x, a.y + b.y);
  }
  static __device__ __forceinline__ bool is_zero(double2 a) { return a.x == 0.0 && a.y == 0.0; }
};

template <class T> struct Args {
  int M, N, K;
  const T* A; i64 sAm, sAk;
  const T* B; i64 sBk, sBn;
  T* C; i64 sCm, sCn;
  T alpha, beta;
  int nb1;
  i64 bA1, bA2, bB1, bB2, bC1, bC2;
  int splitk, kchunk;
  bool conjA, conjB;
};

constexpr int BK = 16;
constexpr int NT = 256;

template <class T, int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__(NT) gemm_kernel(Args<T> g) {
  using O = Ops<T>;
  constexpr int TX = BN / TN;          // threads along n
  constexpr int TY = BM / TM;          // threads along m
  static_assert(TX * TY == NT, "tile/thread mismatch");
  constexpr int A_PER = BM * BK / NT;
  constexpr int B_PER = BN * BK / NT;
  constexpr int SMEM_AB = BK * (BM + 1) + BK * (BN + 1);
  constexpr int SMEM_C = BN * (BM + 1);
  constexpr int SMEM = SMEM_AB > SMEM_C ? SMEM_AB : SMEM_C;
  __shared__ T smem[SMEM];
  T* As = smem;                       // [BK][BM+1]
  T* Bs = smem + BK * (BM + 1);       // [BK][BN+1]

  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int zb = blockIdx.z / g.splitk, ks = blockIdx.z % g.splitk;
  const int b1 = zb % g.nb1, b2 = zb / g.nb1;
  const T* A = g.A + b1 * g.bA1 + b2 * g.bA2;
  const T* Bp = g.B + b1 * g.bB1 + b2 * g.bB2;
  T* C = g.C + b1 * g.bC1 + b2 * g.bC2;
  const int kbeg = ks * g.kchunk;
  const int kend = min(g.K, kbeg + g.kchunk);

  const bool a_mfast = (g.sAm == 1);
  const bool b_kfast = (g.sBk == 1);

  T ra[A_PER], rb[B_PER];
  auto load = [&](int k0) {
#pragma unroll
    for (int r = 0; r < A_PER; ++r) {
      int e = tid + NT * r;
      int mm, kk;
      if (a_mfast) { mm = e % BM; kk = e / BM; } else { kk = e % BK; mm = e / BK; }
      int gm = m0 + mm, gk = k0 + kk;
      T v = O::zero();
      if (gm < g.M && gk < kend) v = A[(i64)gm * g.sAm + (i64)gk * g.sAk];
      ra[r] = g.conjA ? O::conj(v) : v;
    }
#pragma unroll
    for (int r = 0; r < B_PER; ++r) {
      int e = tid + NT * r;
      int nn, kk;
      if (b_kfast) { kk = e % BK; nn = e / BK; } else { nn = e % BN; kk = e / BN; }
      int gn = n0 + nn, gk = k0 + kk;
      T v = O::zero();
      if (gn < g.N && gk < kend) v = Bp[(i64)gk * g.sBk + (i64)gn * g.sBn];
      rb[r] = g.conjB ? O::conj(v) : v;
    }
  };
  auto store = [&]() {
#pragma unroll
    for (int r = 0; r < A_PER; ++r) {
      int e = tid + NT * r;
      int mm, kk;
      if (a_mfast) { mm = e % BM; kk = e / BM; } else { kk = e % BK; mm = e / BK; }
      As[kk * (BM + 1) + mm] = ra[r];
    }
#pragma unroll
    for (int r = 0; r < B_PER; ++r) {
      int e = tid + NT * r;
      int nn, kk;
      if (b_kfast) { kk = e % BK; nn = e / BK; } else { nn = e % BN; kk = e / BN; }
      Bs[kk * (BN + 1) + nn] = rb[r];
    }
  };

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = O::zero();

  if (kbeg < kend) load(kbeg);
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    __syncthreads();
    store();
    __syncthreads();
    if (k0 + BK < kend) load(k0 + BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T av[TM], bv[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) av[i] = As[kk * (BM + 1) + ty + TY * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) bv[j] = Bs[kk * (BN + 1) + tx + TX * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = O::fma(av[i], bv[j], acc[i][j]);
    }
  }
  __syncthreads();
  // stage the tile in shared memory, then store along the unit output stride
  T* Cs = smem;   // [BN][BM+1] (m fastest)
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) Cs[(tx + TX * j) * (BM + 1) + ty + TY * i] = acc[i][j];
  __syncthreads();
  const bool c_mfast = (g.sCm == 1) || (g.sCn != 1 && g.sCm < g.sCn);
  if (g.splitk > 1) {
    // the splitk CTAs of this tile are one cluster (rank = ks); CTA ks
    // finishes elements ks*NT + tid + j*NT*splitk, adding the partial tiles of
    // ranks 0..splitk-1 in that order
    namespace cgr = cooperative_groups;
    cgr::cluster_group cl = cgr::this_cluster();
    cl.sync();
    for (int e = ks * NT + tid; e < BM * BN; e += NT * g.splitk) {
      int mm, nn;
      if (c_mfast) { mm = e % BM; nn = e / BM; } else { nn = e % BN; mm = e / BN; }
      int gm = m0 + mm, gn = n0 + nn;
      if (gm >= g.M || gn >= g.N) continue;
      T acc_e = O::zero();
      for (int r = 0; r < g.splitk; ++r)
        acc_e = O::add(acc_e, cl.map_shared_rank(Cs, r)[nn * (BM + 1) + mm]);
      T v = O::mul(g.alpha, acc_e);
      T* p = C + (i64)gm * g.sCm + (i64)gn * g.sCn;
      if (!O::is_zero(g.beta)) v = O::add(v, O::mul(g.beta, *p));
      *p = v;
    }
    cl.sync();   // no CTA leaves while another still reads its tile
    return;
  }
  for (int e = tid; e < BM * BN; e += NT) {
    int mm, nn;
    if (c_mfast) { mm = e % BM; nn = e / BM; } else { nn = e % BN; mm = e / BN; }
    int gm = m0 + mm, gn = n0 + nn;
    if (gm >= g.M || gn >= g.N) continue;
    T v = O::mul(g.alpha, Cs[nn * (BM + 1) + mm]);
    T* p = C + (i64)gm * g.sCm + (i64)gn * g.sCn;
    if (!O::is_zero(g.beta)) v = O::add(v, O::mul(g.beta, *p));
    *p = v;
  }
}

template <class T>
__global__ void scale_kernel(T* C, int M, int N, i64 sCm, i64 sCn, int nb1, i64 bC1, i64 bC2,
                             T beta) {
  using O = Ops<T>;
  int b = blockIdx.z;
  T* Cb = C + (b % nb1) * bC1 + (b / nb1) * bC2;
  i64 total = (i64)M * N;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total;
       e += (i64)gridDim.x * blockDim.x) {
    int mm = (int)(e % M), nn = (int)(e / M);
    T* p = Cb + mm * sCm + nn * sCn;
    *p = O::is_zero(beta) ? O::zero() : O::mul(beta, *p);
  }
}

template <class T, int BM, int BN, int TM, int TN>
void launch_tile(const Args<T>& a, int nbatch, cudaStream_t s) {
  dim3 grid(ceil_div(a.M, BM), ceil_div(a.N, BN), nbatch * a.splitk);
  if (a.splitk > 1)
    launch_clustered(gemm_kernel<T, BM, BN, TM, TN>, grid, dim3(NT), dim3(1, 1, a.splitk), 0, s,
                     a);
  else {
    gemm_kernel<T, BM, BN, TM, TN><<<grid, NT, 0, s>>>(a);
    TTG_CHECK_LAUNCH();
  }
}

template <class T>
void launch(Args<T> a, int nbatch, cudaStream_t s) {
  if (a.M <= 0 || a.N <= 0 || nbatch <= 0) return;
  if (a.K <= 0) {
    // C = beta*C
    TTG_REQUIRE(nbatch < 65536, "gemm: batch too large");
    int blocks = std::min<i64>(4096, ((i64)a.M * a.N + 255) / 256);
    scale_kernel<T><<<dim3(blocks, 1, nbatch), 256, 0, s>>>(a.C, a.M, a.N, a.sCm, a.sCn, a.nb1,
                                                            a.bC1, a.bC2, a.beta);
    TTG_CHECK_LAUNCH();
    return;
  }
  if (a.splitk < 1) a.splitk = 1;
  // FP64 runs at about two FMAs per clock per SM on GB300, so a product is
  // only fast when its CTAs cover every SM: real products whose 64 x 64 tiles
  // give fewer than two CTAs per SM use 32 x 32 tiles, and products that still
  // leave SMs idle split K over the CTAs of a cluster (at most kMaxCluster
  // chunks, added in a fixed order).
  const bool small_tiles = sizeof(T) <= 8 && a.N > 16 && a.M > 16 &&
                           (i64)ceil_div(a.M, 64) * ceil_div(a.N, 64) * nbatch < 2 * 152;
  if constexpr (sizeof(T) == 16) {
    // complex128 (the KSL products): small ranks give thin products, so the
    // tiles are 32 x 16 / 16 x 32 / 32 x 32 and K splits (chunks of >= 16)
    // until about two CTAs per SM carry the FP64 work
    if (a.splitk == 1 && a.K >= 32) {
      const int bm = a.N <= 16 ? 32 : (a.M <= 16 ? 16 : 32);
      const int bn = a.N <= 16 ? 16 : (a.M <= 16 ? 32 : 32);
      const i64 ctas = (i64)ceil_div(a.M, bm) * ceil_div(a.N, bn) * nbatch;
      if (ctas < 152) {
        const i64 want = (304 + ctas - 1) / ctas;
        a.splitk = (int)std::max<i64>(1, std::min<i64>(want, a.K / 16));
      }
    }
  } else if (a.splitk == 1 && a.K >= 128) {
    int bm = a.N <= 16 ? 128 : (a.M <= 16 ? 16 : ((sizeof(T) <= 8 && !small_tiles) ? 64 : 32));
    int bn = a.N <= 16 ? 16 : (a.M <= 16 ? 128 : ((sizeof(T) <= 8 && !small_tiles) ? 64 : 32));
    i64 ctas = (i64)ceil_div(a.M, bm) * ceil_div(a.N, bn) * nbatch;
    if (ctas < 152) {
      i64 want = (304 + ctas - 1) / ctas;
      a.splitk = (int)std::max<i64>(1, std::min<i64>(want, a.K / 64));
    }
  }
  a.splitk = std::min(a.splitk, kMaxCluster);
  a.kchunk = ceil_div(ceil_div(a.K, a.splitk), BK) * BK;
  a.splitk = ceil_div(a.K, a.kchunk);
  // every limit is checked before anything is launched, so a rejected call
  // leaves C untouched
  TTG_REQUIRE((i64)nbatch * a.splitk < 65536, "gemm: batch*splitk too large");
  TTG_REQUIRE(ceil_div(a.N, 16) < 65536, "gemm: N too large");
  if constexpr (sizeof(T) == 16) {
    if (a.N <= 16)
      launch_tile<T, 32, 16, 2, 1>(a, nbatch, s);
    else if (a.M <= 16)
      launch_tile<T, 16, 32, 1, 2>(a, nbatch, s);
    else
      launch_tile<T, 32, 32, 2, 2>(a, nbatch, s);
    return;
  }
  if (a.N <= 16) {
    launch_tile<T, 128, 16, 4, 2>(a, nbatch, s);
  } else if (a.M <= 16) {
    launch_tile<T, 16, 128, 2, 4>(a, nbatch, s);
  } else {
    if constexpr (sizeof(T) <= 8) {
      if (small_tiles)
        launch_tile<T, 32, 32, 2, 2>(a, nbatch, s);
      else
        launch_tile<T, 64, 64, 4, 4>(a, nbatch, s);
    } else {
      // complex128: 32x32 tiles keep the static shared memory under 48 KB
      launch_tile<T, 32, 32, 2, 2>(a, nbatch, s);
    }
  }
}

}  // namespace

void gemm_f64(const GemmF64& g, cudaStream_t s) {
  Args<double> a{g.M, g.N, g.K, g.A, g.sAm, g.sAk, g.B, g.sBk, g.sBn, g.C, g.sCm, g.sCn,
                 g.alpha, g.beta, g.nb1, g.bA1, g.bA2, g.bB1, g.bB2, g.bC1, g.bC2,
                 g.splitk, 0, false, false};
  launch<double>(a, g.nb1 * g.nb2, s);
}

void gemm_f32(const GemmF32& g, cudaStream_t s) {
  Args<float> a{g.M, g.N, g.K, g.A, g.sAm, g.sAk, g.B, g.sBk, g.sBn, g.C, g.sCm, g.sCn,
                g.alpha, g.beta, g.nb1, g.bA1, g.bA2, g.bB1, g.bB2, g.bC1, g.bC2,
                g.splitk, 0, false, false};
  launch<float>(a, g.nb1 * g.nb2, s);
}

void gemm_z(const GemmZ& g, cudaStream_t s) {
  Args<double2> a{g.M, g.N, g.K, g.A, g.sAm, g.sAk, g.B, g.sBk, g.sBn, g.C, g.sCm, g.sCn,
                  g.alpha, g.beta, g.nb1, g.bA1, g.bA2, g.bB1, g.bB2, g.bC1, g.bC2,
                  g.splitk, 0, g.conjA, g.conjB};
  launch<double2>(a, g.nb1 * g.nb2, s);
}

}  // namespace ttg
