// Split-precision (BF16x3) tensor-core local operator for sm_103a.
//
// y = Phi1 * A * Phi2 * x  (dbfun3, ttals.f90:9-32) as two tcgen05 GEMMs and a
// CUDA-core contraction with the TT-matrix core:
//
//   GEMM1  T1[(b1,j,v), (a2,c2)] = sum_b2 X_v[(b1,j), b2] Phi2[b2, (a2,c2)]
//          M = rx1*m*nvec (all vectors of the block stacked), N = ra2*ry2, K = rx2
//   CORE   T2[(i,c2,v), (b1,a1)] = sum_(j,a2) A[(a1,i),(j,a2)] T1[(b1,j,v),(a2,c2)]
//   GEMM3  Y[c1, (i,c2,v)]       = sum_(b1,a1) Phi1[c1,(b1,a1)] T2[(i,c2,v),(b1,a1)]
//          M = ry1, N = n*ry2*nvec, K = rx1*ra1
//
// Both GEMMs put the index that is contiguous in their output (b1 in T1, c1
// in y) on the MMA M side, i.e. on TMEM lanes, so the epilogue stores of a
// warp are coalesced.
// Every FP64 operand a is split as a_hi = bf16(a), a_lo = bf16(a - a_hi) and a
// product is accumulated as a_hi b_hi + a_hi b_lo + a_lo b_hi in FP32 in
// tensor memory (the dropped a_lo b_lo term is ~2^-16 relative).  Operands
// are stored in global memory already in the tcgen05 K-major, no-swizzle
// canonical layout, tile by tile (128 or BN rows x 64 K-elements, core
// matrices of 8 rows x 16 bytes), so each pipeline stage is a handful of
// contiguous cp.async.bulk copies completing on an mbarrier.  One thread
// issues the MMAs (3 per 16-wide K step), tcgen05.commit releases the smem
// stage, and four epilogue warps read the FP32 accumulator with tcgen05.ld.
// Phi1 and Phi2 are split once per local problem (split_op_prepare); X is
// split per call.
//
// Every mbarrier wait is bounded: on timeout the kernel records an error
// code, waits (bounded) for the MMAs it issued, frees its tensor memory and
// returns; the host turns the code into TTG_ERR_CUDA.
#include "ttg_davidson.cuh"
#include <cuda_bf16.h>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

namespace ttg {
namespace tc {

constexpr int TM = 128;        // rows of the A tile (MMA M)
constexpr int TK = 64;         // K elements per pipeline stage (4 MMA K-steps)
constexpr int NTHREADS = 128;  // 4 warps: all read TMEM in the epilogue
constexpr long long WAIT_LIMIT = 1ll << 22;
constexpr int SMEM_PAD = 0;

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long i = 0; i < WAIT_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// K-major, no-swizzle shared memory descriptor: lbo = byte stride between the
// two 8x16B core matrices along K, sbo = byte stride between 8-row groups.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;   // descriptor version of sm_100-family tcgen05
  return d;                 // base offset 0, relative LBO, layout type 0 (no swizzle)
}

// kind::f16 instruction descriptor: BF16 x BF16 -> FP32, both K-major, M x N
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
  return (1u << 4)                     // D format F32
         | (1u << 7)                   // A format BF16
         | (1u << 10)                  // B format BF16
         | ((uint32_t)(N >> 3) << 17)  // N / 8
         | ((uint32_t)(M >> 4) << 24); // M / 16
}

// byte offset of element (r, k) inside one R x TK tile.  The tile is four
// 16-wide K slabs of R*32 bytes (one MMA K-step each); inside a slab the 8x8
// core matrices (8 rows x 16 bytes) of one 8-row group sit side by side
// (K-direction stride LBO = 128 B) and row groups follow each other
// (M/N-direction stride SBO = 256 B).  Every address one MMA can form from
// these two strides stays inside its slab.
__host__ __device__ __forceinline__ uint32_t tile_offset(int r, int k, int R) {
  return (uint32_t)((k >> 4) * (R * 32) + (r >> 3) * 256 + ((k >> 3) & 1) * 128 + (r & 7) * 16 +
                    (k & 7) * 2);
}
constexpr uint32_t LBO = 128;   // between the two core matrices along K
constexpr uint32_t SBO = 256;   // between consecutive 8-row groups

struct Tiled {            // one split operand (hi and lo planes) in tile order
  bf16* hi;
  bf16* lo;
  int rows, cols;         // logical sizes
  int R;                  // tile rows (128 for A operands, BN for B operands)
  int rtiles, ktiles;
  size_t elems() const { return (size_t)rtiles * R * ktiles * TK; }
};

// element (r, k) -> tile-order element index
__device__ __forceinline__ size_t tiled_index(int r, int k, int R, int ktiles) {
  size_t tile = (size_t)(r / R) * ktiles + (k / TK);
  return tile * (size_t)R * TK + (tile_offset(r % R, k % TK, R) >> 1);
}

__device__ __forceinline__ void split2(double v, bf16& hi, bf16& lo) {
  hi = __float2bfloat16_rn((float)v);
  lo = __float2bfloat16_rn((float)(v - (double)__bfloat162float(hi)));
}

// split an FP64 matrix into tiled hi/lo planes; element (r, k) is read at
// src[(r / rv) * vs + (r % rv) * sr + k * sk]; padding is written as zero.
// One thread per (row, 8-wide K group): rows vary fastest across a warp
// (coalesced reads when sr == 1) and each thread stores one 16-byte core
// matrix row per plane.
__global__ void split_kernel(const double* __restrict__ src, i64 rv, i64 vs, i64 sr, i64 sk,
                             int rows, int cols, int R, int rtiles, int ktiles,
                             bf16* __restrict__ hi, bf16* __restrict__ lo) {
  const i64 tr = (i64)rtiles * R, tk8 = (i64)ktiles * (TK / 8);
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tr * tk8;
       e += (i64)gridDim.x * blockDim.x) {
    const int r = (int)(e % tr), k0 = (int)(e / tr) * 8;
    const double* row = src + (r / rv) * vs + (r % rv) * sr;
    __align__(16) bf16 h[8], l[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      double v = 0.0;
      if (r < rows && k0 + q < cols) v = row[(i64)(k0 + q) * sk];
      split2(v, h[q], l[q]);
    }
    const size_t idx = tiled_index(r, k0, R, ktiles);
    *reinterpret_cast<uint4*>(hi + idx) = *reinterpret_cast<const uint4*>(h);
    *reinterpret_cast<uint4*>(lo + idx) = *reinterpret_cast<const uint4*>(l);
  }
}

// C[m, n] (m < M, n < N) = sum_k A[m, k] B[n, k], split-3 on tcgen05.
// C[m, n] goes to out[(m / rpv) * vstride + (m % rpv) * rstride + n * cstride].
// The accumulator row m sits in TMEM lane m % 128, so with rstride == 1 the
// 32 lanes of a warp store 32 consecutive elements (coalesced).
template <int BN, int STAGES, class OutT>
__global__ void __launch_bounds__(NTHREADS, 1)
    split_gemm_kernel(const bf16* __restrict__ Ahi, const bf16* __restrict__ Alo,
                      const bf16* __restrict__ Bhi, const bf16* __restrict__ Blo, int M, int N,
                      int ktiles, OutT* __restrict__ out, i64 rpv, i64 vstride, i64 rstride,
                      i64 cstride, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  constexpr uint32_t A_BYTES = TM * TK * 2;
  constexpr uint32_t B_BYTES = BN * TK * 2;
  constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int fail;

  // 1024-byte aligned stage area
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = blockIdx.x, nt = blockIdx.y;

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    mbar_init(smem_u32(&done_bar), 1);
    fail = 0;
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(smem_u32(&tmem_slot), BN);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t taddr = tmem_slot;

  if (tid == 0) {
    constexpr uint32_t idesc = make_idesc(TM, BN);
    const size_t a_tile = (size_t)TM * TK, b_tile = (size_t)BN * TK;
    auto issue = [&](int c, int s) {
      unsigned char* st = base + (size_t)s * STAGE_BYTES;
      uint32_t bar = smem_u32(&full_bar[s]);
      mbar_expect_tx(bar, STAGE_BYTES);
      size_t ao = ((size_t)mt * ktiles + c) * a_tile;
      size_t bo = ((size_t)nt * ktiles + c) * b_tile;
      bulk_g2s(smem_u32(st), Ahi + ao, A_BYTES, bar);
      bulk_g2s(smem_u32(st + A_BYTES), Alo + ao, A_BYTES, bar);
      bulk_g2s(smem_u32(st + 2 * A_BYTES), Bhi + bo, B_BYTES, bar);
      bulk_g2s(smem_u32(st + 2 * A_BYTES + B_BYTES), Blo + bo, B_BYTES, bar);
    };
    int issued = 0;
    for (int c = 0; c < STAGES && c < ktiles; ++c) { issue(c, c); ++issued; }
    bool ok = true;
    for (int c = 0; c < ktiles && ok; ++c) {
      const int s = c % STAGES;
      const uint32_t ph = (uint32_t)((c / STAGES) & 1);
      if (!mbar_wait(smem_u32(&full_bar[s]), ph)) { ok = false; break; }
      tc_fence_after();
      unsigned char* st = base + (size_t)s * STAGE_BYTES;
      const uint32_t a_hi = smem_u32(st), a_lo = smem_u32(st + A_BYTES);
      const uint32_t b_hi = smem_u32(st + 2 * A_BYTES), b_lo = smem_u32(st + 2 * A_BYTES + B_BYTES);
#pragma unroll
      for (int kk = 0; kk < TK / 16; ++kk) {
        // one 16-wide K slab per MMA
        const uint32_t aoff = kk * (TM * 32), boff = kk * (BN * 32);
        const uint64_t dAh = make_desc(a_hi + aoff, LBO, SBO);
        const uint64_t dAl = make_desc(a_lo + aoff, LBO, SBO);
        const uint64_t dBh = make_desc(b_hi + boff, LBO, SBO);
        const uint64_t dBl = make_desc(b_lo + boff, LBO, SBO);
        mma_bf16(taddr, dAh, dBh, idesc, (c > 0 || kk > 0) ? 1u : 0u);
        mma_bf16(taddr, dAh, dBl, idesc, 1u);
        mma_bf16(taddr, dAl, dBh, idesc, 1u);
      }
      mma_commit(smem_u32(&empty_bar[s]));
      const int nc = c + STAGES;
      if (nc < ktiles) {
        if (!mbar_wait(smem_u32(&empty_bar[s]), ph)) { ok = false; break; }
        issue(nc, s);
        ++issued;
      }
    }
    if (!ok) {
      fail = 1;
      atomicExch(err, 1);
      // let every copy that was issued land before the CTA can exit: the
      // copies read valid global memory and complete in microseconds, so
      // these waits end long before their limit; a drain that still gives up
      // is reported as its own error code (3)
      bool drained = true;
      for (int c = 0; c < issued; ++c) {
        const int s = c % STAGES;
        drained = mbar_wait(smem_u32(&full_bar[s]), (uint32_t)((c / STAGES) & 1)) && drained;
      }
      if (!drained) atomicExch(err, 3);
    }
    mma_commit(smem_u32(&done_bar));
  }
  __syncwarp();
  const bool done_ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&done_bar), 0));
  tc_fence_after();
  if (!done_ok && lane == 0) atomicExch(err, 2);
  if (done_ok && !fail) {
    const int row = mt * TM + warp * 32 + lane;
    OutT* orow = out + (row / rpv) * vstride + (row % rpv) * rstride;
    const int n0 = nt * BN;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      uint32_t r[16];
      tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
      tmem_ld_wait();
      if (row < M) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int n = n0 + c0 + q;
          if (n < N) orow[(i64)n * cstride] = (OutT)__uint_as_float(r[q]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(taddr, BN);
}

// CORE: T2[(i,c2,v),(b1,a1)] = sum_(j,a2) A[(a1,i),(j,a2)] T1[(b1,j,v),(a2,c2)]
// T1 is column-major with leading dimension ld1 over the rows (b1,j,v), so
// b1 is contiguous; the result is written split and tiled as the B operand of
// GEMM3 (rows (i,c2,v), K (b1,a1), tile rows 1 << lgR3).

__device__ __forceinline__ size_t tiled_index_pow2(int r, int k, int lgR, int ktiles) {
  const size_t tile = (size_t)(r >> lgR) * ktiles + (k >> 6);
  return (tile << (lgR + 6)) + (tile_offset(r & ((1 << lgR) - 1), k & (TK - 1), 1 << lgR) >> 1);
}
__device__ __forceinline__ void split2f(float v, bf16& hi, bf16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));   // v - hi is exact in FP32
}

// the TT-matrix core as a kernel parameter: a[q * NA + p] = A(a1,i,j,a2) with
// q = j + m*a2 and p = a1 + ra1*i, so every FMA reads it from the constant bank
template <int JA, int NA>
struct CoreCoef {
  float a[JA * NA];
};

// small cores (m*ra2 <= JA, n*ra1 <= NA): one thread per (B1 consecutive b1,
// c2, v); with B1 == 8 a thread loads 2 float4 per input and stores one
// 16-byte core-matrix row per output and plane.
template <int JA, int NA, int B1>
__global__ void __launch_bounds__(128)
    core_small_kernel(const float* __restrict__ T1, i64 ld1, const CoreCoef<JA, NA> A, int rx1,
                      int m, int ra2, int n, int ra1, int ry2, int nvec, int lgR3, int ktiles3,
                      bf16* __restrict__ hi, bf16* __restrict__ lo) {
  const int ja = m * ra2, na = n * ra1;
  const int nb = rx1 / B1;
  const i64 total = (i64)nb * ry2 * nvec;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total;
       e += (i64)gridDim.x * blockDim.x) {
    const int b1 = (int)(e % nb) * B1;
    const int c2 = (int)((e / nb) % ry2);
    const int v = (int)(e / ((i64)nb * ry2));
    const float* tb = T1 + b1 + (i64)rx1 * m * v + ld1 * ((i64)ra2 * c2);
    float t[JA][B1];
    {
      int j = 0, a2 = 0;
#pragma unroll
      for (int q = 0; q < JA; ++q) {
        if (q < ja) {
          const float* src = tb + (i64)rx1 * j + ld1 * a2;
          if (B1 == 8) {
            const float4 u = *reinterpret_cast<const float4*>(src);
            const float4 w = *reinterpret_cast<const float4*>(src + 4);
            t[q][0] = u.x; t[q][1 % B1] = u.y; t[q][2 % B1] = u.z; t[q][3 % B1] = u.w;
            t[q][4 % B1] = w.x; t[q][5 % B1] = w.y; t[q][6 % B1] = w.z; t[q][7 % B1] = w.w;
          } else {
#pragma unroll
            for (int b = 0; b < B1; ++b) t[q][b] = src[b];
          }
          if (++j == m) { j = 0; ++a2; }
        }
      }
    }
    int a1 = 0, i = 0;
#pragma unroll
    for (int p = 0; p < NA; ++p) {
      if (p < na) {
        float acc[B1];
#pragma unroll
        for (int b = 0; b < B1; ++b) acc[b] = 0.f;
#pragma unroll
        for (int q = 0; q < JA; ++q) {
          if (q < ja) {
            const float a = A.a[q * NA + p];
#pragma unroll
            for (int b = 0; b < B1; ++b) acc[b] = fmaf(a, t[q][b], acc[b]);
          }
        }
        const int r = i + n * (c2 + ry2 * v);
        const int k = b1 + rx1 * a1;
        const size_t idx = tiled_index_pow2(r, k, lgR3, ktiles3);
        if (B1 == 8) {
          __align__(16) bf16 h[8], l[8];
#pragma unroll
          for (int b = 0; b < 8; ++b) split2f(acc[b % B1], h[b], l[b]);
          *reinterpret_cast<uint4*>(hi + idx) = *reinterpret_cast<const uint4*>(h);
          *reinterpret_cast<uint4*>(lo + idx) = *reinterpret_cast<const uint4*>(l);
        } else {
#pragma unroll
          for (int b = 0; b < B1; ++b) {
            bf16 h, l;
            split2f(acc[b], h, l);
            const size_t ib = tiled_index_pow2(r, k + b, lgR3, ktiles3);
            hi[ib] = h;
            lo[ib] = l;
          }
        }
        if (++a1 == ra1) { a1 = 0; ++i; }
      }
    }
  }
}

// large cores (KSL/AMEn mode sizes n = 32..64): a tiled FP32 product over the
// flattened rows e = b1 + rx1*(c2 + ry2*v) (64 per block) and the outputs
// p = (a1, i) (64 per block), K = (j, a2) in chunks of 32; 256 threads with
// 4 x 4 results each.  A(a1,i,j,a2) sits at A[p + n*ra1*q].
// Few rows (small ranks, one vector) leave most SMs idle, so K may be split
// over gridDim.z chunks of qchunk: each chunk then writes its FP32 partial
// product to part[(z * rows + row) * na + p] and core_finish_kernel adds the
// chunks in order and splits the sum (deterministic, no atomics).
constexpr int CT_R = 64, CT_P = 64, CT_Q = 32;
__global__ void __launch_bounds__(256)
    core_tiled_kernel(const float* __restrict__ T1, i64 ld1, const double* __restrict__ A,
                      int rx1, int m, int ra2, int n, int ra1, int ry2, int nvec, int lgR3,
                      int ktiles3, bf16* __restrict__ hi, bf16* __restrict__ lo, int qchunk,
                      float* __restrict__ part) {
  __shared__ float Ts[CT_Q][CT_R + 4];
  __shared__ float As[CT_Q][CT_P + 4];
  __shared__ i64 rbase[CT_R];
  const int ja = m * ra2, na = n * ra1;
  const i64 rows = (i64)rx1 * ry2 * nvec;
  const i64 row0 = (i64)blockIdx.x * CT_R;
  const int p0 = blockIdx.y * CT_P;
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  if (tid < CT_R) {
    const i64 row = row0 + tid;
    i64 base = -1;
    if (row < rows) {
      const int b1 = (int)(row % rx1);
      const i64 cv = row / rx1;
      const int c2 = (int)(cv % ry2), v = (int)(cv / ry2);
      base = b1 + (i64)rx1 * m * v + ld1 * ((i64)ra2 * c2);
    }
    rbase[tid] = base;
  }
  float acc[4][4];
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) acc[x][y] = 0.f;
  const int qbeg = blockIdx.z * qchunk, qend = min(ja, qbeg + qchunk);
  for (int q0 = qbeg; q0 < qend; q0 += CT_Q) {
    __syncthreads();
    for (int l = tid; l < CT_R * CT_Q; l += 256) {
      const int rr = l % CT_R, qq = l / CT_R, q = q0 + qq;
      const i64 base = rbase[rr];
      float val = 0.f;
      if (base >= 0 && q < qend) val = T1[base + (i64)rx1 * (q % m) + ld1 * (q / m)];
      Ts[qq][rr] = val;
    }
    for (int l = tid; l < CT_P * CT_Q; l += 256) {
      const int pp = l % CT_P, qq = l / CT_P, p = p0 + pp, q = q0 + qq;
      As[qq][pp] = (p < na && q < qend) ? (float)A[p + (i64)na * q] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int qq = 0; qq < CT_Q; ++qq) {
      const float4 t4 = *reinterpret_cast<const float4*>(&Ts[qq][ty * 4]);
      const float4 a4 = *reinterpret_cast<const float4*>(&As[qq][tx * 4]);
      const float tv[4] = {t4.x, t4.y, t4.z, t4.w}, av[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) acc[x][y] = fmaf(tv[x], av[y], acc[x][y]);
    }
  }
  if (part) {
#pragma unroll
    for (int x = 0; x < 4; ++x) {
      const i64 row = row0 + ty * 4 + x;
      if (row >= rows) continue;
      float* dst = part + ((i64)blockIdx.z * rows + row) * na;
#pragma unroll
      for (int y = 0; y < 4; ++y) {
        const int p = p0 + tx * 4 + y;
        if (p < na) dst[p] = acc[x][y];
      }
    }
    return;
  }
#pragma unroll
  for (int x = 0; x < 4; ++x) {
    const i64 row = row0 + ty * 4 + x;
    if (row >= rows) continue;
    const int b1 = (int)(row % rx1);
    const i64 cv = row / rx1;
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      const int p = p0 + tx * 4 + y;
      if (p >= na) continue;
      const int a1 = p % ra1, i = p / ra1;
      const int r = (int)(i + (i64)n * cv);
      const int k = b1 + rx1 * a1;
      bf16 h, l;
      split2f(acc[x][y], h, l);
      const size_t idx = tiled_index_pow2(r, k, lgR3, ktiles3);
      hi[idx] = h;
      lo[idx] = l;
    }
  }
}

// sum of the K chunks of core_tiled_kernel, split into the GEMM3 operand
__global__ void core_finish_kernel(const float* __restrict__ part, int nz, i64 rows, int na,
                                   int rx1, int n, int ra1, int lgR3, int ktiles3,
                                   bf16* __restrict__ hi, bf16* __restrict__ lo) {
  const i64 total = rows * na;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total;
       e += (i64)gridDim.x * blockDim.x) {
    float acc = 0.f;
    for (int z = 0; z < nz; ++z) acc += part[(i64)z * total + e];
    const i64 row = e / na;
    const int p = (int)(e % na);
    const int b1 = (int)(row % rx1);
    const i64 cv = row / rx1;
    const int a1 = p % ra1, i = p / ra1;
    const int r = (int)(i + (i64)n * cv);
    const int k = b1 + rx1 * a1;
    bf16 h, l;
    split2f(acc, h, l);
    const size_t idx = tiled_index_pow2(r, k, lgR3, ktiles3);
    hi[idx] = h;
    lo[idx] = l;
  }
}

// K chunks of the tiled CORE product for rows x na outputs over ja
inline void core_chunks(i64 rows, int na, int ja, int& nz, int& qchunk) {
  const i64 base = ceil_div(rows, (i64)CT_R) * ceil_div(na, CT_P);
  nz = 1;
  qchunk = ja;
  if (base < 152 && ja > CT_Q) {
    const i64 want = std::min<i64>(ceil_div(ja, CT_Q), ceil_div((i64)304, base));
    qchunk = (int)ceil_div((i64)ceil_div((i64)ja, want), (i64)CT_Q) * CT_Q;
    nz = (int)ceil_div((i64)ja, (i64)qchunk);
  }
}

static int num_sms() {
  static const int nsm = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      v = 148;
    return v;
  }();
  return nsm;
}

constexpr int stages_for(int bn) { return bn == 256 ? 2 : (bn == 128 ? 3 : 2); }
constexpr size_t smem_for(int bn) {
  return (size_t)stages_for(bn) * ((size_t)2 * TM * TK * 2 + (size_t)2 * bn * TK * 2) + 1024;
}

// B-operand tile rows for an M x N x K product: the estimated time is the
// number of waves (CTAs over SMs x resident CTAs) times the per-tile cost
// (K loop of MMAs and bulk copies plus the epilogue), so small products pick
// narrow tiles that spread over more SMs and large ones pick wide tiles.
static int pick_bn(int M, int N, int K) {
  const int mt = ceil_div(M, TM), kt = ceil_div(K, TK), nsm = num_sms();
  int best = 64;
  double best_cost = 1e300;
  for (int bn : {256, 128, 64}) {
    const int per_sm = (int)std::max<size_t>(1, 228 * 1024 / (smem_for(bn) + 1024));
    const long long ctas = (long long)mt * ceil_div(N, bn);
    const long long waves = (ctas + (long long)nsm * per_sm - 1) / ((long long)nsm * per_sm);
    const double cost = (double)waves * (kt * (bn / 64.0 + 1.0) + bn / 64.0 + 2.0);
    if (cost < best_cost - 1e-9) { best_cost = cost; best = bn; }
  }
  return best;
}

static Tiled make_tiled(int rows, int cols, int R, char*& p) {
  Tiled t;
  t.rows = rows; t.cols = cols; t.R = R;
  t.rtiles = ceil_div(rows, R);
  t.ktiles = ceil_div(cols, TK);
  size_t bytes = (t.elems() * sizeof(bf16) + 1023) & ~size_t(1023);
  t.hi = (bf16*)p; p += bytes;
  t.lo = (bf16*)p; p += bytes;
  return t;
}
static size_t tiled_bytes(int rows, int cols, int R) {
  size_t e = (size_t)ceil_div(rows, R) * R * ceil_div(cols, TK) * TK;
  return 2 * ((e * sizeof(bf16) + 1023) & ~size_t(1023));
}

static void split_into(const double* src, i64 rv, i64 vs, i64 sr, i64 sk, const Tiled& t,
                       cudaStream_t s) {
  i64 total = (i64)t.rtiles * t.R * t.ktiles * (TK / 8);
  int blocks = (int)std::min<i64>(8192, (total + 255) / 256);
  split_kernel<<<blocks, 256, 0, s>>>(src, rv, vs, sr, sk, t.rows, t.cols, t.R, t.rtiles,
                                      t.ktiles, t.hi, t.lo);
  TTG_CHECK_LAUNCH();
}

template <int BN, class OutT>
static void gemm_launch_bn(const Tiled& A, const Tiled& B, int M, int N, OutT* out, i64 rpv,
                           i64 vstride, i64 rstride, i64 cstride, int* err, cudaStream_t s) {
  constexpr int STAGES = stages_for(BN);
  constexpr size_t smem = smem_for(BN) + SMEM_PAD;
  auto kern = split_gemm_kernel<BN, STAGES, OutT>;
  static const cudaError_t attr_rc =
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  TTG_CUDA(attr_rc);
  dim3 grid(A.rtiles, B.rtiles);
  kern<<<grid, NTHREADS, smem, s>>>(A.hi, A.lo, B.hi, B.lo, M, N, A.ktiles, out, rpv, vstride,
                                    rstride, cstride, err);
  TTG_CHECK_LAUNCH();
}

template <class OutT>
static void gemm_launch(const Tiled& A, const Tiled& B, int M, int N, OutT* out, i64 rpv,
                        i64 vstride, i64 rstride, i64 cstride, int* err, cudaStream_t s) {
  TTG_REQUIRE(A.ktiles == B.ktiles, "split gemm: K tiles differ");
  TTG_REQUIRE(A.R == TM, "split gemm: A tiles must have 128 rows");
  if (B.R == 256) gemm_launch_bn<256>(A, B, M, N, out, rpv, vstride, rstride, cstride, err, s);
  else if (B.R == 128) gemm_launch_bn<128>(A, B, M, N, out, rpv, vstride, rstride, cstride, err, s);
  else gemm_launch_bn<64>(A, B, M, N, out, rpv, vstride, rstride, cstride, err, s);
}

// Tile-width autotuner.  The first product of each shape class (tile counts
// ceil(M/128), ceil(N/64), ceil(K/64) and the output type) times the three
// tile widths on zeroed operands of that shape, three launches each after a
// warm-up, with CUDA events on the caller's stream, and keeps the fastest;
// later products of the class reuse it.  The cost model above is the choice
// while a stream is being captured into a graph and when TTG_AUTOTUNE=0;
// TTG_AUTOTUNE=2 prints each choice.
struct TuneKey {
  int mt, nt, kt, dbl;
  bool operator<(const TuneKey& o) const {
    return std::tie(mt, nt, kt, dbl) < std::tie(o.mt, o.nt, o.kt, o.dbl);
  }
};
static std::mutex g_tune_mu;
static std::map<TuneKey, int> g_tuned;

template <class OutT>
static float time_bn(int bn, const Tiled& A, char* bbuf, int M, int N, int K, OutT* out,
                     int* err, cudaStream_t s) {
  char* p = bbuf;
  const Tiled B = make_tiled(N, K, bn, p);
  cudaEvent_t e0, e1;
  TTG_CUDA(cudaEventCreate(&e0));
  TTG_CUDA(cudaEventCreate(&e1));
  gemm_launch<OutT>(A, B, M, N, out, 1ll << 40, 0, 1, M, err, s);
  TTG_CUDA(cudaEventRecord(e0, s));
  for (int r = 0; r < 3; ++r) gemm_launch<OutT>(A, B, M, N, out, 1ll << 40, 0, 1, M, err, s);
  TTG_CUDA(cudaEventRecord(e1, s));
  TTG_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  TTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

static int tuned_bn(int M, int N, int K, bool out_double, cudaStream_t s) {
  static const bool enabled = [] {
    const char* v = std::getenv("TTG_AUTOTUNE");
    return !(v && v[0] == '0');
  }();
  const int model = pick_bn(M, N, K);
  if (!enabled) return model;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
    return model;
  const TuneKey key{ceil_div(M, TM), ceil_div(N, 64), ceil_div(K, TK), out_double ? 1 : 0};
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tuned.find(key);
  if (it != g_tuned.end()) return it->second;
  // zeroed operands of this shape: A tiles, B tiles at the widest padding,
  // the output and the wait flag
  const size_t abytes = tiled_bytes(M, K, TM) + 1024, bbytes = tiled_bytes(N, K, 256) + 1024;
  const size_t obytes = (size_t)M * N * (out_double ? 8 : 4) + 1024;
  char* mem = nullptr;
  if (cudaMalloc(&mem, abytes + bbytes + obytes + 1024) != cudaSuccess) {
    (void)cudaGetLastError();
    g_tuned[key] = model;
    return model;
  }
  struct Free { char* p; ~Free() { cudaFree(p); } } fr{mem};
  TTG_CUDA(cudaMemsetAsync(mem, 0, abytes + bbytes + obytes + 1024, s));
  char* p = mem;
  const Tiled A = make_tiled(M, K, TM, p);
  char* bbuf = mem + abytes;
  void* out = mem + abytes + bbytes;
  int* err = (int*)(mem + abytes + bbytes + obytes);
  int best = model;
  float best_ms = 1e30f;
  for (int bn : {64, 128, 256}) {
    const float ms = out_double ? time_bn<double>(bn, A, bbuf, M, N, K, (double*)out, err, s)
                                : time_bn<float>(bn, A, bbuf, M, N, K, (float*)out, err, s);
    if (ms < best_ms * 0.97f || (bn == model && ms < best_ms * 1.03f)) { best_ms = ms; best = bn; }
  }
  int herr = 0;
  TTG_CUDA(cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) throw Error{TTG_ERR_CUDA, "split gemm autotune: mbarrier wait timed out"};
  g_tuned[key] = best;
  static const bool verbose = [] {
    const char* v = std::getenv("TTG_AUTOTUNE");
    return v && v[0] == '2';
  }();
  if (verbose)
    fprintf(stderr, "[ttg autotune] M=%d N=%d K=%d %s: BN=%d (%.1f us; cost model %d)\n", M, N, K,
            out_double ? "f64" : "f32", best, best_ms * 1000.f / 3.f, model);
  return best;
}

}  // namespace tc

// prepared split operator of one local problem
//   GEMM1: A = X (rows (b1,j,v), K b2), B = Phi2 (rows (a2,c2), K b2),
//          T1 column-major (rows (b1,j,v), ld1 = rx1*m*nvec_max)
//   CORE : T1 -> T2 (GEMM3 B operand: rows (i,c2,v), K (b1,a1))
//   GEMM3: A = Phi1 (rows c1, K (b1,a1)), B = T2, y[c1 + ry1*(i,c2,v)]
struct SplitOp {
  LocalDims L;
  int nvec_max;
  int bn1, bn3;
  tc::Tiled X, P2, P1, T2;
  float* T1;
  i64 ld1;
  const double* A;
  int* err;
  float* part;          // K-chunk partials of the tiled CORE kernel (or null)
  int coef_kind;        // 0: tiled CORE kernel; 1..4: small CORE with (JA, NA) bound
  float coef[256];      // A as FP32 in its own column-major order (small CORE)
};

// Sizing (op == nullptr) takes the widest tile padding so that the bytes
// bound every tile width the autotuner may pick at layout time.
static size_t split_layout(const LocalDims& L, int nvec_max, SplitOp* op, char* base,
                           cudaStream_t s = nullptr) {
  const int M1 = (int)(L.rx1 * L.m * nvec_max), N1 = (int)(L.ra2 * L.ry2), K1 = (int)L.rx2;
  const int M3 = (int)L.ry1, N3 = (int)(L.n * L.ry2 * nvec_max), K3 = (int)(L.rx1 * L.ra1);
  const bool sizing = !(op && base);
  const int bn1 = sizing ? 256 : tc::tuned_bn(M1, N1, K1, false, s);
  const int bn3 = sizing ? 256 : tc::tuned_bn(M3, N3, K3, true, s);
  size_t tot = 0;
  tot += tc::tiled_bytes(M1, K1, tc::TM) + tc::tiled_bytes(N1, K1, bn1);
  tot += tc::tiled_bytes(M3, K3, tc::TM) + tc::tiled_bytes(N3, K3, bn3);
  const i64 ld1 = (i64)ceil_div(M1, 4) * 4;
  size_t t1 = ((size_t)ld1 * ceil_div(N1, 4) * 4 * sizeof(float) + 1023) & ~size_t(1023);
  tot += t1 + 1024 + sizeof(SplitOp) + 1024;
  // K-chunk partials of the tiled CORE kernel, the largest over 1..nvec_max
  const int ja = (int)(L.m * L.ra2), na = (int)(L.n * L.ra1);
  size_t part = 0;
  if (!(ja <= 16 && na <= 16)) {
    for (int v = 1; v <= nvec_max; ++v) {
      int nz, qc;
      tc::core_chunks(L.rx1 * L.ry2 * v, na, ja, nz, qc);
      const size_t b = (size_t)(nz * L.rx1 * L.ry2 * v * na) * sizeof(float);
      if (nz > 1 && b > part) part = b;
    }
  }
  part = (part + 1023) & ~size_t(1023);
  tot += part;
  if (op && base) {
    char* p = base;
    op->L = L;
    op->nvec_max = nvec_max;
    op->bn1 = bn1; op->bn3 = bn3;
    op->X = tc::make_tiled(M1, K1, tc::TM, p);
    op->P2 = tc::make_tiled(N1, K1, bn1, p);
    op->P1 = tc::make_tiled(M3, K3, tc::TM, p);
    op->T2 = tc::make_tiled(N3, K3, bn3, p);
    op->T1 = (float*)p; p += t1;
    op->ld1 = ld1;
    op->err = (int*)p; p += 1024;
    op->part = part ? (float*)p : nullptr; p += part;
  }
  return tot;
}

size_t split_op_bytes(const LocalDims& L, int nvec_max) { return split_layout(L, nvec_max, nullptr, nullptr); }

bool split_op_supported(const LocalDims& L) {
  return L.rx1 * L.m * 64 < (1ll << 31) && L.n * L.ry2 * 64 < (1ll << 31) &&
         L.rx1 * L.m * 64 * L.ra2 * L.ry2 < (1ll << 40);
}

// prepare: split Phi2 (GEMM1 B: rows (a2,c2), K b2) and Phi1 (GEMM3 A: rows
// c1, K (b1,a1)) once per local problem.  The SplitOp header lives in host
// memory owned by the caller; mem holds the device buffers.
void split_op_prepare(SplitOp* op, const LocalDims& L, int nvec_max, const double* phi1,
                      const double* A, const double* phi2, void* mem, cudaStream_t s) {
  split_layout(L, nvec_max, op, (char*)mem, s);
  op->A = A;
  // small TT-matrix cores travel as a kernel parameter of the CORE kernel
  const int ja = (int)(L.m * L.ra2), na = (int)(L.n * L.ra1);
  op->coef_kind = 0;
  if (ja <= 4 && na <= 4) op->coef_kind = 1;
  else if (ja <= 8 && na <= 8) op->coef_kind = 2;
  else if (ja <= 10 && na <= 10) op->coef_kind = 3;
  else if (ja <= 16 && na <= 16) op->coef_kind = 4;
  if (op->coef_kind) {
    double ah[256];
    TTG_CUDA(cudaMemcpyAsync(ah, A, (size_t)ja * na * sizeof(double), cudaMemcpyDeviceToHost, s));
    TTG_CUDA(cudaStreamSynchronize(s));
    for (int e = 0; e < ja * na; ++e) op->coef[e] = (float)ah[e];
  }
  // Phi2 element (n=(a2,c2), k=b2) at phi2[b2 + rx2*n]
  tc::split_into(phi2, 1ll << 40, 0, L.rx2, 1, op->P2, s);
  // Phi1 element (c1, k=(b1,a1)) at phi1[c1 + ry1*k]
  tc::split_into(phi1, 1ll << 40, 0, 1, L.ry1, op->P1, s);
  // T2 padding (K columns the CORE kernel never writes) must be zero: padded
  // K columns meet zero columns of Phi1, and 0 * garbage could be NaN
  TTG_CUDA(cudaMemsetAsync(op->T2.hi, 0, op->T2.elems() * sizeof(tc::bf16), s));
  TTG_CUDA(cudaMemsetAsync(op->T2.lo, 0, op->T2.elems() * sizeof(tc::bf16), s));
  TTG_CUDA(cudaMemsetAsync(op->err, 0, sizeof(int), s));
}

static void core_apply(SplitOp* op, int nvec, cudaStream_t s) {
  const LocalDims& L = op->L;
  const tc::Tiled& T2 = op->T2;
  const int lgR3 = T2.R == 256 ? 8 : (T2.R == 128 ? 7 : 6);
  const int ja = (int)(L.m * L.ra2), na = (int)(L.n * L.ra1);
  if (op->coef_kind > 0) {
    const bool wide = L.rx1 % 8 == 0 && (L.rx1 / 8) * L.ry2 * nvec >= 32768;
    const i64 total = (wide ? L.rx1 / 8 : L.rx1) * L.ry2 * nvec;
    const int blocks = (int)std::min<i64>(8192, (total + 127) / 128);
#define TTG_CORE_SMALL(JA, NA)                                                                  \
  do {                                                                                          \
    tc::CoreCoef<JA, NA> cc;                                                                    \
    for (int q = 0; q < JA; ++q)                                                                \
      for (int p = 0; p < NA; ++p)                                                              \
        cc.a[q * NA + p] = (q < ja && p < na) ? op->coef[(size_t)q * na + p] : 0.f;            \
    if (wide)                                                                                   \
      tc::core_small_kernel<JA, NA, 8><<<blocks, 128, 0, s>>>(                                 \
          op->T1, op->ld1, cc, (int)L.rx1, (int)L.m, (int)L.ra2, (int)L.n, (int)L.ra1,         \
          (int)L.ry2, nvec, lgR3, T2.ktiles, T2.hi, T2.lo);                                    \
    else                                                                                        \
      tc::core_small_kernel<JA, NA, 1><<<blocks, 128, 0, s>>>(                                 \
          op->T1, op->ld1, cc, (int)L.rx1, (int)L.m, (int)L.ra2, (int)L.n, (int)L.ra1,         \
          (int)L.ry2, nvec, lgR3, T2.ktiles, T2.hi, T2.lo);                                    \
  } while (0)
    switch (op->coef_kind) {
      case 1: TTG_CORE_SMALL(4, 4); break;
      case 2: TTG_CORE_SMALL(8, 8); break;
      case 3: TTG_CORE_SMALL(10, 10); break;
      default: TTG_CORE_SMALL(16, 16); break;
    }
#undef TTG_CORE_SMALL
  } else {
    const i64 rows = L.rx1 * L.ry2 * nvec;
    int nz, qchunk;
    tc::core_chunks(rows, na, ja, nz, qchunk);
    if (nz > 1 && !op->part) nz = 1, qchunk = ja;
    float* part = nz > 1 ? op->part : nullptr;
    dim3 grid((unsigned)ceil_div(rows, (i64)tc::CT_R), (unsigned)ceil_div(na, tc::CT_P), nz);
    tc::core_tiled_kernel<<<grid, 256, 0, s>>>(op->T1, op->ld1, op->A, (int)L.rx1, (int)L.m,
                                              (int)L.ra2, (int)L.n, (int)L.ra1, (int)L.ry2, nvec,
                                              lgR3, T2.ktiles, T2.hi, T2.lo, qchunk, part);
    if (part) {
      TTG_CHECK_LAUNCH();
      const i64 tot = rows * na;
      tc::core_finish_kernel<<<(int)std::min<i64>(4096, ceil_div(tot, (i64)256)), 256, 0, s>>>(
          part, nz, rows, na, (int)L.rx1, (int)L.n, (int)L.ra1, lgR3, T2.ktiles, T2.hi, T2.lo);
    }
  }
  TTG_CHECK_LAUNCH();
}

void split_op_apply(SplitOp* op, const double* x, double* y, int nvec, cudaStream_t s) {
  const LocalDims& L = op->L;
  TTG_REQUIRE(nvec >= 1 && nvec <= op->nvec_max, "split matvec: nvec out of range");
  const int M1 = (int)(L.rx1 * L.m * nvec), N1 = (int)(L.ra2 * L.ry2);
  const int M3 = (int)L.ry1, N3 = (int)(L.n * L.ry2 * nvec);
  // X_v element (row (b1,j), k=b2) at x[v*xsize + row + rx1*m*b2]
  tc::Tiled X = op->X;
  X.rows = M1;
  X.rtiles = ceil_div(M1, tc::TM);
  tc::split_into(x, L.rx1 * L.m, L.xsize(), 1, L.rx1 * L.m, X, s);
  // GEMM1 -> T1 column-major: T1[row + ld1 * col]
  tc::gemm_launch<float>(X, op->P2, M1, N1, op->T1, 1ll << 40, 0, 1, op->ld1, op->err, s);
  // CORE -> T2 tiled
  core_apply(op, nvec, s);
  // GEMM3 -> y: C[c1, col] with col = (i,c2,v) goes to y[c1 + ry1 * col]
  tc::Tiled T2b = op->T2;
  T2b.rtiles = ceil_div(N3, T2b.R);
  tc::gemm_launch<double>(op->P1, T2b, M3, N3, y, 1ll << 40, 0, 1, L.ry1, op->err, s);
}

// Davidson matvec factory for the chosen method (host-side SplitOp header is
// kept in a small per-thread pool so the functor stays trivially copyable).
size_t split_matvec_bytes(const LocalDims& L, int nvec_max) {
  return split_op_bytes(L, nvec_max) + 4096;
}

// Two prepared operators per host thread (an operator and its adjoint).
constexpr int kSplitSlots = 2;
static thread_local SplitOp op_store[kSplitSlots];
static thread_local bool op_store_set[kSplitSlots] = {};

void split_matvec_factory(const LocalDims& L, const double* phi1, const double* A,
                          const double* phi2, int nvec_max, void* mem, cudaStream_t s,
                          MatvecFn* out, int slot) {
  TTG_REQUIRE(slot >= 0 && slot < kSplitSlots, "split matvec: bad operator slot");
  TTG_REQUIRE(split_op_supported(L), "split matvec: local problem too large");
  op_store_set[slot] = true;
  split_op_prepare(&op_store[slot], L, nvec_max, phi1, A, phi2, mem, s);
  SplitOp* op = &op_store[slot];
  *out = [op, s](const double* X, double* Y, int nv) { split_op_apply(op, X, Y, nv, s); };
}

// Reads the bounded-wait flags of the calling thread's prepared split
// operators in slots [0, nslots) (set by a GEMM whose mbarrier wait gave up);
// throws when set.  Only slots the caller prepared itself may be named: a
// slot left from an earlier call points into memory that call has freed.
void split_matvec_check(cudaStream_t s, int nslots) {
  TTG_REQUIRE(nslots >= 1 && nslots <= kSplitSlots, "split matvec: bad slot count");
  int herr[kSplitSlots] = {};
  bool any = false;
  for (int k = 0; k < nslots; ++k) {
    if (!op_store_set[k] || !op_store[k].err) continue;
    TTG_CUDA(cudaMemcpyAsync(&herr[k], op_store[k].err, sizeof(int), cudaMemcpyDeviceToHost, s));
    any = true;
  }
  if (!any) return;
  TTG_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k < nslots; ++k)
    if (herr[k]) throw Error{TTG_ERR_CUDA, "split gemm: mbarrier wait timed out"};
}

}  // namespace ttg

using namespace ttg;

extern "C" int ttg_dbfun3_split(ttg_ctx* c, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1,
                                ttg_int n, ttg_int ry2, ttg_int ra1, ttg_int ra2,
                                const double* phi1, const double* A, const double* phi2,
                                const double* x, double* y, ttg_int nvec) {
  if (!c) return TTG_ERR_ARG;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    TTG_REQUIRE(rx1 > 0 && m > 0 && rx2 > 0 && ry1 > 0 && n > 0 && ry2 > 0 && ra1 > 0 && ra2 > 0,
                "all sizes must be positive");
    TTG_REQUIRE(phi1 && A && phi2 && x && y && nvec > 0 && nvec <= 32, "bad pointer or nvec");
    LocalDims L{rx1, m, rx2, ry1, n, ry2, ra1, ra2};
    TTG_REQUIRE(split_op_supported(L), "local problem too large for the split kernel");
    size_t bytes = split_op_bytes(L, (int)nvec);
    c->ws.reset();
    c->ws.reserve(bytes);
    void* mem = c->ws.take(bytes);
    SplitOp op;
    split_op_prepare(&op, L, (int)nvec, phi1, A, phi2, mem, c->stream);
    split_op_apply(&op, x, y, (int)nvec, c->stream);
    int herr = 0;
    TTG_CUDA(cudaMemcpyAsync(&herr, op.err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TTG_CUDA(cudaStreamSynchronize(c->stream));
    if (herr) throw Error{TTG_ERR_CUDA, "split gemm: mbarrier wait timed out"};
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}

// ------------------------------------------------------------- prepared operator
struct ttg_localop {
  ttg_ctx* ctx;
  LocalDims L;
  int method;
  int nvec_max;
  const double *phi1, *A, *phi2;
  void* mem;
  SplitOp split;
};

extern "C" int ttg_localop_create(ttg_ctx* c, ttg_int rx1, ttg_int m, ttg_int rx2, ttg_int ry1,
                                  ttg_int n, ttg_int ry2, ttg_int ra1, ttg_int ra2,
                                  const double* phi1, const double* A, const double* phi2,
                                  ttg_int nvec_max, int method, ttg_localop** out) {
  if (!c || !out) return TTG_ERR_ARG;
  *out = nullptr;
  ttg_localop* op = nullptr;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    TTG_REQUIRE(rx1 > 0 && m > 0 && rx2 > 0 && ry1 > 0 && n > 0 && ry2 > 0 && ra1 > 0 && ra2 > 0,
                "all sizes must be positive");
    TTG_REQUIRE(phi1 && A && phi2 && nvec_max > 0 && nvec_max <= 64, "bad pointer or nvec_max");
    TTG_REQUIRE(method == TTG_METHOD_PLAIN || method == TTG_METHOD_SPLIT, "unknown method");
    LocalDims L{rx1, m, rx2, ry1, n, ry2, ra1, ra2};
    TTG_REQUIRE(L.xsize() < (1ll << 31) && L.ysize() < (1ll << 31), "local problem too large");
    op = new ttg_localop();
    op->ctx = c; op->L = L; op->method = method; op->nvec_max = (int)nvec_max;
    op->phi1 = phi1; op->A = A; op->phi2 = phi2; op->mem = nullptr;
    size_t bytes = method == TTG_METHOD_SPLIT ? split_op_bytes(L, (int)nvec_max)
                                              : bfun3_f64_scratch(L, (int)nvec_max);
    if (method == TTG_METHOD_SPLIT) TTG_REQUIRE(split_op_supported(L), "too large for split");
    TTG_CUDA(cudaMalloc(&op->mem, bytes));
    if (method == TTG_METHOD_SPLIT)
      split_op_prepare(&op->split, L, (int)nvec_max, phi1, A, phi2, op->mem, c->stream);
    *out = op;
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    if (op) { if (op->mem) cudaFree(op->mem); delete op; }
    return e.code;
  }
  return TTG_OK;
}

extern "C" int ttg_localop_apply(ttg_localop* op, const double* x, double* y, ttg_int nvec) {
  if (!op) return TTG_ERR_ARG;
  ttg_ctx* c = op->ctx;
  try {
    TTG_CUDA(cudaSetDevice(c->device));
    TTG_REQUIRE(x && y && nvec > 0 && nvec <= op->nvec_max, "bad pointer or nvec");
    if (op->method == TTG_METHOD_SPLIT)
      split_op_apply(&op->split, x, y, (int)nvec, c->stream);
    else
      bfun3_f64(op->L, op->phi1, op->A, op->phi2, x, y, (int)nvec, (double*)op->mem, c->stream);
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}

extern "C" int ttg_localop_destroy(ttg_localop* op) {
  if (!op) return TTG_ERR_ARG;
  cudaSetDevice(op->ctx->device);
  cudaStreamSynchronize(op->ctx->stream);
  if (op->mem) cudaFree(op->mem);
  delete op;
  return TTG_OK;
}
