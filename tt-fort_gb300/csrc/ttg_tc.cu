// Split-precision (BF16x3) tensor-core local operator for sm_103a.
//
// y = Phi1 * A * Phi2 * x  (dbfun3, ttals.f90:9-32).  Two forms:
//
// Core-contracted (small mode sizes, n*m <= 4, rx1 % 8 == 0: the spin chains
// of tt_eigb): the TT-matrix core is folded into Phi2 once per local problem,
//   Q      Q[(i,c2,a1), (j,b2)] = sum_a2 A(a1,i,j,a2) Phi2(b2,a2,c2)   (FP64)
//   GEMM1  T2[(i,c2,v), (b1,a1)] = sum_(j,b2) Q[(i,c2,a1),(j,b2)] X_v[b1,(j,b2)]
//          M = n*ry2*ra1, N = rx1*nvec, K = m*rx2; the epilogue writes T2 split
//          and tiled as the B operand of GEMM3 (no FP32 intermediate)
//   GEMM3  Y[c1, (i,c2,v)]       = sum_(b1,a1) Phi1[c1,(b1,a1)] T2[(i,c2,v),(b1,a1)]
//          M = ry1, N = n*ry2*nvec, K = rx1*ra1
// General (any mode size): two tcgen05 GEMMs around a CUDA-core contraction,
//   GEMM1  T1[(b1,j,v), (a2,c2)] = sum_b2 X_v[(b1,j), b2] Phi2[b2, (a2,c2)]
//          M = rx1*m*nvec (all vectors of the block stacked), N = ra2*ry2, K = rx2
//   CORE   T2[(i,c2,v), (b1,a1)] = sum_(j,a2) A[(a1,i),(j,a2)] T1[(b1,j,v),(a2,c2)]
//   GEMM3  as above.
//
// The GEMMs put the index that is contiguous in their output (b1 in T1, c1
// in y) on the MMA M side, i.e. on TMEM lanes, so the epilogue stores of a
// warp are coalesced.
// Every FP64 operand a is split as a_hi = bf16(a), a_lo = bf16(a - a_hi) and a
// product is accumulated as a_hi b_hi + a_hi b_lo + a_lo b_hi in FP32 in
// tensor memory (the dropped a_lo b_lo term is ~2^-16 relative).  Operands
// are stored in global memory already in the tcgen05 K-major, no-swizzle
// canonical layout, tile by tile (128 or BN rows x 64 K-elements, core
// matrices of 8 rows x 16 bytes), so each pipeline stage is a handful of
// contiguous cp.async.bulk copies completing on an mbarrier.  The products
// run in a persistent warp-specialised kernel (split_gemm_ws_kernel: one
// copy thread, one MMA thread issuing 3 MMAs per 16-wide K step, eight
// epilogue warps reading a double-buffered FP32 accumulator with tcgen05.ld);
// split_gemm_kernel is the one-tile-per-CTA form (TTG_GEMM_WS=0).
// Phi1, Phi2 (or Q) are split once per local problem (split_op_prepare); X is
// split per call.
//
// Every mbarrier wait is bounded: on timeout the kernel records an error
// code, waits (bounded) for the copies and MMAs it issued, frees its tensor
// memory and returns; the host turns the code into TTG_ERR_CUDA.
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

// v ~ hi + lo in bf16: one FP64 -> FP32 conversion, then FP32 arithmetic.
// GB300 issues FP64 conversions and arithmetic at a small fraction of its
// FP32 rate, so the remainder is taken from f = fl32(v): the split then
// carries |v - f| <= 2^-24 |v| beyond the lo term's own rounding (2^-9 of
// |v - hi|, itself <= 2^-9 |v|), far below what the products keep.
// fl32(v) truncated toward zero from the two 32-bit halves of v with 32-bit
// integer operations only (|v - f| < 2^-23 |v|); values outside FP32's
// normal range, and zeros, take the FP64 conversion
__device__ __forceinline__ float d2f_trunc(double v) {
  const unsigned int h = (unsigned int)__double2hiint(v), l = (unsigned int)__double2loint(v);
  const unsigned int e = (h >> 20) & 0x7FF;
  if (e < 897 || e > 1150) return __double2float_rn(v);
  return __uint_as_float((h & 0x80000000u) | ((e - 896) << 23) | ((h & 0xFFFFFu) << 3) | (l >> 29));
}

__device__ __forceinline__ void split2(double v, bf16& hi, bf16& lo) {
  const float f = __double2float_rn(v);
  hi = __float2bfloat16_rn(f);
  lo = __float2bfloat16_rn(f - __bfloat162float(hi));   // exact in FP32
}


// split an FP64 matrix into tiled hi/lo planes; element (r, k) is read at
// src[(r / rv) * vs + (r % rv) * sr + k * sk]; padding is written as zero.
// One thread per (row, 8-wide K group): rows vary fastest across a warp
// (coalesced reads when sr == 1) and each thread stores one 16-byte core
// matrix row per plane.
__global__ void split_kernel(const double* __restrict__ src, i64 rv, i64 vs, i64 sr, i64 sk,
                             int rows, int cols, int R, int rtiles, int ktiles,
                             bf16* __restrict__ hi, bf16* __restrict__ lo) {
  pdl_trigger();
  pdl_wait();
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

// The TT-matrix core contracted into Phi2 once per local problem:
//   Q[mq, kq] = sum_a2 A(a1,i,j,a2) Phi2(b2,a2,c2),
//   mq = (i + n*c2) + n*ry2*a1, kq = j + m*b2,
// in FP64, then split and tiled as a 128-row A operand.  With Q the local
// operator's first product gives its core-contracted intermediate directly:
// T2[(i,c2,v),(b1,a1)] = sum_kq Q[(i,c2,a1), kq] X_v[b1, kq].  One thread per
// (row, 8-wide K group) as in split_kernel; padding is written as zero.
__global__ void build_q_kernel(const double* __restrict__ A, const double* __restrict__ phi2,
                               int m, int rx2, int n, int ry2, int ra1, int ra2, int rtiles,
                               int ktiles, bf16* __restrict__ hi, bf16* __restrict__ lo) {
  const int nry2 = n * ry2, MQ = nry2 * ra1, KQ = m * rx2;
  const i64 tr = (i64)rtiles * TM, tk8 = (i64)ktiles * (TK / 8);
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tr * tk8;
       e += (i64)gridDim.x * blockDim.x) {
    const int r = (int)(e % tr), k0 = (int)(e / tr) * 8;
    const int ic2 = r % nry2, a1 = r / nry2, i = ic2 % n, c2 = ic2 / n;
    __align__(16) bf16 h[8], l[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int kq = k0 + q;
      double v = 0.0;
      if (r < MQ && kq < KQ) {
        const int j = kq % m, b2 = kq / m;
        const double* a = A + a1 + (i64)ra1 * (i + (i64)n * j);   // a2 stride ra1*n*m
        const double* p2 = phi2 + b2 + (i64)rx2 * ra2 * c2;      // a2 stride rx2
        for (int a2 = 0; a2 < ra2; ++a2)
          v = fma(a[(i64)ra1 * n * m * a2], p2[(i64)rx2 * a2], v);
      }
      split2(v, h[q], l[q]);
    }
    const size_t idx = tiled_index(r, k0, TM, ktiles);
    *reinterpret_cast<uint4*>(hi + idx) = *reinterpret_cast<const uint4*>(h);
    *reinterpret_cast<uint4*>(lo + idx) = *reinterpret_cast<const uint4*>(l);
  }
}

// C[m, n] (m < M, n < N) = sum_k A[m, k] B[n, k], split-3 on tcgen05
// (NPROD = 3: hi hi + hi lo + lo hi) or plain BF16 (NPROD = 1: hi hi only,
// the lo planes are not read).
// C[m, n] goes to out[(m / rpv) * vstride + (m % rpv) * rstride + n * cstride].
// The accumulator row m sits in TMEM lane m % 128, so with rstride == 1 the
// 32 lanes of a warp store 32 consecutive elements (coalesced).
// K split: CTA z of gridDim.z takes the K tiles [z * kchunk, z * kchunk +
// kchunk) of the ktiles the operands hold and writes its partial product at
// out + z * zstride (the caller adds the partials in a fixed order).
template <int BN, int STAGES, class OutT, int NPROD = 3>
__global__ void __launch_bounds__(NTHREADS, 1)
    split_gemm_kernel(const bf16* __restrict__ Ahi, const bf16* __restrict__ Alo,
                      const bf16* __restrict__ Bhi, const bf16* __restrict__ Blo, int M, int N,
                      int ktiles, OutT* __restrict__ out, i64 rpv, i64 vstride, i64 rstride,
                      i64 cstride, int* __restrict__ err, int kchunk = 0, i64 zstride = 0) {
  static_assert(NPROD == 1 || NPROD == 3, "one or three bf16 products");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  constexpr uint32_t A_BYTES = TM * TK * 2;
  constexpr uint32_t B_BYTES = BN * TK * 2;
  constexpr uint32_t PLANES = NPROD == 3 ? 2 : 1;
  constexpr uint32_t STAGE_BYTES = PLANES * (A_BYTES + B_BYTES);
  constexpr uint32_t B_OFF = PLANES * A_BYTES;   // B hi after the A plane(s)
  const int ktot = ktiles;                        // K tiles the operands hold
  const int kt0 = kchunk > 0 ? (int)blockIdx.z * kchunk : 0;
  if (kchunk > 0) {
    ktiles = min(kchunk, ktot - kt0);
    out += (i64)blockIdx.z * zstride;
  }
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
      size_t ao = ((size_t)mt * ktot + kt0 + c) * a_tile;
      size_t bo = ((size_t)nt * ktot + kt0 + c) * b_tile;
      bulk_g2s(smem_u32(st), Ahi + ao, A_BYTES, bar);
      bulk_g2s(smem_u32(st + B_OFF), Bhi + bo, B_BYTES, bar);
      if constexpr (NPROD == 3) {
        bulk_g2s(smem_u32(st + A_BYTES), Alo + ao, A_BYTES, bar);
        bulk_g2s(smem_u32(st + B_OFF + B_BYTES), Blo + bo, B_BYTES, bar);
      }
    };
    int issued = 0, waited = 0;
    for (int c = 0; c < STAGES && c < ktiles; ++c) { issue(c, c); ++issued; }
    bool ok = true;
    for (int c = 0; c < ktiles && ok; ++c) {
      const int s = c % STAGES;
      const uint32_t ph = (uint32_t)((c / STAGES) & 1);
      if (!mbar_wait(smem_u32(&full_bar[s]), ph)) { ok = false; break; }
      ++waited;
      tc_fence_after();
      unsigned char* st = base + (size_t)s * STAGE_BYTES;
      const uint32_t a_hi = smem_u32(st), a_lo = smem_u32(st + A_BYTES);
      const uint32_t b_hi = smem_u32(st + B_OFF), b_lo = smem_u32(st + B_OFF + B_BYTES);
#pragma unroll
      for (int kk = 0; kk < TK / 16; ++kk) {
        // one 16-wide K slab per MMA
        const uint32_t aoff = kk * (TM * 32), boff = kk * (BN * 32);
        const uint64_t dAh = make_desc(a_hi + aoff, LBO, SBO);
        const uint64_t dBh = make_desc(b_hi + boff, LBO, SBO);
        mma_bf16(taddr, dAh, dBh, idesc, (c > 0 || kk > 0) ? 1u : 0u);
        if constexpr (NPROD == 3) {
          const uint64_t dAl = make_desc(a_lo + aoff, LBO, SBO);
          const uint64_t dBl = make_desc(b_lo + boff, LBO, SBO);
          mma_bf16(taddr, dAh, dBl, idesc, 1u);
          mma_bf16(taddr, dAl, dBh, idesc, 1u);
        }
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
      // ones not yet waited for (at most one per stage, each in its stage's
      // current phase) are waited for here.  The copies read valid global
      // memory and complete in microseconds, so these waits end long before
      // their limit; a drain that still gives up is reported as code 3
      bool drained = true;
      for (int c = waited; c < issued; ++c) {
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

__device__ __forceinline__ size_t tiled_index_pow2(int r, int k, int lgR, int ktiles) {
  const size_t tile = (size_t)(r >> lgR) * ktiles + (k >> 6);
  return (tile << (lgR + 6)) + (tile_offset(r & ((1 << lgR) - 1), k & (TK - 1), 1 << lgR) >> 1);
}
__device__ __forceinline__ void split2f(float v, bf16& hi, bf16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));   // v - hi is exact in FP32
}

// ---------------------------------------------------------------------------
// Persistent, warp-specialised form of the same product (same operand tile
// layout, same output addressing, same K split).  One CTA per SM walks the
// output tiles t = blockIdx.x, blockIdx.x + gridDim.x, ...; tile t is
// (mt, nt, z) with mt fastest.  Ten warps:
//   warp 0 (one lane)  bulk copies of the A/B stages into a STAGES-deep ring,
//                      running ahead across tile boundaries;
//   warp 1 (one lane)  tcgen05.mma issue; owns the tensor memory, two FP32
//                      accumulators of BN columns, used alternately by
//                      consecutive tiles of the CTA;
//   warps 2-9          epilogue: warp w reads TMEM lanes 32*(w%4).. of one
//                      half of the columns ((w-2)/4) with tcgen05.ld and
//                      stores them, while the MMAs of the next tile run on
//                      the other accumulator (eight storing warps per SM:
//                      four cannot keep enough stores in flight).
// Ring barriers: full[s] (copies landed), empty[s] (MMAs that read the stage
// done, tcgen05.commit); accumulator barriers: acc_full[a] (tile's MMAs done,
// tcgen05.commit) and acc_empty[a] (the eight epilogue warps have read it).
// Every wait is bounded and also gives up once another role has failed; a
// failing CTA records the code in *err, waits (bounded) for the copies and
// MMAs it issued and frees its tensor memory.
// ---------------------------------------------------------------------------
#ifndef TTG_WS_EPI_WARPS
#define TTG_WS_EPI_WARPS 8
#endif
constexpr int WS_EPI_WARPS = TTG_WS_EPI_WARPS;   // 4, 8 or 16
constexpr int WS_THREADS = 64 + 32 * WS_EPI_WARPS;

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_wait_f(uint32_t bar, uint32_t parity, volatile int* fail) {
  for (long long i = 0; i < WAIT_LIMIT; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63) == 63 && *fail) return false;
  }
  return false;
}

template <int BN, int NPROD>
__host__ __device__ constexpr int ws_stages() {
  // as many stages as fit in ~192 KB of shared memory (at most 8)
  return (192 * 1024) / ((NPROD == 3 ? 2 : 1) * (TM * TK * 2 + BN * TK * 2)) > 8
             ? 8
             : (192 * 1024) / ((NPROD == 3 ? 2 : 1) * (TM * TK * 2 + BN * TK * 2));
}
template <int BN, int NPROD>
__host__ __device__ constexpr size_t ws_smem() {
  return (size_t)ws_stages<BN, NPROD>() * (NPROD == 3 ? 2 : 1) * (TM * TK * 2 + BN * TK * 2) + 1024;
}

// Epilogue that writes the product, split into bf16 hi/lo, straight into the
// tiled B operand of the local operator's last product (EPI = 1): product row
// mq = (i + n*c2) + n*ry2*a1, column nx = b1 + rx1*v go to operand row
// i + n*c2 + n*ry2*v, K index b1 + rx1*a1.  rx1 is a multiple of 8, so the
// eight columns of a 16-byte core-matrix row are eight consecutive b1 of one
// v: each thread stores them as one 16-byte vector per plane.
struct EpiT2 {
  int rx1 = 8, nry2 = 1, lgR3 = 6, ktiles3 = 1;
  bf16* hi = nullptr;
  bf16* lo = nullptr;
};

template <int BN, class OutT, int NPROD = 3, int EPI = 0>
__global__ void __launch_bounds__(WS_THREADS, 1)
    split_gemm_ws_kernel(const bf16* __restrict__ Ahi, const bf16* __restrict__ Alo,
                         const bf16* __restrict__ Bhi, const bf16* __restrict__ Blo, int M, int N,
                         int ktot, int mtiles, int ntiles, int nz, OutT* __restrict__ out,
                         i64 rpv, i64 vstride, i64 rstride, i64 cstride, int* __restrict__ err,
                         int kchunk, i64 zstride, const EpiT2 ep) {
  static_assert(NPROD == 1 || NPROD == 3, "one or three bf16 products");
  static_assert(BN == 64 || BN == 128 || BN == 256, "tile width");
  constexpr int STAGES = ws_stages<BN, NPROD>();
  constexpr uint32_t A_BYTES = TM * TK * 2;
  constexpr uint32_t B_BYTES = BN * TK * 2;
  constexpr uint32_t PLANES = NPROD == 3 ? 2 : 1;
  constexpr uint32_t STAGE_BYTES = PLANES * (A_BYTES + B_BYTES);
  constexpr uint32_t B_OFF = PLANES * A_BYTES;
  constexpr uint32_t TMEM_COLS = 2 * BN;   // 128, 256 or 512: a power of two
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t acc_full[2];
  __shared__ __align__(8) uint64_t acc_empty[2];
  __shared__ __align__(8) uint64_t done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int fail_s;
  volatile int* fail = &fail_s;

  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int per_z = mtiles * ntiles, total = per_z * nz;

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(smem_u32(&acc_full[a]), 1);
      mbar_init(smem_u32(&acc_empty[a]), WS_EPI_WARPS);
    }
    mbar_init(smem_u32(&done_bar), 1);
    fail_s = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(smem_u32(&tmem_slot), TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t taddr = tmem_slot;
  // the prologue above may overlap the kernel before this one
  pdl_wait();
  pdl_trigger();

  // K tiles [k0, k0 + kn) of tile t
  auto krange = [&](int t, int& k0, int& kn) {
    if (kchunk > 0) {
      k0 = (t / per_z) * kchunk;
      kn = min(kchunk, ktot - k0);
    } else {
      k0 = 0;
      kn = ktot;
    }
  };

  if (warp == 0) {
    if (lane == 0) {
      // ---- producer ----
      const size_t a_tile = (size_t)TM * TK, b_tile = (size_t)BN * TK;
      int it = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < total && ok; t += gridDim.x) {
        const int r = t % per_z, mt = r % mtiles, nt = r / mtiles;
        int k0, kn;
        krange(t, k0, kn);
        for (int c = 0; c < kn; ++c, ++it) {
          const int s = it % STAGES;
          if (it >= STAGES &&
              !mbar_wait_f(smem_u32(&empty_bar[s]), (uint32_t)((it / STAGES - 1) & 1), fail)) {
            ok = false;
            break;
          }
          unsigned char* st = base + (size_t)s * STAGE_BYTES;
          const uint32_t bar = smem_u32(&full_bar[s]);
          mbar_expect_tx(bar, STAGE_BYTES);
          const size_t ao = ((size_t)mt * ktot + k0 + c) * a_tile;
          const size_t bo = ((size_t)nt * ktot + k0 + c) * b_tile;
          bulk_g2s(smem_u32(st), Ahi + ao, A_BYTES, bar);
          bulk_g2s(smem_u32(st + B_OFF), Bhi + bo, B_BYTES, bar);
          if constexpr (NPROD == 3) {
            bulk_g2s(smem_u32(st + A_BYTES), Alo + ao, A_BYTES, bar);
            bulk_g2s(smem_u32(st + B_OFF + B_BYTES), Blo + bo, B_BYTES, bar);
          }
        }
      }
      if (!ok) {
        *fail = 1;
        atomicExch(err, 1);
      }
      if (!ok || *fail) {
        // the last fill of each stage may not have been consumed: let it land
        bool drained = true;
        for (int s = 0; s < STAGES; ++s) {
          const int last = it - 1 - ((it - 1 - s) % STAGES + STAGES) % STAGES;
          if (last >= 0 && last < it)
            drained = mbar_wait(smem_u32(&full_bar[s]), (uint32_t)((last / STAGES) & 1)) && drained;
        }
        if (!drained) atomicExch(err, 3);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issue ----
      constexpr uint32_t idesc = make_idesc(TM, BN);
      int it = 0, lt = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < total && ok; t += gridDim.x, ++lt) {
        const int acc = lt & 1, use = lt >> 1;
        if (use > 0 && !mbar_wait_f(smem_u32(&acc_empty[acc]), (uint32_t)((use - 1) & 1), fail)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t d = taddr + (uint32_t)(acc * BN);
        int k0, kn;
        krange(t, k0, kn);
        for (int c = 0; c < kn; ++c, ++it) {
          const int s = it % STAGES;
          if (!mbar_wait_f(smem_u32(&full_bar[s]), (uint32_t)((it / STAGES) & 1), fail)) {
            ok = false;
            break;
          }
          tc_fence_after();
          unsigned char* st = base + (size_t)s * STAGE_BYTES;
          const uint32_t a_hi = smem_u32(st), a_lo = smem_u32(st + A_BYTES);
          const uint32_t b_hi = smem_u32(st + B_OFF), b_lo = smem_u32(st + B_OFF + B_BYTES);
#pragma unroll
          for (int kk = 0; kk < TK / 16; ++kk) {
            const uint32_t aoff = kk * (TM * 32), boff = kk * (BN * 32);
            const uint64_t dAh = make_desc(a_hi + aoff, LBO, SBO);
            const uint64_t dBh = make_desc(b_hi + boff, LBO, SBO);
            mma_bf16(d, dAh, dBh, idesc, (c > 0 || kk > 0) ? 1u : 0u);
            if constexpr (NPROD == 3) {
              mma_bf16(d, dAh, make_desc(b_lo + boff, LBO, SBO), idesc, 1u);
              mma_bf16(d, make_desc(a_lo + aoff, LBO, SBO), dBh, idesc, 1u);
            }
          }
          mma_commit(smem_u32(&empty_bar[s]));
        }
        if (!ok) break;
        mma_commit(smem_u32(&acc_full[acc]));
      }
      if (!ok) {
        *fail = 1;
        atomicExch(err, 1);
      }
      // every MMA this thread issued has completed once done_bar flips
      mma_commit(smem_u32(&done_bar));
      if (!mbar_wait(smem_u32(&done_bar), 0)) atomicExch(err, 2);
    }
    __syncwarp();
  } else {
    // ---- epilogue ----
    const int q = warp & 3;   // TMEM lane quadrant this warp may read
    constexpr int CW = BN / (WS_EPI_WARPS / 4);   // columns per epilogue warp
    static_assert(CW % 16 == 0, "epilogue column share");
    const int cb = ((warp - 2) >> 2) * CW, ce = cb + CW;   // its columns
    int lt = 0;
    for (int t = blockIdx.x; t < total; t += gridDim.x, ++lt) {
      const int acc = lt & 1, use = lt >> 1;
      const bool got = __all_sync(0xffffffffu,
                                  mbar_wait_f(smem_u32(&acc_full[acc]), (uint32_t)(use & 1), fail));
      if (!got) {
        if (lane == 0) {
          *fail = 1;
          atomicExch(err, 1);
        }
        break;
      }
      tc_fence_after();
      const int r = t % per_z, mt = r % mtiles, nt = r / mtiles;
      const int row = mt * TM + q * 32 + lane;
      const int n0 = nt * BN;
      const uint32_t tbase = taddr + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN);
      if constexpr (EPI == 1) {
        // operand row base (i + n*c2) and K base rx1*a1 of this product row
        const int ic2 = row % ep.nry2, kb = ep.rx1 * (row / ep.nry2);
#pragma unroll 1
        for (int c0 = cb; c0 < ce; c0 += 16) {
          uint32_t v[16];
          tmem_ld16(tbase + (uint32_t)c0, v);
          tmem_ld_wait();
          if (c0 + 16 >= ce) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&acc_empty[acc]));
          }
          if (row < M) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const int nx = n0 + c0 + 8 * h;   // multiple of 8: eight b1 of one v
              if (nx < N) {
                const int vv = nx / ep.rx1, b1 = nx - vv * ep.rx1;
                const size_t idx =
                    tiled_index_pow2(ic2 + ep.nry2 * vv, b1 + kb, ep.lgR3, ep.ktiles3);
                __align__(16) bf16 hh[8], ll[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) split2f(__uint_as_float(v[8 * h + e]), hh[e], ll[e]);
                *reinterpret_cast<uint4*>(ep.hi + idx) = *reinterpret_cast<const uint4*>(hh);
                *reinterpret_cast<uint4*>(ep.lo + idx) = *reinterpret_cast<const uint4*>(ll);
              }
            }
          }
        }
        continue;
      }
      OutT* o = out + (i64)(t / per_z) * zstride;
      OutT* orow = o + (row / rpv) * vstride + (row % rpv) * rstride;
#pragma unroll 1
      for (int c0 = cb; c0 < ce; c0 += 16) {
        uint32_t v[16];
        tmem_ld16(tbase + (uint32_t)c0, v);
        tmem_ld_wait();
        if (c0 + 16 >= ce) {
          // this warp's share of the accumulator is in registers: hand it back
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&acc_empty[acc]));
        }
        if (row < M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int n = n0 + c0 + j;
            if (n < N) orow[(i64)n * cstride] = (OutT)__uint_as_float(v[j]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(taddr, TMEM_COLS);
}

// CORE: T2[(i,c2,v),(b1,a1)] = sum_(j,a2) A[(a1,i),(j,a2)] T1[(b1,j,v),(a2,c2)]
// T1 is column-major with leading dimension ld1 over the rows (b1,j,v), so
// b1 is contiguous; the result is written split and tiled as the B operand of
// GEMM3 (rows (i,c2,v), K (b1,a1), tile rows 1 << lgR3).

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
  pdl_trigger();
  pdl_wait();
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

// ---------------------------------------------------------------------------
// Fused small local operator: GEMM1, the core contraction and GEMM3 of one
// (vector, block of c2) in a single CTA, with every intermediate on chip.
// For local problems whose X_v fits one 128-row tile (rx1*m <= 128, rx2 <= 64,
// ry1 <= 128) and whose TT-matrix core is small (m*ra2, n*ra1 <= 16, n == m)
// -- the tt_eigb sizes up to r = 64 -- the four launches of the general path
// (X split, GEMM1, CORE, GEMM3) and the T1/T2 round trips through memory
// become one launch:
//
//   1. X_v (FP64) is split into bf16 hi/lo straight into shared memory, rows
//      rho = j + m*b1 (j fastest, so every b1's m rows sit in one tile),
//      while the Phi2 tile of the CTA (rows kappa = a2 + ra2*c2l for the C
//      values of c2 the CTA owns) and the first Phi1 tiles land by bulk copy;
//   2. GEMM1 D1[rho, kappa] = sum_b2 X[rho, b2] Phi2[kappa, b2] on tcgen05
//      (BF16x3, FP32 in TMEM);
//   3. D1 goes TMEM -> registers -> shared memory; thread (b1, j) forms
//      T2[(i = j, c2l), (b1, a1)] = sum_(j', a2) A[a1, i, j', a2] D1[(j', b1), (a2, c2l)]
//      reading its own and its partners' rows, and writes it split into the
//      shared-memory B operand of GEMM3 (rows (i, c2l), K = (b1, a1));
//   4. GEMM3 D3[c1, (i, c2l)] = sum_(b1,a1) Phi1[c1, (b1,a1)] T2[(i,c2l), (b1,a1)]
//      with the Phi1 tiles streamed through two stages;
//   5. y[c1 + ry1 (i + n c2)] of vector v is stored from TMEM (lane = c1).
// ---------------------------------------------------------------------------
// dynamic shared memory bound of the fused kernel: the 227 KB a CTA may opt
// into, less the kernel's static shared memory (barriers, 1024-aligned)
constexpr int FUSED_MAX_SMEM = 225 * 1024;

struct FusedArgs {
  const double* x;          // x[v*xs + b1 + rx1*(j + m*b2)]
  double* y;                // y[v*ys + c1 + ry1*(i + n*c2)]
  const bf16 *p2hi, *p2lo;  // Phi2 tiles (BN1 rows kappa, 64 K = b2), one per block of c2
  const bf16 *p1hi, *p1lo;  // Phi1 tiles (128 rows c1, K = b1 + rx1*a1), k3tiles of them
  int rx1, m, rx2, ry1, n, ry2, ra1, ra2;
  int C;                    // values of c2 per CTA
  int k3tiles;              // ceil(rx1*ra1 / 64)
  i64 xs, ys;               // vector strides
  int* err;
  // A(a1,i,j,a2) at a[q * NA + p], p = a1 + ra1*i, q = j + m*a2, zero
  // outside p < n*ra1, q < m*ra2 (NA: the kernel's compile-time bound)
  float a[256];
};

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// shared memory plan of fused_small_kernel (bytes from the 1024-aligned base)
__host__ __device__ constexpr size_t fused_r0(int bn1) {
  // GEMM1 operands (X and Phi2 tiles, hi and lo) and, after GEMM1, the FP32
  // copy of D1 with rows of bn1 + 1 floats
  return (((size_t)2 * TM * TK * 2 + (size_t)2 * bn1 * TK * 2) > (size_t)TM * (bn1 + 1) * 4
              ? ((size_t)2 * TM * TK * 2 + (size_t)2 * bn1 * TK * 2)
              : (size_t)TM * (bn1 + 1) * 4 + 1023) & ~(size_t)1023;
}
__host__ __device__ constexpr size_t fused_t2(int n3p, int k3tiles) {
  return (size_t)2 * n3p * TK * 2 * k3tiles;   // hi and lo planes
}
constexpr size_t FUSED_P1_STAGE = (size_t)2 * TM * TK * 2;
__host__ __device__ constexpr size_t fused_smem(int bn1, int n3p, int k3tiles) {
  return fused_r0(bn1) + fused_t2(n3p, k3tiles) + 2 * FUSED_P1_STAGE + 1024;
}

template <int BN1, int N3P, int JA, int NA>
__global__ void __launch_bounds__(NTHREADS, 1) fused_small_kernel(const __grid_constant__ FusedArgs g) {
  static_assert(JA * NA <= 256, "core coefficients exceed the parameter array");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_p2, bar_mma1, bar_mma3;
  __shared__ __align__(8) uint64_t full3[2], empty3[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int fail;

  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA1 = base;                                  // X tile, hi then lo
  unsigned char* sB1 = base + 2 * TM * TK * 2;                // Phi2 tile, hi then lo
  float* sD1 = (float*)base;                                  // after GEMM1
  unsigned char* sT2 = base + fused_r0(BN1);                  // GEMM3 B operand
  const size_t t2plane = (size_t)N3P * TK * 2 * g.k3tiles;
  unsigned char* sP1 = sT2 + 2 * t2plane;                     // two Phi1 stages
  constexpr int LD1 = BN1 + 1;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nt = blockIdx.x, v = blockIdx.y;
  const int c20 = nt * g.C;
  const int ncol = min(g.C, g.ry2 - c20);     // valid c2 of this CTA
  const int na = g.n * g.ra1;

  if (tid == 0) {
    mbar_init(smem_u32(&bar_p2), 1);
    mbar_init(smem_u32(&bar_mma1), 1);
    mbar_init(smem_u32(&bar_mma3), 1);
    for (int s = 0; s < 2; ++s) {
      mbar_init(smem_u32(&full3[s]), 1);
      mbar_init(smem_u32(&empty3[s]), 1);
    }
    fail = 0;
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(smem_u32(&tmem_slot), 256);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t taddr = tmem_slot;
  constexpr uint32_t B1_BYTES = BN1 * TK * 2, A_BYTES = TM * TK * 2;

  // bulk copies: the Phi2 tile and the first two Phi1 tiles
  int p1_issued = 0;
  auto issue_p1 = [&](int c, int s) {
    unsigned char* st = sP1 + (size_t)s * FUSED_P1_STAGE;
    const uint32_t bar = smem_u32(&full3[s]);
    mbar_expect_tx(bar, 2 * A_BYTES);
    const size_t off = (size_t)c * TM * TK;
    bulk_g2s(smem_u32(st), g.p1hi + off, A_BYTES, bar);
    bulk_g2s(smem_u32(st + A_BYTES), g.p1lo + off, A_BYTES, bar);
  };
  if (tid == 0) {
    const uint32_t bar = smem_u32(&bar_p2);
    mbar_expect_tx(bar, 2 * B1_BYTES);
    const size_t off = (size_t)nt * BN1 * TK;
    bulk_g2s(smem_u32(sB1), g.p2hi + off, B1_BYTES, bar);
    bulk_g2s(smem_u32(sB1 + B1_BYTES), g.p2lo + off, B1_BYTES, bar);
    for (int c = 0; c < 2 && c < g.k3tiles; ++c) { issue_p1(c, c); ++p1_issued; }
  }

  // (1) X_v -> sA1, rows rho = j + m*b1, K = b2; one 16-byte core-matrix row
  // of each plane per item; zero outside rho < rx1*m, b2 < rx2
  {
    // thread tid owns row rho = tid; its 64 elements (b2 = 0..63) are loaded
    // in two batches of 32 independent loads before any conversion, so the
    // global-memory latency is paid twice, not 64 times
    const double* __restrict__ xv = g.x + (i64)v * g.xs;
    const int rho = tid;
    const int j = rho % g.m, b1 = rho / g.m;
    const bool row_ok = rho < g.rx1 * g.m;
    const double* __restrict__ xr = xv + b1 + (i64)g.rx1 * j;
    const i64 kstride = (i64)g.rx1 * g.m;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      double val[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const int k = half * 32 + q;
        val[q] = (row_ok && k < g.rx2) ? xr[kstride * k] : 0.0;
      }
#pragma unroll
      for (int gq = 0; gq < 4; ++gq) {
        __align__(16) bf16 h[8], l[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          // every CTA of a vector splits the whole X_v, so the conversion
          // stays on the integer pipe (truncation: |v - f| < 2^-23 |v|)
          const float f = d2f_trunc(val[gq * 8 + q]);
          h[q] = __float2bfloat16_rn(f);
          l[q] = __float2bfloat16_rn(f - __bfloat162float(h[q]));
        }
        const uint32_t off = tile_offset(rho, half * 32 + gq * 8, TM);
        *reinterpret_cast<uint4*>(sA1 + off) = *reinterpret_cast<const uint4*>(h);
        *reinterpret_cast<uint4*>(sA1 + A_BYTES + off) = *reinterpret_cast<const uint4*>(l);
      }
    }
    // zero the padding of the GEMM3 B operand (rows past n*ncol, K columns
    // past rx1*ra1): those 16-byte row pieces meet zero rows or columns of
    // the products, and 0 * garbage could be NaN.  The core writes the rest.
    const int nrow = g.n * ncol, kvalid = g.rx1 * g.ra1, kg = g.k3tiles * (TK / 8);
    for (int e = tid; e < N3P * kg; e += NTHREADS) {
      const int r = e % N3P, k0 = (e / N3P) * 8;
      if (r < nrow && k0 + 8 <= kvalid) continue;
      const uint32_t o = (uint32_t)(k0 >> 6) * (N3P * TK * 2) + tile_offset(r, k0 & 63, N3P);
      *reinterpret_cast<uint4*>(sT2 + o) = make_uint4(0u, 0u, 0u, 0u);
      *reinterpret_cast<uint4*>(sT2 + t2plane + o) = make_uint4(0u, 0u, 0u, 0u);
    }
  }
  fence_proxy_async();
  __syncthreads();

  // (2) GEMM1 into TMEM columns [0, BN1)
  bool p2_ok = true;    // thread 0: the Phi2 copy was waited for
  if (tid == 0) {
    if (!mbar_wait(smem_u32(&bar_p2), 0)) {
      p2_ok = false;
      fail = 1;
      atomicExch(g.err, 4);
    } else {
      tc_fence_after();
      constexpr uint32_t idesc = make_idesc(TM, BN1);
      const uint32_t a_hi = smem_u32(sA1), a_lo = a_hi + A_BYTES;
      const uint32_t b_hi = smem_u32(sB1), b_lo = b_hi + B1_BYTES;
#pragma unroll
      for (int kk = 0; kk < TK / 16; ++kk) {
        const uint32_t aoff = kk * (TM * 32), boff = kk * (BN1 * 32);
        const uint64_t dAh = make_desc(a_hi + aoff, LBO, SBO), dAl = make_desc(a_lo + aoff, LBO, SBO);
        const uint64_t dBh = make_desc(b_hi + boff, LBO, SBO), dBl = make_desc(b_lo + boff, LBO, SBO);
        mma_bf16(taddr, dAh, dBh, idesc, kk > 0 ? 1u : 0u);
        mma_bf16(taddr, dAh, dBl, idesc, 1u);
        mma_bf16(taddr, dAl, dBh, idesc, 1u);
      }
    }
    mma_commit(smem_u32(&bar_mma1));
  }
  __syncwarp();
  if (!mbar_wait(smem_u32(&bar_mma1), 0)) { fail = 1; atomicExch(g.err, 5); }
  tc_fence_after();
  __syncthreads();
  const bool ok1 = fail == 0;

  // (3) D1 -> shared memory (row rho = this thread's TMEM lane), then the
  // core contraction into the split GEMM3 operand
  if (ok1) {
    const int rho = warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN1; c0 += 16) {
      uint32_t r[16];
      tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
      tmem_ld_wait();
#pragma unroll
      for (int q = 0; q < 16; ++q) sD1[rho * LD1 + c0 + q] = __uint_as_float(r[q]);
    }
  }
  __syncthreads();
  if (ok1) {
    // thread (b1, j) forms every output p = (a1, i) of its b1 for the c2
    // values c2l = j, j + m, ...: the JA inputs of a c2 come from the m rows
    // of b1 in shared memory, the NA outputs are independent FMA chains with
    // the core coefficients as compile-time-indexed constants
    const int rho = tid;
    const int j = rho % g.m, b1 = rho / g.m;
    const int ja = g.m * g.ra2, na = g.n * g.ra1;
    if (b1 < g.rx1) {
      const float* rows0 = sD1 + (size_t)(g.m * b1) * LD1;
      int off[JA];
#pragma unroll
      for (int q = 0; q < JA; ++q) off[q] = (q % g.m) * LD1 + q / g.m;
      // per output p = (a1, i): its row i and the K part (k3 = b1 + rx1*a1)
      // of its byte offset in the tiled operand, computed once
      int ip[NA];
      uint32_t koff[NA];
#pragma unroll
      for (int p = 0; p < NA; ++p) {
        const int i = p / g.ra1, a1 = p - i * g.ra1;
        const int k3 = b1 + g.rx1 * a1, kk = k3 & 63;
        ip[p] = i;
        koff[p] = (uint32_t)(k3 >> 6) * (N3P * TK * 2) + (uint32_t)(kk >> 4) * (N3P * 32) +
                  (uint32_t)((kk >> 3) & 1) * 128 + (uint32_t)(kk & 7) * 2;
      }
      const uint32_t plane = (uint32_t)t2plane;
#pragma unroll 1
      for (int c2l = j; c2l < ncol; c2l += g.m) {
        const float* rc = rows0 + g.ra2 * c2l;
        const int rbase = g.n * c2l;
        float t[JA];
#pragma unroll
        for (int q = 0; q < JA; ++q) t[q] = q < ja ? rc[off[q]] : 0.f;
        // all NA chains unconditionally (the coefficients are zero past na),
        // q outer so the NA accumulators are independent FMA chains
        float acc[NA];
#pragma unroll
        for (int p = 0; p < NA; ++p) acc[p] = 0.f;
#pragma unroll
        for (int q = 0; q < JA; ++q)
#pragma unroll
          for (int p = 0; p < NA; ++p) acc[p] = fmaf(g.a[q * NA + p], t[q], acc[p]);
#pragma unroll
        for (int p = 0; p < NA; ++p) {
          if (p < na) {
            const int r3 = ip[p] + rbase;
            bf16 h, l;
            split2f(acc[p], h, l);
            const uint32_t o = koff[p] + (uint32_t)(r3 >> 3) * 256 + (uint32_t)(r3 & 7) * 16;
            *reinterpret_cast<bf16*>(sT2 + o) = h;
            *reinterpret_cast<bf16*>(sT2 + plane + o) = l;
          }
        }
      }
    }
  }
  fence_proxy_async();
  __syncthreads();

  // (4) GEMM3 into TMEM columns [BN1, BN1 + N3P), Phi1 tiles through two stages
  if (tid == 0) {
    bool ok = ok1;
    int p1_waited = 0;
    if (ok) {
      constexpr uint32_t idesc = make_idesc(TM, N3P);
      const uint32_t t2hi = smem_u32(sT2), t2lo = t2hi + (uint32_t)t2plane;
      for (int c = 0; c < g.k3tiles && ok; ++c) {
        const int s = c & 1;
        const uint32_t ph = (uint32_t)((c >> 1) & 1);
        if (!mbar_wait(smem_u32(&full3[s]), ph)) { ok = false; break; }
        ++p1_waited;
        tc_fence_after();
        const uint32_t a_hi = smem_u32(sP1 + (size_t)s * FUSED_P1_STAGE), a_lo = a_hi + A_BYTES;
        const uint32_t bt = (uint32_t)c * (N3P * TK * 2);
#pragma unroll
        for (int kk = 0; kk < TK / 16; ++kk) {
          const uint32_t aoff = kk * (TM * 32), boff = bt + kk * (N3P * 32);
          const uint64_t dAh = make_desc(a_hi + aoff, LBO, SBO), dAl = make_desc(a_lo + aoff, LBO, SBO);
          const uint64_t dBh = make_desc(t2hi + boff, LBO, SBO), dBl = make_desc(t2lo + boff, LBO, SBO);
          mma_bf16(taddr + BN1, dAh, dBh, idesc, (c > 0 || kk > 0) ? 1u : 0u);
          mma_bf16(taddr + BN1, dAh, dBl, idesc, 1u);
          mma_bf16(taddr + BN1, dAl, dBh, idesc, 1u);
        }
        mma_commit(smem_u32(&empty3[s]));
        if (c + 2 < g.k3tiles) {
          if (!mbar_wait(smem_u32(&empty3[s]), ph)) { ok = false; break; }
          issue_p1(c + 2, s);
          ++p1_issued;
        }
      }
    }
    if (!ok) {
      fail = 1;
      atomicExch(g.err, 6);
    }
    // every bulk copy this CTA issued lands before it can exit: the copies
    // not yet waited for (at most one per stage, each in its stage's current
    // phase) are waited for here.  They read valid global memory and complete
    // in microseconds; a drain that still gives up is its own code.
    bool drained = true;
    if (!p2_ok) drained = mbar_wait(smem_u32(&bar_p2), 0);
    for (int c = p1_waited; c < p1_issued; ++c)
      drained = mbar_wait(smem_u32(&full3[c & 1]), (uint32_t)((c >> 1) & 1)) && drained;
    if (!drained) atomicExch(g.err, 3);
    mma_commit(smem_u32(&bar_mma3));
  }
  __syncwarp();
  const bool done3 = mbar_wait(smem_u32(&bar_mma3), 0);
  tc_fence_after();
  if (!done3) {
    fail = 1;
    if (lane == 0) atomicExch(g.err, 2);
  }
  __syncthreads();

  // (5) y of vector v: TMEM lane = c1 (coalesced stores along c1); the
  // condition is CTA-uniform, so every warp's tcgen05.ld is converged
  if (fail == 0) {
    const int c1 = warp * 32 + lane;
    double* yv = g.y + (i64)v * g.ys;
    const int cols = g.n * ncol;
#pragma unroll 1
    for (int c0 = 0; c0 < N3P; c0 += 16) {
      if (c0 >= cols) break;
      uint32_t r[16];
      tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)(BN1 + c0), r);
      tmem_ld_wait();
      if (c1 < g.ry1) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int col = c0 + q;
          if (col < cols) {
            const int i = col % g.n, c2 = c20 + col / g.n;
            yv[c1 + (i64)g.ry1 * (i + (i64)g.n * c2)] = (double)__uint_as_float(r[q]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(taddr, 256);
}

// Phi2 rows for the fused kernel: tile t row kappa < ra2*C is (a2, c2) =
// (kappa % ra2, t*C + kappa / ra2), K = b2; Phi2[b2, a2, c2] at
// phi2[b2 + rx2*(a2 + ra2*c2)]; other rows, c2 >= ry2 and b2 >= rx2 are zero
__global__ void split_p2_fused_kernel(const double* __restrict__ phi2, int rx2, int ra2, int ry2,
                                      int C, int bn1, int ntiles, bf16* __restrict__ hi,
                                      bf16* __restrict__ lo) {
  const i64 total = (i64)ntiles * bn1 * (TK / 8);
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total;
       e += (i64)gridDim.x * blockDim.x) {
    const int r = (int)(e % ((i64)ntiles * bn1)), k0 = (int)(e / ((i64)ntiles * bn1)) * 8;
    const int t = r / bn1, kappa = r % bn1;
    const int a2 = kappa % ra2, c2 = t * C + kappa / ra2;
    const bool row_ok = kappa < ra2 * C && c2 < ry2;
    __align__(16) bf16 h[8], l[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      double val = 0.0;
      if (row_ok && k0 + q < rx2) val = phi2[(k0 + q) + (i64)rx2 * (a2 + (i64)ra2 * c2)];
      split2(val, h[q], l[q]);
    }
    const size_t idx = (size_t)t * bn1 * TK + (tile_offset(kappa, k0, bn1) >> 1);
    *reinterpret_cast<uint4*>(hi + idx) = *reinterpret_cast<const uint4*>(h);
    *reinterpret_cast<uint4*>(lo + idx) = *reinterpret_cast<const uint4*>(l);
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
  pdl_trigger();
  pdl_wait();
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
  pdl_trigger();
  pdl_wait();
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

static bool use_ws() {
  static const bool on = [] {
    const char* v = std::getenv("TTG_GEMM_WS");
    return !(v && v[0] == '0');
  }();
  return on;
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
    const int per_sm = use_ws() ? 1 : (int)std::max<size_t>(1, 228 * 1024 / (smem_for(bn) + 1024));
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
  launch_pdl(split_kernel, dim3(blocks), dim3(256), 0, s, src, rv, vs, sr, sk, t.rows, t.cols, t.R,
             t.rtiles, t.ktiles, t.hi, t.lo);
}

// persistent launch: one CTA per SM, at most one per output tile
template <int BN, class OutT, int NPROD, int EPI = 0>
static void ws_launch(const bf16* Ahi, const bf16* Alo, const bf16* Bhi, const bf16* Blo, int M,
                      int N, int ktot, int mtiles, int ntiles, int nz, OutT* out, i64 rpv,
                      i64 vstride, i64 rstride, i64 cstride, int* err, int kchunk, i64 zstride,
                      cudaStream_t s, const EpiT2& ep = EpiT2()) {
  constexpr size_t smem = ws_smem<BN, NPROD>();
  auto kern = split_gemm_ws_kernel<BN, OutT, NPROD, EPI>;
  static const cudaError_t attr_rc =
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  TTG_CUDA(attr_rc);
  const i64 total = (i64)mtiles * ntiles * nz;
  TTG_REQUIRE(total < (1ll << 31), "split gemm: too many tiles");
  const int grid = (int)std::min<i64>(total, num_sms());
  launch_pdl(kern, dim3(grid), dim3(WS_THREADS), smem, s, Ahi, Alo, Bhi, Blo, M, N, ktot, mtiles,
             ntiles, nz, out, rpv, vstride, rstride, cstride, err, kchunk, zstride, ep);
}

template <int BN, class OutT>
static void gemm_launch_bn(const Tiled& A, const Tiled& B, int M, int N, OutT* out, i64 rpv,
                           i64 vstride, i64 rstride, i64 cstride, int* err, cudaStream_t s) {
  if (use_ws()) {
    ws_launch<BN, OutT, 3>(A.hi, A.lo, B.hi, B.lo, M, N, A.ktiles, A.rtiles, B.rtiles, 1, out, rpv,
                           vstride, rstride, cstride, err, 0, 0, s);
    return;
  }
  constexpr int STAGES = stages_for(BN);
  constexpr size_t smem = smem_for(BN) + SMEM_PAD;
  auto kern = split_gemm_kernel<BN, STAGES, OutT>;
  static const cudaError_t attr_rc =
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  TTG_CUDA(attr_rc);
  dim3 grid(A.rtiles, B.rtiles);
  kern<<<grid, NTHREADS, smem, s>>>(A.hi, A.lo, B.hi, B.lo, M, N, A.ktiles, out, rpv, vstride,
                                    rstride, cstride, err, 0, 0);
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

// product whose epilogue writes the split T2 operand (EPI = 1)
static void gemm_launch_t2(const Tiled& A, const Tiled& B, int M, int N, const EpiT2& ep, int* err,
                           cudaStream_t s) {
  TTG_REQUIRE(A.ktiles == B.ktiles, "split gemm: K tiles differ");
  TTG_REQUIRE(A.R == TM, "split gemm: A tiles must have 128 rows");
  TTG_REQUIRE(ep.rx1 % 8 == 0 && N % 8 == 0, "split gemm: T2 epilogue needs rx1 % 8 == 0");
  float* none = nullptr;
  if (B.R == 256)
    ws_launch<256, float, 3, 1>(A.hi, A.lo, B.hi, B.lo, M, N, A.ktiles, A.rtiles, B.rtiles, 1, none,
                                1ll << 40, 0, 1, 0, err, 0, 0, s, ep);
  else if (B.R == 128)
    ws_launch<128, float, 3, 1>(A.hi, A.lo, B.hi, B.lo, M, N, A.ktiles, A.rtiles, B.rtiles, 1, none,
                                1ll << 40, 0, 1, 0, err, 0, 0, s, ep);
  else
    ws_launch<64, float, 3, 1>(A.hi, A.lo, B.hi, B.lo, M, N, A.ktiles, A.rtiles, B.rtiles, 1, none,
                               1ll << 40, 0, 1, 0, err, 0, 0, s, ep);
}

// ---------------------------------------------------------------------------
// Plain BF16 tensor-core GEMM on FP32 operands (the learned network's layers):
//   C[m, n] = sum_k A(m, k) B(n, k),  A(m, k) = a[m*sam + k*sak],
//   B(n, k) = b[n*sbn + k*sbk],  C[m, n] -> c[m*scm + n*scn]   (FP32),
// each operand rounded once to bf16 into the tcgen05 tile layout, products
// accumulated in FP32 in TMEM (NPROD = 1 instance of split_gemm_kernel).
// K is split over CTAs when the output tiles leave SMs idle; the partial
// products are added in a fixed order (deterministic).
// ---------------------------------------------------------------------------
__global__ void tile_f32_kernel(const float* __restrict__ src, i64 sr, i64 sk, int rows, int cols,
                                int R, int rtiles, int ktiles, bf16* __restrict__ out) {
  const i64 tr = (i64)rtiles * R, tk8 = (i64)ktiles * (TK / 8);
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tr * tk8;
       e += (i64)gridDim.x * blockDim.x) {
    const int r = (int)(e % tr), k0 = (int)(e / tr) * 8;
    __align__(16) bf16 h[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      float v = 0.f;
      if (r < rows && k0 + q < cols) v = src[(i64)r * sr + (i64)(k0 + q) * sk];
      h[q] = __float2bfloat16_rn(v);
    }
    *reinterpret_cast<uint4*>(out + tiled_index(r, k0, R, ktiles)) =
        *reinterpret_cast<const uint4*>(h);
  }
}

__global__ void sum_partials_kernel(const float* __restrict__ part, int nz, int M, int N,
                                    float* __restrict__ c, i64 scm, i64 scn) {
  const i64 total = (i64)M * N;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total;
       e += (i64)gridDim.x * blockDim.x) {
    float acc = 0.f;
    for (int z = 0; z < nz; ++z) acc += part[(i64)z * total + e];
    const int m = (int)(e % M), n = (int)(e / M);
    c[(i64)m * scm + (i64)n * scn] = acc;
  }
}

constexpr int BF_BN = 128, BF_STAGES = 3;
constexpr size_t BF_SMEM = (size_t)BF_STAGES * ((size_t)TM * TK * 2 + (size_t)BF_BN * TK * 2) + 1024;

struct Bf16Plan {
  int mt, nt, kt, nz, kchunk;
  size_t abytes, bbytes, pbytes;
};
static Bf16Plan bf16_plan(int M, int N, int K) {
  Bf16Plan p;
  p.mt = ceil_div(M, TM);
  p.nt = ceil_div(N, BF_BN);
  p.kt = ceil_div(K, TK);
  const i64 base = (i64)p.mt * p.nt;
  int z = base >= 2 * 152 ? 1 : (int)std::min<i64>(p.kt, ceil_div((i64)2 * 152, base));
  p.kchunk = ceil_div(p.kt, std::max(1, z));
  p.nz = ceil_div(p.kt, p.kchunk);
  p.abytes = ((size_t)p.mt * TM * p.kt * TK * 2 + 1023) & ~size_t(1023);
  p.bbytes = ((size_t)p.nt * BF_BN * p.kt * TK * 2 + 1023) & ~size_t(1023);
  p.pbytes = p.nz > 1 ? (((size_t)p.nz * M * N * 4 + 1023) & ~size_t(1023)) : 0;
  return p;
}

size_t bf16_gemm_ws_impl(int M, int N, int K) {
  const Bf16Plan p = bf16_plan(M, N, K);
  return p.abytes + p.bbytes + p.pbytes + 1024;
}

void bf16_gemm_impl(int M, int N, int K, const float* a, i64 sam, i64 sak, const float* b,
                    i64 sbn, i64 sbk, float* c, i64 scm, i64 scn, void* ws, int* err,
                    cudaStream_t s) {
  if (M <= 0 || N <= 0) return;
  TTG_REQUIRE(K > 0, "bf16 gemm: K must be positive");
  const Bf16Plan p = bf16_plan(M, N, K);
  TTG_REQUIRE(p.nt < 65536 && p.nz < 65536, "bf16 gemm: grid too large");
  char* w = (char*)ws;
  bf16* at = (bf16*)w;
  bf16* bt = (bf16*)(w + p.abytes);
  float* part = p.nz > 1 ? (float*)(w + p.abytes + p.bbytes) : nullptr;
  {
    const i64 tot = (i64)p.mt * TM * p.kt * (TK / 8);
    tile_f32_kernel<<<(int)std::min<i64>(8192, (tot + 255) / 256), 256, 0, s>>>(
        a, sam, sak, M, K, TM, p.mt, p.kt, at);
    TTG_CHECK_LAUNCH();
  }
  {
    const i64 tot = (i64)p.nt * BF_BN * p.kt * (TK / 8);
    tile_f32_kernel<<<(int)std::min<i64>(8192, (tot + 255) / 256), 256, 0, s>>>(
        b, sbn, sbk, N, K, BF_BN, p.nt, p.kt, bt);
    TTG_CHECK_LAUNCH();
  }
  if (use_ws()) {
    if (p.nz > 1) {
      ws_launch<BF_BN, float, 1>(at, at, bt, bt, M, N, p.kt, p.mt, p.nt, p.nz, part, 1ll << 40, 0,
                                 1, M, err, p.kchunk, (i64)M * N, s);
      const i64 tot = (i64)M * N;
      sum_partials_kernel<<<(int)std::min<i64>(4096, (tot + 255) / 256), 256, 0, s>>>(
          part, p.nz, M, N, c, scm, scn);
      TTG_CHECK_LAUNCH();
    } else {
      ws_launch<BF_BN, float, 1>(at, at, bt, bt, M, N, p.kt, p.mt, p.nt, 1, c, 1ll << 40, 0, scm,
                                 scn, err, 0, 0, s);
    }
    return;
  }
  auto kern = split_gemm_kernel<BF_BN, BF_STAGES, float, 1>;
  static const cudaError_t attr_rc =
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BF_SMEM);
  TTG_CUDA(attr_rc);
  dim3 grid(p.mt, p.nt, p.nz);
  if (p.nz > 1) {
    // partial z at part + z*M*N, column-major (m fastest)
    kern<<<grid, NTHREADS, BF_SMEM, s>>>(at, at, bt, bt, M, N, p.kt, part, 1ll << 40, 0, 1, M,
                                         err, p.kchunk, (i64)M * N);
    TTG_CHECK_LAUNCH();
    const i64 tot = (i64)M * N;
    sum_partials_kernel<<<(int)std::min<i64>(4096, (tot + 255) / 256), 256, 0, s>>>(
        part, p.nz, M, N, c, scm, scn);
    TTG_CHECK_LAUNCH();
  } else {
    kern<<<grid, NTHREADS, BF_SMEM, s>>>(at, at, bt, bt, M, N, p.kt, c, 1ll << 40, 0, scm, scn,
                                         err, 0, 0);
    TTG_CHECK_LAUNCH();
  }
}

// Tile-width autotuner.  The first product of each shape class (tile counts
// ceil(M/128), ceil(N/64), ceil(K/64) and the output type) times the three
// tile widths on zeroed operands of that shape, three launches each after a
// warm-up, with CUDA events on the caller's stream, and keeps the fastest;
// later products of the class reuse it.  The cost model above is the choice
// while a stream is being captured into a graph and when TTG_AUTOTUNE=0;
// TTG_AUTOTUNE=2 prints each choice; TTG_SPLIT_BN fixes the width instead.
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
  // TTG_SPLIT_BN=64|128|256 fixes the tile width of every split product
  static const int forced = [] {
    const char* v = std::getenv("TTG_SPLIT_BN");
    const int b = v ? std::atoi(v) : 0;
    return (b == 64 || b == 128 || b == 256) ? b : 0;
  }();
  if (forced) return forced;
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

size_t bf16_gemm_ws(int M, int N, int K) { return tc::bf16_gemm_ws_impl(M, N, K); }
void bf16_gemm(int M, int N, int K, const float* a, i64 sam, i64 sak, const float* b, i64 sbn,
               i64 sbk, float* c, i64 scm, i64 scn, void* ws, int* err, cudaStream_t s) {
  tc::bf16_gemm_impl(M, N, K, a, sam, sak, b, sbn, sbk, c, scm, scn, ws, err, s);
}

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
  // core-contracted path: Q = A x Phi2 built at prepare, one product writes
  // the last product's operand (no T1, no CORE launch); X tiled as its B
  // operand (rows (b1,v), K (j,b2))
  bool pre = false;
  tc::Tiled Q;
  // fused single-launch path (fused_small_kernel) when the shape allows it
  bool fused = false;
  int fbn1 = 0, fn3p = 0, fC = 0, fntiles = 0;
  tc::bf16 *p2f_hi = nullptr, *p2f_lo = nullptr;
};

// Tile widths of the fused path for a local problem, or false when the shape
// needs the general four-launch path: X_v in one 128-row tile (rx1*m <= 128,
// rx2 <= 64), Phi1 in one 128-row tile (ry1 <= 128), a small square core
// (n == m, m*ra2 and n*ra1 <= 16) and the shared memory plan within 227 KB.
// The narrow tiles (64 columns of GEMM1, 32 of GEMM3) are taken when the wide
// ones would leave more than half the SMs without a CTA.
// The path is opt-in (TTG_FUSED=1): measured on GB300 (CUDA-graph replays,
// r = 64, n = 2, ra = 5, block of 5) one fused launch takes 18.7 us against
// 17.5 us for the four launches of the general path.  Its phases run on one
// CTA of four warps per block of c2, so each is latency-bound: the X split
// (64 loads and conversions per thread) ~7.6k cycles, the core contraction
// ~11k cycles (about 1.8k instructions per thread at ~6 cycles each), GEMM3
// with its streamed Phi1 tiles ~6.7k, the FP64 stores ~6k; the general path
// spreads the X split and the core over many CTAs instead.
static bool fused_enabled() {
  static const bool enabled = [] {
    const char* v = std::getenv("TTG_FUSED");
    return v && v[0] == '1';
  }();
  return enabled;
}
static bool fused_plan(const LocalDims& L, int nvec, int& bn1, int& n3p, int& C, int& ntiles) {
  if (!fused_enabled()) return false;
  if (L.n != L.m || 128 % L.m != 0 || L.rx1 * L.m > 128 || L.rx2 > 64 || L.ry1 > 128) return false;
  if (L.m * L.ra2 > 16 || L.n * L.ra1 > 16) return false;
  const int k3tiles = ceil_div(L.rx1 * L.ra1, tc::TK);
  bool feasible[2] = {false, false};
  int cc[2] = {0, 0};
  i64 ctas[2] = {0, 0};
  for (int cand = 0; cand < 2; ++cand) {
    const int b = cand == 0 ? 128 : 64, n3 = cand == 0 ? 64 : 32;
    cc[cand] = (int)std::min<i64>(b / L.ra2, n3 / L.n);
    feasible[cand] = cc[cand] >= 1 &&
                     tc::fused_smem(b, n3, k3tiles) <= (size_t)tc::FUSED_MAX_SMEM;
    if (feasible[cand]) ctas[cand] = (i64)nvec * ceil_div(L.ry2, cc[cand]);
  }
  int pick = -1;
  if (feasible[0] && (2 * ctas[0] >= 152 || !feasible[1])) pick = 0;
  else if (feasible[1]) pick = 1;
  if (pick < 0) return false;
  bn1 = pick == 0 ? 128 : 64;
  n3p = pick == 0 ? 64 : 32;
  C = cc[pick];
  ntiles = ceil_div(L.ry2, C);
  return true;
}

// The core-contracted path for small mode sizes (n*m <= 4: spin chains),
// where contracting A into Phi2 costs the first product only n*ra1/ra2 times
// its FLOPs but saves the FP32 intermediate T1 (written and read back once per
// apply) and the CUDA-core CORE launch; rx1 a multiple of 8 for the 16-byte
// epilogue stores.  TTG_SPLIT_PRE=0 keeps the four-launch path.
static bool pre_plan(const LocalDims& L) {
  static const bool enabled = [] {
    const char* v = std::getenv("TTG_SPLIT_PRE");
    return !(v && v[0] == '0');
  }();
  return enabled && tc::use_ws() && L.rx1 % 8 == 0 && L.n * L.m <= 4;
}

// Sizing (op == nullptr) takes the widest tile padding so that the bytes
// bound every tile width the autotuner may pick at layout time, and the
// larger of the two forms' layouts: callers size one buffer from the largest
// ranks a sweep may reach, and a smaller local problem may take the other
// form (the core-contracted one needs rx1 % 8 == 0).
static size_t split_layout(const LocalDims& L, int nvec_max, SplitOp* op, char* base,
                           cudaStream_t s = nullptr);
static size_t split_layout_pre(const LocalDims& L, int nvec_max, SplitOp* op, char* base,
                               cudaStream_t s);

static size_t split_layout(const LocalDims& L, int nvec_max, SplitOp* op, char* base,
                           cudaStream_t s) {
  const bool sizing0 = !(op && base);
  {
    int b_, n_, c_, t_;
    if (!sizing0 && !fused_plan(L, nvec_max, b_, n_, c_, t_) && pre_plan(L))
      return split_layout_pre(L, nvec_max, op, base, s);
  }
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
  // K-chunk partials of the tiled CORE kernel: for this problem the largest
  // over 1..nvec_max vectors; when sizing, the largest over every row count
  // up to this problem's (fewer rows split K into more chunks, so a smaller
  // local problem can need more partials than the largest; K is split only
  // below 152 row tiles, which bounds the scan)
  const int ja = (int)(L.m * L.ra2), na = (int)(L.n * L.ra1);
  size_t part = 0;
  if (!(ja <= 16 && na <= 16)) {
    auto need = [&](i64 rows) {
      int nz, qc;
      tc::core_chunks(rows, na, ja, nz, qc);
      return nz > 1 ? (size_t)(nz * rows * na) * sizeof(float) : (size_t)0;
    };
    if (sizing) {
      const i64 rmax = std::min<i64>(L.rx1 * L.ry2 * nvec_max, (i64)152 * tc::CT_R);
      for (i64 r = 1; r <= rmax; ++r) part = std::max(part, need(r));
    } else {
      for (int v = 1; v <= nvec_max; ++v) part = std::max(part, need(L.rx1 * L.ry2 * v));
    }
  }
  part = (part + 1023) & ~size_t(1023);
  tot += part;
  // permuted Phi2 tiles of the fused path (the larger of its two tile plans;
  // when sizing, whenever the path is enabled: a smaller local problem may
  // take it where the largest does not)
  size_t p2f = 0;
  {
    int b, n3, c, nt;
    if (sizing ? fused_enabled() : fused_plan(L, nvec_max, b, n3, c, nt)) {
      for (int bb : {128, 64}) {
        const int cb = (int)std::min<i64>(bb / L.ra2, (bb == 128 ? 64 : 32) / L.n);
        if (cb < 1) continue;
        const size_t e = (size_t)ceil_div(L.ry2, cb) * bb * tc::TK;
        p2f = std::max(p2f, 2 * ((e * sizeof(tc::bf16) + 1023) & ~size_t(1023)));
      }
    }
  }
  tot += p2f;
  if (op && base) {
    char* p = base;
    op->L = L;
    op->nvec_max = nvec_max;
    op->bn1 = bn1; op->bn3 = bn3;
    op->pre = false;
    op->X = tc::make_tiled(M1, K1, tc::TM, p);
    op->P2 = tc::make_tiled(N1, K1, bn1, p);
    op->P1 = tc::make_tiled(M3, K3, tc::TM, p);
    op->T2 = tc::make_tiled(N3, K3, bn3, p);
    op->T1 = (float*)p; p += t1;
    op->ld1 = ld1;
    op->err = (int*)p; p += 1024;
    op->part = part ? (float*)p : nullptr; p += part;
    op->fused = p2f > 0 && fused_plan(L, nvec_max, op->fbn1, op->fn3p, op->fC, op->fntiles);
    if (op->fused) {
      const size_t e = (size_t)op->fntiles * op->fbn1 * tc::TK;
      const size_t b = (e * sizeof(tc::bf16) + 1023) & ~size_t(1023);
      op->p2f_hi = (tc::bf16*)p;
      op->p2f_lo = (tc::bf16*)(p + b);
    }
    p += p2f;
  }
  // sizing bounds both forms
  return sizing ? std::max(tot, split_layout_pre(L, nvec_max, nullptr, nullptr, s)) : tot;
}

// layout of the core-contracted form (see pre_plan)
static size_t split_layout_pre(const LocalDims& L, int nvec_max, SplitOp* op, char* base,
                               cudaStream_t s) {
  const int MQ = (int)(L.n * L.ry2 * L.ra1), KQ = (int)(L.m * L.rx2);
  const int NX = (int)(L.rx1 * nvec_max);
  const int M3 = (int)L.ry1, N3 = (int)(L.n * L.ry2 * nvec_max), K3 = (int)(L.rx1 * L.ra1);
  const bool sizing = !(op && base);
  const int bnq = sizing ? 256 : tc::tuned_bn(MQ, NX, KQ, false, s);
  const int bn3 = sizing ? 256 : tc::tuned_bn(M3, N3, K3, true, s);
  size_t tot = tc::tiled_bytes(MQ, KQ, tc::TM) + tc::tiled_bytes(NX, KQ, bnq) +
               tc::tiled_bytes(M3, K3, tc::TM) + tc::tiled_bytes(N3, K3, bn3) + 1024 +
               sizeof(SplitOp) + 1024;
  if (op && base) {
    char* p = base;
    op->L = L;
    op->nvec_max = nvec_max;
    op->bn1 = bnq; op->bn3 = bn3;
    op->pre = true;
    op->fused = false;
    op->Q = tc::make_tiled(MQ, KQ, tc::TM, p);
    op->X = tc::make_tiled(NX, KQ, bnq, p);
    op->P1 = tc::make_tiled(M3, K3, tc::TM, p);
    op->T2 = tc::make_tiled(N3, K3, bn3, p);
    op->T1 = nullptr;
    op->ld1 = 0;
    op->err = (int*)p; p += 1024;
    op->part = nullptr;
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
                      const double* A, const double* phi2, void* mem, size_t mem_bytes,
                      cudaStream_t s) {
  // the layout of this local problem's form must fit the caller's buffer
  // (sized with split_op_bytes for the largest problem it serves); checked
  // before anything is written to it
  const size_t need = split_layout(L, nvec_max, op, (char*)mem, s);
  TTG_REQUIRE(need <= mem_bytes, "split matvec: workspace too small for this local problem");
  op->A = A;
  if (op->pre) {
    const i64 total = (i64)op->Q.rtiles * tc::TM * op->Q.ktiles * (tc::TK / 8);
    tc::build_q_kernel<<<(int)std::min<i64>(8192, (total + 255) / 256), 256, 0, s>>>(
        A, phi2, (int)L.m, (int)L.rx2, (int)L.n, (int)L.ry2, (int)L.ra1, (int)L.ra2,
        op->Q.rtiles, op->Q.ktiles, op->Q.hi, op->Q.lo);
    TTG_CHECK_LAUNCH();
    tc::split_into(phi1, 1ll << 40, 0, 1, L.ry1, op->P1, s);
    TTG_CUDA(cudaMemsetAsync(op->err, 0, sizeof(int), s));
    // K columns of T2 beyond rx1*ra1 must be zero (they meet Phi1's zero padding)
    TTG_CUDA(cudaMemsetAsync(op->T2.hi, 0, op->T2.elems() * sizeof(tc::bf16), s));
    TTG_CUDA(cudaMemsetAsync(op->T2.lo, 0, op->T2.elems() * sizeof(tc::bf16), s));
    return;
  }
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
  // Phi1 element (c1, k=(b1,a1)) at phi1[c1 + ry1*k]
  tc::split_into(phi1, 1ll << 40, 0, 1, L.ry1, op->P1, s);
  TTG_CUDA(cudaMemsetAsync(op->err, 0, sizeof(int), s));
  if (op->fused) {
    // fused path: Phi2 rows (a2, c2) grouped per block of C values of c2
    TTG_REQUIRE(op->coef_kind > 0, "fused split matvec: core too large");
    const i64 total = (i64)op->fntiles * op->fbn1 * (tc::TK / 8);
    const int blocks = (int)std::min<i64>(4096, (total + 255) / 256);
    tc::split_p2_fused_kernel<<<blocks, 256, 0, s>>>(phi2, (int)L.rx2, (int)L.ra2, (int)L.ry2,
                                                      op->fC, op->fbn1, op->fntiles, op->p2f_hi,
                                                      op->p2f_lo);
    TTG_CHECK_LAUNCH();
    return;
  }
  // Phi2 element (n=(a2,c2), k=b2) at phi2[b2 + rx2*n]
  tc::split_into(phi2, 1ll << 40, 0, L.rx2, 1, op->P2, s);
  // T2 padding (K columns the CORE kernel never writes) must be zero: padded
  // K columns meet zero columns of Phi1, and 0 * garbage could be NaN
  TTG_CUDA(cudaMemsetAsync(op->T2.hi, 0, op->T2.elems() * sizeof(tc::bf16), s));
  TTG_CUDA(cudaMemsetAsync(op->T2.lo, 0, op->T2.elems() * sizeof(tc::bf16), s));
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
    launch_pdl(wide ? tc::core_small_kernel<JA, NA, 8> : tc::core_small_kernel<JA, NA, 1>,       \
               dim3(blocks), dim3(128), 0, s, (const float*)op->T1, op->ld1, cc, (int)L.rx1,    \
               (int)L.m, (int)L.ra2, (int)L.n, (int)L.ra1, (int)L.ry2, nvec, lgR3, T2.ktiles,   \
               T2.hi, T2.lo);                                                                   \
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
    launch_pdl(tc::core_tiled_kernel, grid, dim3(256), 0, s, (const float*)op->T1, op->ld1, op->A,
               (int)L.rx1, (int)L.m, (int)L.ra2, (int)L.n, (int)L.ra1, (int)L.ry2, nvec, lgR3,
               T2.ktiles, T2.hi, T2.lo, qchunk, part);
    if (part) {
      const i64 tot = rows * na;
      launch_pdl(tc::core_finish_kernel, dim3((unsigned)std::min<i64>(4096, ceil_div(tot, (i64)256))),
                 dim3(256), 0, s, (const float*)part, nz, rows, na, (int)L.rx1, (int)L.n,
                 (int)L.ra1, lgR3, T2.ktiles, T2.hi, T2.lo);
    }
  }
}

template <int BN1, int N3P, int JA, int NA>
static void fused_launch(const tc::FusedArgs& a, int ntiles, int nvec, cudaStream_t s) {
  auto kern = tc::fused_small_kernel<BN1, N3P, JA, NA>;
  const size_t smem = tc::fused_smem(BN1, N3P, a.k3tiles);
  static const cudaError_t attr_rc = cudaFuncSetAttribute(
      kern, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::FUSED_MAX_SMEM);
  TTG_CUDA(attr_rc);
  TTG_REQUIRE(smem <= (size_t)tc::FUSED_MAX_SMEM, "fused split matvec: shared memory plan");
  kern<<<dim3(ntiles, nvec), tc::NTHREADS, smem, s>>>(a);
  TTG_CHECK_LAUNCH();
}

static void fused_apply(SplitOp* op, const double* x, double* y, int nvec, cudaStream_t s) {
  const LocalDims& L = op->L;
  TTG_REQUIRE(nvec < 65536, "fused split matvec: too many vectors");
  tc::FusedArgs a;
  a.x = x; a.y = y;
  a.p2hi = op->p2f_hi; a.p2lo = op->p2f_lo;
  a.p1hi = op->P1.hi; a.p1lo = op->P1.lo;
  a.rx1 = (int)L.rx1; a.m = (int)L.m; a.rx2 = (int)L.rx2; a.ry1 = (int)L.ry1;
  a.n = (int)L.n; a.ry2 = (int)L.ry2; a.ra1 = (int)L.ra1; a.ra2 = (int)L.ra2;
  a.C = op->fC;
  a.k3tiles = op->P1.ktiles;
  a.xs = L.xsize(); a.ys = L.ysize();
  a.err = op->err;
  const int na = (int)(L.n * L.ra1), ja = (int)(L.m * L.ra2);
  // coefficients at a[q * NA + p] for the kernel's bound NA
  auto fill = [&](int NA) {
    for (int e = 0; e < 256; ++e) a.a[e] = 0.f;
    for (int q = 0; q < ja; ++q)
      for (int p = 0; p < na; ++p) a.a[q * NA + p] = op->coef[(size_t)q * na + p];
  };
#define TTG_FUSED(JA_, NA_)                                                       \
  do {                                                                            \
    fill(NA_);                                                                    \
    if (op->fbn1 == 128) fused_launch<128, 64, JA_, NA_>(a, op->fntiles, nvec, s); \
    else fused_launch<64, 32, JA_, NA_>(a, op->fntiles, nvec, s);                 \
  } while (0)
  switch (op->coef_kind) {
    case 1: TTG_FUSED(4, 4); break;
    case 2: TTG_FUSED(8, 8); break;
    case 3: TTG_FUSED(10, 10); break;
    default: TTG_FUSED(16, 16); break;
  }
#undef TTG_FUSED
}

void split_op_apply(SplitOp* op, const double* x, double* y, int nvec, cudaStream_t s) {
  const LocalDims& L = op->L;
  TTG_REQUIRE(nvec >= 1 && nvec <= op->nvec_max, "split matvec: nvec out of range");
  if (op->fused) {
    fused_apply(op, x, y, nvec, s);
    return;
  }
  if (op->pre) {
    // X_v element (row (b1,v), k=(j,b2)) at x[v*xsize + b1 + rx1*k]
    const int NX = (int)(L.rx1 * nvec), MQ = (int)(L.n * L.ry2 * L.ra1);
    tc::Tiled X = op->X;
    X.rows = NX;
    X.rtiles = ceil_div(NX, X.R);
    tc::split_into(x, L.rx1, L.xsize(), 1, L.rx1, X, s);
    tc::Tiled T2b = op->T2;
    const int N3 = (int)(L.n * L.ry2 * nvec);
    T2b.rtiles = ceil_div(N3, T2b.R);
    tc::EpiT2 ep;
    ep.rx1 = (int)L.rx1;
    ep.nry2 = (int)(L.n * L.ry2);
    ep.lgR3 = T2b.R == 256 ? 8 : (T2b.R == 128 ? 7 : 6);
    ep.ktiles3 = T2b.ktiles;
    ep.hi = T2b.hi;
    ep.lo = T2b.lo;
    tc::gemm_launch_t2(op->Q, X, MQ, NX, ep, op->err, s);
    tc::gemm_launch<double>(op->P1, T2b, (int)L.ry1, N3, y, 1ll << 40, 0, 1, L.ry1, op->err, s);
    return;
  }
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
                          const double* phi2, int nvec_max, void* mem, size_t mem_bytes,
                          cudaStream_t s, MatvecFn* out, int slot) {
  TTG_REQUIRE(slot >= 0 && slot < kSplitSlots, "split matvec: bad operator slot");
  TTG_REQUIRE(split_op_supported(L), "split matvec: local problem too large");
  op_store_set[slot] = true;
  split_op_prepare(&op_store[slot], L, nvec_max, phi1, A, phi2, mem, mem_bytes, s);
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
    split_op_prepare(&op, L, (int)nvec, phi1, A, phi2, mem, bytes, c->stream);
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
      split_op_prepare(&op->split, L, (int)nvec_max, phi1, A, phi2, op->mem, bytes, c->stream);
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
