// Shared definitions of the tt-fort GB300 sweep library (libttgpu).
//
// Layout conventions follow the reference Fortran (column-major, flat arrays):
//   x    (rx1, m, rx2)        b1, j, b2
//   y    (ry1, n, ry2)        c1, i, c2
//   A    (ra1, n, m, ra2)     a1, i, j, a2
//   phi1 (ry1, rx1, ra1)      c1, b1, a1
//   phi2 (rx2, ra2, ry2)      b2, a2, c2
// (ttals.f90:9-32 index comments).
#pragma once
#include <cuda_runtime.h>
#include <cooperative_groups.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include <complex>
#include <atomic>
#include <utility>

#include "../../include/ttgpu.h"

namespace ttg {

using i64 = long long;

// -------------------------------------------------------------------------
// errors
// -------------------------------------------------------------------------
struct Error {
  int code;
  std::string msg;
};

#define TTG_CUDA(call)                                                          \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      throw ::ttg::Error{TTG_ERR_CUDA, std::string(#call) + ": " +              \
                                           cudaGetErrorString(e_)};             \
    }                                                                           \
  } while (0)

// every kernel launch site is followed by TTG_CHECK_LAUNCH(); it also counts
// the launches (reported as gpu_launches by the benchmark)
extern std::atomic<long long> g_launches;
#define TTG_CHECK_LAUNCH()                                                      \
  do {                                                                          \
    ++::ttg::g_launches;                                                        \
    TTG_CUDA(cudaGetLastError());                                               \
  } while (0)

#define TTG_REQUIRE(cond, msg)                                                  \
  do {                                                                          \
    if (!(cond)) throw ::ttg::Error{TTG_ERR_ARG, std::string(msg)};             \
  } while (0)

// -------------------------------------------------------------------------
// Deterministic reductions across CTAs.  Partial sums of several CTAs are
// combined inside one thread block cluster through distributed shared memory
// in a fixed order (lanes, then warps, then cluster ranks), never by atomics,
// so a result does not depend on which CTA finishes first.  Clusters hold at
// most kMaxCluster CTAs (the portable limit), which bounds every split.
// -------------------------------------------------------------------------
constexpr int kMaxCluster = 8;

// Sum of v over every thread of every CTA in the cluster.  All threads of all
// CTAs of the cluster must call it (it holds two cluster barriers); the sum is
// returned in thread 0 of cluster rank 0, every other thread gets 0.  A kernel
// launched without a cluster is a cluster of one CTA.
__device__ __forceinline__ double cluster_sum(double v) {
  namespace cg = cooperative_groups;
  __shared__ double red[33];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) t += red[w];
    red[32] = t;
  }
  cg::cluster_group cl = cg::this_cluster();
  cl.sync();
  double out = 0.0;
  if (cl.block_rank() == 0 && threadIdx.x == 0)
    for (unsigned r = 0; r < cl.num_blocks(); ++r) out += *cl.map_shared_rank(&red[32], r);
  cl.sync();
  return out;
}

// -------------------------------------------------------------------------
// Programmatic dependent launch.  A kernel launched with launch_pdl may start
// while the kernel before it in the stream is still running: its CTAs run
// their prologue (index set-up, barrier initialisation, tensor memory
// allocation), then every thread calls pdl_wait(), which returns once the
// preceding grid has completed and its memory is visible.  Every kernel
// launched this way calls pdl_wait() before its first global load or store,
// in every thread, so the completion order of the stream is kept transitively
// (a kernel completes only after the one before it).  pdl_trigger() lets the
// next kernel's CTAs be scheduled before this one finishes.  Kernels launched
// without the attribute (or when TTG_PDL=0) see both as no-ops.
// -------------------------------------------------------------------------
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
bool pdl_enabled();

// launch kernel k on grid/block with a cluster of cx x cy x cz CTAs (cluster.x
// == 0: no cluster attribute), optionally as a programmatic dependent launch
template <class... KArgs, class... Args>
void launch_ex(void (*k)(KArgs...), dim3 grid, dim3 block, dim3 cluster, bool pdl, size_t smem,
               cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[2];
  int na = 0;
  if (cluster.x > 0) {
    at[na].id = cudaLaunchAttributeClusterDimension;
    at[na].val.clusterDim.x = cluster.x;
    at[na].val.clusterDim.y = cluster.y;
    at[na].val.clusterDim.z = cluster.z;
    ++na;
  }
  if (pdl && pdl_enabled()) {
    at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[na].val.programmaticStreamSerializationAllowed = 1;
    ++na;
  }
  cfg.attrs = at;
  cfg.numAttrs = na;
  TTG_CUDA(cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...));
  TTG_CHECK_LAUNCH();
}

template <class... KArgs, class... Args>
void launch_clustered(void (*k)(KArgs...), dim3 grid, dim3 block, dim3 cluster, size_t smem,
                      cudaStream_t s, Args&&... args) {
  launch_ex(k, grid, block, cluster, false, smem, s, std::forward<Args>(args)...);
}

template <class... KArgs, class... Args>
void launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                Args&&... args) {
  launch_ex(k, grid, block, dim3(0, 1, 1), true, smem, s, std::forward<Args>(args)...);
}

// -------------------------------------------------------------------------
// device workspace: a bump allocator over one growing cudaMalloc block.
// Allocation happens only at sizing points (never inside a timed inner loop).
// -------------------------------------------------------------------------
struct Workspace {
  char* base = nullptr;
  size_t cap = 0;
  size_t top = 0;
  void reserve(size_t bytes);   // may reallocate: only when nothing is live
  void* take(size_t bytes);     // 256-byte aligned
  template <class T> T* takeT(size_t count) { return (T*)take(count * sizeof(T)); }
  void reset() { top = 0; }
  void release();
};

}  // namespace ttg

struct ttg_mlp;   // learned preconditioner network (ttg_learned.cu)

namespace ttg {
// one local problem recorded for training the learned preconditioner: the
// start Ritz block X (N x B) with values theta and residuals R, the diagonal
// D of the local operator, and V = the converged block rotated onto X,
// minus X, projected off span(X)
struct LearnedRecord {
  i64 N = 0;
  int B = 0;
  std::vector<double> D, theta, X, R, V;
};
}  // namespace ttg

// The opaque context handed across the C-ABI.  One context per host thread;
// it replaces the reference's module-level globals (tt_eigb.f90:1-50,
// tt_ksl.f90:1-166) and module result arrays (result_core, zresult_core).
struct ttg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  ttg::Workspace ws;          // scratch for kernel-level calls
  std::string last_error;
  int verb = 0;
  // driver results (host copies), freed by ttg_free_result
  std::vector<double> result_core;
  std::vector<std::complex<double>> zresult_core;
  std::vector<long long> result_ry;
  // counters of the last driver call
  long long stat_matvecs = 0;
  long long stat_sweeps = 0;
  long long stat_launches = 0;
  double stat_res = 0.0;
  long long stat_capped = 0;  // local solves of the last driver call that hit a cap
  // iteration caps (0 = the reference's values) and whether reaching one is
  // an error (TTG_ERR_NOCONV) instead of being tolerated as the reference does
  int lim_matvecs = 0;        // local eigensolver matvec budget (maxMatvecs, 500)
  int lim_expsteps = 0;       // Expokit integration steps per exponential (mxstep, 500)
  int strict = 0;
  // learned preconditioner: mode bit 0 = precondition the plain Davidson
  // expansions, bit 1 = record training problems from the sweeps
  ttg_mlp* learned = nullptr;
  int learned_mode = 0;
  std::vector<ttg::LearnedRecord> records;
};

namespace ttg {

static inline int ceil_div(i64 a, i64 b) { return (int)((a + b - 1) / b); }

// ---------------------------------------------------------------------------
// FP64 generic strided batched GEMM (ttg_gemm_f64.cu)
//   C[m,n] = alpha * sum_k A[m*sAm + k*sAk] * B[k*sBk + n*sBn] + beta * C[...]
//   batch index b = b1 + nb1*b2, operand offset = b1*s?1 + b2*s?2
// ---------------------------------------------------------------------------
struct GemmF64 {
  int M = 0, N = 0, K = 0;
  const double* A = nullptr; i64 sAm = 0, sAk = 0;
  const double* B = nullptr; i64 sBk = 0, sBn = 0;
  double* C = nullptr;       i64 sCm = 0, sCn = 0;
  double alpha = 1.0, beta = 0.0;
  int nb1 = 1, nb2 = 1;
  i64 bA1 = 0, bA2 = 0, bB1 = 0, bB2 = 0, bC1 = 0, bC2 = 0;
  int splitk = 1;   // > 1: K split over the CTAs of one cluster (at most kMaxCluster),
                    // partial tiles added in a fixed order (deterministic)
};
void gemm_f64(const GemmF64& g, cudaStream_t s);

// standard normals from the splitmix64/Box-Muller stream shared with the oracle
void sm_normals(unsigned long long seed, i64 count, double* out);

// FP32 variant (learned preconditioner network)
struct GemmF32 {
  int M = 0, N = 0, K = 0;
  const float* A = nullptr; i64 sAm = 0, sAk = 0;
  const float* B = nullptr; i64 sBk = 0, sBn = 0;
  float* C = nullptr;       i64 sCm = 0, sCn = 0;
  float alpha = 1.f, beta = 0.f;
  int nb1 = 1, nb2 = 1;
  i64 bA1 = 0, bA2 = 0, bB1 = 0, bB2 = 0, bC1 = 0, bC2 = 0;
  int splitk = 1;
};
void gemm_f32(const GemmF32& g, cudaStream_t s);

// complex128 variant (KSL path); same strides in units of complex elements.
struct GemmZ {
  int M = 0, N = 0, K = 0;
  const double2* A = nullptr; i64 sAm = 0, sAk = 0; bool conjA = false;
  const double2* B = nullptr; i64 sBk = 0, sBn = 0; bool conjB = false;
  double2* C = nullptr;       i64 sCm = 0, sCn = 0;
  double2 alpha = {1.0, 0.0}, beta = {0.0, 0.0};
  int nb1 = 1, nb2 = 1;
  i64 bA1 = 0, bA2 = 0, bB1 = 0, bB2 = 0, bC1 = 0, bC2 = 0;
  int splitk = 1;
};
void gemm_z(const GemmZ& g, cudaStream_t s);

// ---------------------------------------------------------------------------
// Local operator kernels (ttg_local.cu)
// ---------------------------------------------------------------------------
struct LocalDims {
  i64 rx1, m, rx2, ry1, n, ry2, ra1, ra2;
  i64 xsize() const { return rx1 * m * rx2; }
  i64 ysize() const { return ry1 * n * ry2; }
  i64 t1size() const { return rx1 * m * ra2 * ry2; }
  i64 t2size() const { return rx1 * ra1 * n * ry2; }
};

// bfun3 for nvec vectors (x: xsize*nvec contiguous, y: ysize*nvec).
// scratch: (t1size + t2size) * nvec doubles.
void bfun3_f64(const LocalDims& L, const double* phi1, const double* A, const double* phi2,
               const double* x, double* y, int nvec, double* scratch, cudaStream_t s);
size_t bfun3_f64_scratch(const LocalDims& L, int nvec);

void phi_left_f64(const LocalDims& L, const double* phi1_old, const double* A,
                  const double* x, const double* y, double* phi1_new, double* scratch,
                  cudaStream_t s);
void phi_right_f64(const LocalDims& L, const double* phi2_old, const double* A,
                   const double* x, const double* y, double* phi2_new, double* scratch,
                   cudaStream_t s);
size_t phi_f64_scratch(const LocalDims& L);

void phi2_left_f64(i64 rx1, i64 rx2, i64 ry1, i64 n, i64 ry2, const double* phi1_old,
                   const double* x, const double* y, double* phi1_new, double* scratch,
                   cudaStream_t s);
void phi2_right_f64(i64 rx1, i64 rx2, i64 ry1, i64 n, i64 ry2, const double* phi2_old,
                    const double* x, const double* y, double* phi2_new, double* scratch,
                    cudaStream_t s);

// Dense local matrix B[(c1,i,c2),(b1,j,b2)] (d2d_fullmat, tt_eigb.f90:88-105).
void fullmat_f64(i64 rx1, i64 m, i64 rx2, i64 ra1, i64 ra2, const double* phi1,
                 const double* A, const double* phi2, double* Bmat, cudaStream_t s);

// complex versions (tt_ksl.f90 K- and S-steps)
void bfun3_z(const LocalDims& L, const double2* phi1, const double2* A, const double2* phi2,
             const double2* x, double2* y, int nvec, double2* scratch, cudaStream_t s);
void bfun3_transp_z(const LocalDims& L, const double2* phi1, const double2* A,
                    const double2* phi2, const double2* x, double2* y, int nvec,
                    double2* scratch, cudaStream_t s);
void phi_left_z(const LocalDims& L, const double2* phi1_old, const double2* A,
                const double2* x, const double2* y, double2* phi1_new, double2* scratch,
                cudaStream_t s);
void phi_right_z(const LocalDims& L, const double2* phi2_old, const double2* A,
                 const double2* x, const double2* y, double2* phi2_new, double2* scratch,
                 cudaStream_t s);

// Block-Jacobi preconditioners of the local system (ttg_jac.cu; djac_gen /
// djac_apply): jac_type normalises 'c'/'l'/'r' (0 if none), sizes in doubles.
char jac_type(char p);
i64 jac_size(char p, i64 rx1, i64 n, i64 rx2);
i64 jac_gen_scratch(char p, i64 rx1, i64 n, i64 rx2, i64 ra1, i64 ra2);
void jac_gen_f64(char p, i64 rx1, i64 n, i64 rx2, i64 ra1, i64 ra2, const double* phi1,
                 const double* A, const double* phi2, double* jacs, double* scr, cudaStream_t s);
void jac_apply_f64(char p, i64 rx1, i64 n, i64 rx2, const double* jacs, const double* x,
                   double* y, int nvec, cudaStream_t s);

// ---------------------------------------------------------------------------
// Split-precision (BF16x3, FP32 accumulate) tensor-core local operator
// (ttg_tc.cu).  Operands are prepared once per local problem.
// ---------------------------------------------------------------------------
struct SplitOp;   // opaque prepared operator
size_t split_op_bytes(const LocalDims& L, int nvec_max);
void split_op_prepare(SplitOp* op, const LocalDims& L, int nvec_max, const double* phi1,
                      const double* A, const double* phi2, void* mem, size_t mem_bytes,
                      cudaStream_t s);
void split_op_apply(SplitOp* op, const double* x, double* y, int nvec, cudaStream_t s);
bool split_op_supported(const LocalDims& L);

// Plain BF16 tensor-core GEMM on FP32 operands, FP32 accumulate (ttg_tc.cu):
// C[m*scm + n*scn] = sum_k a[m*sam + k*sak] b[n*sbn + k*sbk]; ws holds
// bf16_gemm_ws(M, N, K) bytes; err is the bounded-wait flag (device int).
size_t bf16_gemm_ws(int M, int N, int K);
void bf16_gemm(int M, int N, int K, const float* a, i64 sam, i64 sak, const float* b, i64 sbn,
               i64 sbk, float* c, i64 scm, i64 scn, void* ws, int* err, cudaStream_t s);

// ---------------------------------------------------------------------------
// Dense FP64 linear algebra (ttg_linalg.cu)
// ---------------------------------------------------------------------------
// Symmetric eigen (cyclic Jacobi, one CTA): A (k x k, lda) overwritten,
// eigenvalues ascending in w, eigenvectors in V (k x k, ldv).  status: iters
// P0 (kp x kp, ldp), optional: eigenvectors of the leading kp x kp block of A
// (warm start, used when A grew by appending rows and columns).
void syev_jacobi(int k, double* A, int lda, double* w, double* V, int ldv, int* status,
                 cudaStream_t s, const double* P0 = nullptr, int kp = 0, int ldp = 0);
// One-sided Jacobi SVD of M (p x q, p >= q, ldm = p), in place.  Outputs:
// sigma (q, descending), U (p x q), Vt (q x q, rows = right singular vectors).
size_t svd_scratch(int p, int q);
// lowest k eigenpairs (ascending) of a symmetric N x N matrix H (overwritten)
// by the Jacobi SVD of H + ||H||_F I; V (N x k), w (k)
size_t syev_lowest_scratch(int N);
void syev_lowest_svd(int N, int k, double* H, double* w, double* V, double* scratch, int* status,
                     cudaStream_t s);
void svd_jacobi(int p, int q, const double* M, double* U, double* sigma, double* Vt,
                double* scratch, int* status, cudaStream_t s);
// Householder QR with LAPACK's convention: A (n x m) -> Q (n x min), R (min x m).
void qr_householder(int n, int m, double* A, double* R, double* tau, cudaStream_t s);
void qr_householder_z(int n, int m, double2* A, double2* R, double2* tau, cudaStream_t s);

// small helpers
void transpose_f64(i64 rows, i64 cols, const double* in, double* out, cudaStream_t s);
void transpose_z(i64 rows, i64 cols, const double2* in, double2* out, cudaStream_t s);
void copy_rows_f64(i64 rows_in, i64 rows_out, i64 cols, const double* in, double* out,
                   cudaStream_t s);   // drow_cut: keep the first rows_out rows
void scale_cols_f64(i64 rows, i64 cols, double* A, i64 lda, const double* s, cudaStream_t st);
void scale_rows_f64(i64 rows, i64 cols, double* A, i64 lda, const double* s, cudaStream_t st);
void fill_f64(double* p, i64 n, double v, cudaStream_t s);

}  // namespace ttg
