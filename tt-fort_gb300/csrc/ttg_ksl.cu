// KSL (projector-splitting) time stepper ztt_ksl (tt_ksl.f90:431-668) on the
// GPU.  One call performs nsteps consecutive time steps, each exactly the
// reference's single call (QR sweep, backward half sweep with K- and S-steps,
// forward half sweep); the cores stay in HBM between steps.
//
//   K-step  exp(+tau0 A_loc) core_i   A_loc x = zbfun3 (Phi_L A_i Phi_R x)
//   S-step  exp(-tau0 S) R            S x = Phi1 (x Phi2)   (sfun_ksl,
//                                     tt_ksl.f90:142-152)
// with tau0 = tau/2 for the symmetric scheme (typ = 2), Krylov order 8 and
// tolerance 1e-8 (tt_ksl.f90:477), anorm from the block 1-norm estimate.
#include "ttg_expokit.cuh"
#include "ttg_davidson.cuh"
#include <algorithm>
#include <cmath>

namespace ttg {

namespace {

struct DevBlockZ {
  char* base = nullptr;
  size_t top = 0, cap = 0;
  ~DevBlockZ() { if (base) cudaFree(base); }
  void alloc(size_t bytes) {
    if (cudaMalloc(&base, bytes) != cudaSuccess) {
      base = nullptr;
      throw Error{TTG_ERR_NOMEM, "ztt_ksl: device allocation failed"};
    }
    cap = bytes;
  }
  template <class T> T* take(size_t count) {
    size_t b = (count * sizeof(T) + 255) & ~size_t(255);
    if (top + b > cap) throw Error{TTG_ERR_NOMEM, "ztt_ksl: device block exhausted"};
    T* p = (T*)(base + top);
    top += b;
    return p;
  }
};

inline size_t alz(size_t b) { return (b + 255) & ~size_t(255); }

// S operator (sfun_ksl): Sy (ry1 x ry2) = phi1 (ry1 x rx1*ra) [Sx (rx1 x rx2) phi2 (rx2 x ra*ry2)]
void sfun_apply(i64 rx1, i64 rx2, i64 ra, i64 ry1, i64 ry2, const double2* phi1,
                const double2* phi2, const double2* X, double2* Y, int t, double2* res,
                cudaStream_t s) {
  {
    GemmZ g;
    g.M = (int)rx1; g.N = (int)(ra * ry2); g.K = (int)rx2;
    g.A = X; g.sAm = 1; g.sAk = rx1;
    g.B = phi2; g.sBk = 1; g.sBn = rx2;
    g.C = res; g.sCm = 1; g.sCn = rx1;
    g.nb2 = t; g.bA2 = rx1 * rx2; g.bC2 = rx1 * ra * ry2;
    gemm_z(g, s);
  }
  {
    GemmZ g;
    g.M = (int)ry1; g.N = (int)ry2; g.K = (int)(rx1 * ra);
    g.A = phi1; g.sAm = 1; g.sAk = ry1;
    g.B = res; g.sBk = 1; g.sBn = rx1 * ra;
    g.C = Y; g.sCm = 1; g.sCn = ry1;
    g.nb2 = t; g.bB2 = rx1 * ra * ry2; g.bC2 = ry1 * ry2;
    gemm_z(g, s);
  }
}

}  // namespace

struct KslParams {
  int d;
  std::vector<i64> n, m, ra, ry;
  const double2* crA;
  const double2* crY0;
  double tau;
  int typ, order, nsteps, verb;
  int method = TTG_METHOD_PLAIN;
  // diag: the operator is diagonal in the physical index (cores A(a1, i, a2),
  // crA holds those); ztt_diag_ksl, tt_diag_ksl.f90:560-804
  bool diag = false;
  // real_scheme: the sweep of the real tt_ksl (tt_ksl.f90:191-428) instead
  // of ztt_ksl's; see run_real_sweep
  bool real_scheme = false;
};

// A(a1, i, j, a2) = delta_ij D(a1, i, a2): the diagonal TT-matrix core as a
// full one, so the interfaces are zphi_left/right of it (equal to the slice
// sums zphi_diag_left/right, tt_diag_ksl.f90:269-301)
__global__ void expand_diag_kernel(i64 ra1, i64 n, i64 ra2, const double2* __restrict__ D,
                                   double2* __restrict__ A) {
  const i64 tot = ra1 * n * n * ra2;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    i64 t = e;
    const i64 a1 = t % ra1; t /= ra1;
    const i64 i = t % n; t /= n;
    const i64 j = t % n; const i64 a2 = t / n;
    A[e] = i == j ? D[a1 + ra1 * (i + n * a2)] : make_double2(0.0, 0.0);
  }
}
// out[a + r1 b] = in[a + r1 (k + n b)]  (zextract_slice, tt_diag_ksl.f90:236-243)
__global__ void slice_get_kernel(i64 r1, i64 n, i64 r2, i64 k, const double2* __restrict__ in,
                                 double2* __restrict__ out) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < r1 * r2; e += (i64)gridDim.x * blockDim.x)
    out[e] = in[e % r1 + r1 * (k + n * (e / r1))];
}
// out[a + r1 (k + n b)] = in[a + r1 b]  (zset_slice, tt_diag_ksl.f90:246-253)
__global__ void slice_set_kernel(i64 r1, i64 n, i64 r2, i64 k, const double2* __restrict__ in,
                                 double2* __restrict__ out) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < r1 * r2; e += (i64)gridDim.x * blockDim.x)
    out[e % r1 + r1 * (k + n * (e / r1))] = in[e];
}

// Chosen form of the K-step product: the complex local operator
// y = Phi1 A Phi2 x (zbfun3) as ONE real BF16x3 tensor-core operator with
// doubled ranks.  A complex factor w acts on (re, im) parts as the real 2x2
// block [[wr, -wi], [wi, wr]]; the re/im part of each contracted index is
// carried by a rank index: x by b2 (rx2 -> 2 rx2), the Phi2 product by a2,
// the A product by a1, the Phi1 product (the result) by c1.  Real dims:
// (rx1, m, 2 rx2, 2 ry1, n, ry2, 2 ra1, 2 ra2).
__device__ __forceinline__ double cmul_block(double2 w, int o, int c) {
  return o == c ? w.x : (o == 0 ? -w.y : w.y);
}
// The adjoint product y = B^H x (zbfun3_transp) is the same kind of operator
// with the roles of x and y exchanged: Phi1'[c1,b1,a1] = conj Phi1[b1,c1,a1],
// A'[a1,i,j,a2] = conj A[a1,j,i,a2], Phi2'[b2,a2,c2] = conj Phi2[c2,a2,b2],
// so the realify kernels take the dims of the operator they build and, with
// adj set, read the original operand through that index map.
__device__ __forceinline__ double2 cadj(double2 w, bool adj) { return adj ? make_double2(w.x, -w.y) : w; }
// Phi2~[(b2 + rx2 c) + 2 rx2 ((a2 + ra2 o) + 2 ra2 c2)] = M(Phi2[b2, a2, c2])[o, c]
__global__ void realify_phi2_kernel(i64 rx2, i64 ra2, i64 ry2, const double2* __restrict__ P,
                                    double* __restrict__ out, bool adj) {
  const i64 tot = 4 * rx2 * ra2 * ry2;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    i64 t = e;
    const i64 bc = t % (2 * rx2); t /= 2 * rx2;
    const i64 ao = t % (2 * ra2); const i64 c2 = t / (2 * ra2);
    const i64 b2 = bc % rx2, c = bc / rx2, a2 = ao % ra2, o = ao / ra2;
    const i64 src = adj ? c2 + ry2 * (a2 + ra2 * b2) : b2 + rx2 * (a2 + ra2 * c2);
    out[e] = cmul_block(cadj(P[src], adj), (int)o, (int)c);
  }
}
// A~[(a1 + ra1 o) + 2 ra1 (i + n (j + m (a2 + ra2 c)))] = M(A[a1, i, j, a2])[o, c]
__global__ void realify_core_kernel(i64 ra1, i64 n, i64 m, i64 ra2, const double2* __restrict__ A,
                                    double* __restrict__ out, bool adj) {
  const i64 tot = 4 * ra1 * n * m * ra2;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    i64 t = e;
    const i64 ao = t % (2 * ra1); t /= 2 * ra1;
    const i64 i = t % n; t /= n;
    const i64 j = t % m; t /= m;
    const i64 ac = t;
    const i64 a1 = ao % ra1, o = ao / ra1, a2 = ac % ra2, c = ac / ra2;
    const i64 src = adj ? a1 + ra1 * (j + m * (i + n * a2)) : a1 + ra1 * (i + n * (j + m * a2));
    out[e] = cmul_block(cadj(A[src], adj), (int)o, (int)c);
  }
}
// Phi1~[(c1 + ry1 o) + 2 ry1 (b1 + rx1 (a1 + ra1 c))] = M(Phi1[c1, b1, a1])[o, c]
__global__ void realify_phi1_kernel(i64 ry1, i64 rx1, i64 ra1, const double2* __restrict__ P,
                                    double* __restrict__ out, bool adj) {
  const i64 tot = 4 * ry1 * rx1 * ra1;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
    i64 t = e;
    const i64 co = t % (2 * ry1); t /= 2 * ry1;
    const i64 b1 = t % rx1; const i64 ac = t / rx1;
    const i64 c1 = co % ry1, o = co / ry1, a1 = ac % ra1, c = ac / ra1;
    const i64 src = adj ? b1 + rx1 * (c1 + ry1 * a1) : c1 + ry1 * (b1 + rx1 * a1);
    out[e] = cmul_block(cadj(P[src], adj), (int)o, (int)c);
  }
}
// x~[b1 + rx1 (j + m (b2 + rx2 c))] = part c of x[b1, j, b2] (per vector)
__global__ void pack_x_kernel(i64 rx1m, i64 rx2, int nv, const double2* __restrict__ x,
                              double* __restrict__ xt) {
  const i64 N = rx1m * rx2;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < N * nv; e += (i64)gridDim.x * blockDim.x) {
    const i64 v = e / N, r = e % N;
    const double2 z = x[e];
    xt[2 * N * v + r] = z.x;
    xt[2 * N * v + N + r] = z.y;
  }
}
// y[c1, i, c2] = y~[c1 + 2 ry1 (i, c2)] + i y~[c1 + ry1 + 2 ry1 (i, c2)]
__global__ void unpack_y_kernel(i64 ry1, i64 rest, int nv, const double* __restrict__ yt,
                                double2* __restrict__ y) {
  const i64 N = ry1 * rest;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < N * nv; e += (i64)gridDim.x * blockDim.x) {
    const i64 v = e / N, r = e % N;
    const i64 c1 = r % ry1, q = r / ry1;
    const double* b = yt + 2 * N * v + 2 * ry1 * q;
    y[e] = make_double2(b[c1], b[c1 + ry1]);
  }
}
inline int ebz(i64 n) { return (int)std::max<i64>(1, std::min<i64>(4096, (n + 255) / 256)); }

static void run_ksl(ttg_ctx* ctx, KslParams P, std::vector<std::complex<double>>& out_cores,
                    std::vector<i64>& out_ry, ExpStats& est) {
  cudaStream_t s = ctx->stream;
  const int d = P.d;
  auto& n = P.n;
  auto& ry = P.ry;
  TTG_REQUIRE(d >= 1, "ztt_ksl: d must be >= 1");
  TTG_REQUIRE(ry[0] == 1 && ry[d] == 1 && P.ra[0] == 1 && P.ra[d] == 1, "boundary ranks must be 1");
  for (int i = 0; i < d; ++i) TTG_REQUIRE(n[i] == P.m[i], "ztt_ksl needs square cores (n == m)");
  TTG_REQUIRE(P.order >= 2 && P.order + 2 <= 16, "Krylov order must be in [2, 14]");
  const double eps = 1e-8;
  std::vector<i64> pa(d + 1, 0);
  for (int i = 0; i < d; ++i) pa[i + 1] = pa[i] + P.ra[i] * n[i] * P.m[i] * P.ra[i + 1];
  // capacities: ranks never grow in ztt_ksl
  std::vector<i64> Rc(ry);
  i64 capmax = 1, Nmax = 1, phimax = 1, scr = 1, rmx = 1;
  for (int i = 0; i < d; ++i) {
    const i64 c = Rc[i] * n[i] * Rc[i + 1];
    capmax = std::max(capmax, c);
    Nmax = std::max(Nmax, c);
    LocalDims L{Rc[i], n[i], Rc[i + 1], Rc[i], n[i], Rc[i + 1], P.ra[i], P.ra[i + 1]};
    scr = std::max<i64>(scr, (i64)(phi_f64_scratch(L) / sizeof(double)) + 1);
    scr = std::max<i64>(scr, (L.t1size() + L.t2size()) * 4 + 16);
    scr = std::max<i64>(scr, (Rc[i] * P.ra[i] * n[i] * Rc[i + 1] + Rc[i] * n[i] * P.ra[i + 1] * Rc[i + 1]) * 4 + 16);
    rmx = std::max(rmx, Rc[i]);
  }
  for (int i = 0; i <= d; ++i) phimax = std::max(phimax, Rc[i] * Rc[i] * P.ra[i]);
  Nmax = std::max(Nmax, rmx * rmx);
  i64 ramax = *std::max_element(P.ra.begin(), P.ra.end());
  scr = std::max<i64>(scr, rmx * ramax * rmx * 4 + 16);
  size_t total = alz(sizeof(double2) * pa[d]);
  for (int i = 0; i < d; ++i) total += alz(sizeof(double2) * Rc[i] * n[i] * Rc[i + 1]);
  for (int i = 0; i <= d; ++i) total += alz(sizeof(double2) * std::max<i64>(1, Rc[i] * Rc[i] * P.ra[i]));
  total += 5 * alz(sizeof(double2) * capmax) + alz(sizeof(double2) * phimax) +
           2 * alz(sizeof(double2) * rmx * rmx) + alz(sizeof(double2) * rmx * 2) +
           alz(sizeof(double2) * scr) + alz(ExpWork::bytes(Nmax, P.order)) + (1 << 16);
  // chosen form: realified local operator (doubled ranks) on the tensor cores
  const bool split = P.method == TTG_METHOD_SPLIT;
  auto Lreal = [&](const LocalDims& L) {
    return LocalDims{L.rx1, L.m, 2 * L.rx2, 2 * L.ry1, L.n, L.ry2, 2 * L.ra1, 2 * L.ra2};
  };
  auto adjoint = [&](const LocalDims& L) {
    return LocalDims{L.ry1, L.n, L.ry2, L.rx1, L.m, L.rx2, L.ra1, L.ra2};
  };
  const int kNvecSplit = 4;   // block width of the norm estimate
  i64 amax = 1;
  size_t split_bytes = 0;
  if (split) {
    for (int i = 0; i < d; ++i) {
      const LocalDims L{Rc[i], n[i], Rc[i + 1], Rc[i], n[i], Rc[i + 1], P.ra[i], P.ra[i + 1]};
      for (const LocalDims& Lr : {Lreal(L), Lreal(adjoint(L))}) {
        TTG_REQUIRE(split_op_supported(Lr), "ztt_ksl: local problem too large for the split kernel");
        split_bytes = std::max(split_bytes, split_matvec_bytes(Lr, kNvecSplit));
      }
      amax = std::max(amax, P.ra[i] * n[i] * P.m[i] * P.ra[i + 1]);
    }
    // operator and adjoint: realified operands and prepared operators
    total += 2 * (2 * alz(sizeof(double) * 4 * phimax) + alz(sizeof(double) * 4 * amax) +
                  alz(split_bytes)) +
             2 * alz(sizeof(double) * 2 * capmax * kNvecSplit);
  }
  i64 pdiag = 0;
  if (P.diag) {
    for (int i = 0; i < d; ++i) pdiag += P.ra[i] * n[i] * P.ra[i + 1];
    total += alz(sizeof(double2) * pdiag) + 2 * alz(sizeof(double2) * rmx * rmx) +
             alz(sizeof(double2) * ramax * ramax);
  }
  DevBlockZ mem;
  mem.alloc(total);
  double2* dA = mem.take<double2>(pa[d]);
  std::vector<double2*> cr(d), phi(d + 1);
  for (int i = 0; i < d; ++i) cr[i] = mem.take<double2>(Rc[i] * n[i] * Rc[i + 1]);
  for (int i = 0; i <= d; ++i) phi[i] = mem.take<double2>(std::max<i64>(1, Rc[i] * Rc[i] * P.ra[i]));
  double2* curcr = mem.take<double2>(capmax);
  double2* t1 = mem.take<double2>(capmax);
  double2* t2 = mem.take<double2>(capmax);
  double2* t3 = mem.take<double2>(capmax);
  double2* Sout = mem.take<double2>(capmax);
  double2* phitmp = mem.take<double2>(phimax);
  double2* R = mem.take<double2>(rmx * rmx);
  double2* Rt = mem.take<double2>(rmx * rmx);
  double2* tau_ws = mem.take<double2>(rmx * 2);
  double2* scratch = mem.take<double2>(scr);
  void* expmem = mem.take<char>(ExpWork::bytes(Nmax, P.order));
  double *rphi1[2] = {}, *rphi2[2] = {}, *rA[2] = {}, *rx = nullptr, *ryv = nullptr;
  void* smem[2] = {};
  if (split) {
    for (int k = 0; k < 2; ++k) {
      rphi1[k] = mem.take<double>(4 * phimax);
      rphi2[k] = mem.take<double>(4 * phimax);
      rA[k] = mem.take<double>(4 * amax);
      smem[k] = mem.take<char>(split_bytes);
    }
    rx = mem.take<double>(2 * capmax * kNvecSplit);
    ryv = mem.take<double>(2 * capmax * kNvecSplit);
  }
  double2 *dD = nullptr, *slc = nullptr, *slc2 = nullptr, *Ak = nullptr;
  if (P.diag) {
    dD = mem.take<double2>(pdiag);
    slc = mem.take<double2>(rmx * rmx);
    slc2 = mem.take<double2>(rmx * rmx);
    Ak = mem.take<double2>(ramax * ramax);
  }
  double* pinned = nullptr;
  TTG_CUDA(cudaMallocHost(&pinned, 4096 * sizeof(double)));
  struct PinGuard { double* p; ~PinGuard() { if (p) cudaFreeHost(p); } } pg{pinned};
  ExpWork w;
  w.bind(expmem, Nmax, P.order, pinned);

  if (P.diag) {
    TTG_CUDA(cudaMemcpyAsync(dD, P.crA, sizeof(double2) * pdiag, cudaMemcpyHostToDevice, s));
    i64 od = 0;
    for (int i = 0; i < d; ++i) {
      expand_diag_kernel<<<ebz(P.ra[i] * n[i] * n[i] * P.ra[i + 1]), 256, 0, s>>>(
          P.ra[i], n[i], P.ra[i + 1], dD + od, dA + pa[i]);
      TTG_CHECK_LAUNCH();
      od += P.ra[i] * n[i] * P.ra[i + 1];
    }
  } else {
    TTG_CUDA(cudaMemcpyAsync(dA, P.crA, sizeof(double2) * pa[d], cudaMemcpyHostToDevice, s));
  }
  {
    i64 off = 0;
    for (int i = 0; i < d; ++i) {
      const i64 sz = ry[i] * n[i] * ry[i + 1];
      TTG_CUDA(cudaMemcpyAsync(cr[i], P.crY0 + off, sizeof(double2) * sz, cudaMemcpyHostToDevice, s));
      off += sz;
    }
  }
  const double2 one = make_double2(1.0, 0.0);
  TTG_CUDA(cudaMemcpyAsync(phi[0], &one, sizeof(double2), cudaMemcpyHostToDevice, s));
  TTG_CUDA(cudaMemcpyAsync(phi[d], &one, sizeof(double2), cudaMemcpyHostToDevice, s));
  auto A_of = [&](int i) { return dA + pa[i]; };
  auto Ld = [&](int i) {
    return LocalDims{ry[i], n[i], ry[i + 1], ry[i], n[i], ry[i + 1], P.ra[i], P.ra[i + 1]};
  };
  const double tau0 = P.typ == 2 || P.real_scheme ? P.tau / 2 : P.tau;

  for (int step = 0; step < P.nsteps; ++step) {
    // QR sweep, tt_ksl.f90:528-550
    for (int i = 0; i + 1 < d; ++i) {
      const i64 rows = ry[i] * n[i];
      const i64 rnew = std::min(rows, ry[i + 1]);
      qr_householder_z((int)rows, (int)ry[i + 1], cr[i], R, tau_ws, s);
      GemmZ g;
      g.M = (int)rnew; g.N = (int)(n[i + 1] * ry[i + 2]); g.K = (int)ry[i + 1];
      g.A = R; g.sAm = 1; g.sAk = rnew;
      g.B = cr[i + 1]; g.sBk = 1; g.sBn = ry[i + 1];
      g.C = t1; g.sCm = 1; g.sCn = rnew;
      gemm_z(g, s);
      TTG_CUDA(cudaMemcpyAsync(cr[i + 1], t1, sizeof(double2) * rnew * n[i + 1] * ry[i + 2],
                               cudaMemcpyDeviceToDevice, s));
      ry[i + 1] = rnew;
      phi_left_z(Ld(i), phi[i], A_of(i), cr[i], cr[i], phi[i + 1], scratch, s);
    }
    unsigned long long counter = 0;   // init_seed() at every call, tt_ksl.f90:556
    auto kstep_diag = [&](int i) {
      // one Krylov exponential per slice k, local operator bfun3 with
      // m = n = 1 and A(:, k, :), anorm = 1 (tt_diag_ksl.f90:688-697,727-733)
      const i64 r1 = ry[i], r2 = ry[i + 1], nk = n[i], N = r1 * r2;
      const LocalDims Lk{r1, 1, r2, r1, 1, r2, P.ra[i], P.ra[i + 1]};
      const double2 *p1 = phi[i], *p2 = phi[i + 1];
      i64 od = 0;
      for (int q = 0; q < i; ++q) od += P.ra[q] * n[q] * P.ra[q + 1];
      for (i64 k = 0; k < nk; ++k) {
        slice_get_kernel<<<ebz(P.ra[i] * P.ra[i + 1]), 256, 0, s>>>(P.ra[i], nk, P.ra[i + 1], k,
                                                                   dD + od, Ak);
        slice_get_kernel<<<ebz(N), 256, 0, s>>>(r1, nk, r2, k, cr[i], slc);
        TTG_CHECK_LAUNCH();
        const double2* Akc = Ak;
        ZMatvecFn mv = [=](const double2* X, double2* Y, int t) {
          bfun3_z(Lk, p1, Akc, p2, X, Y, t, scratch, s);
        };
        zexp_mv_dev(w, N, (int)std::min<i64>(P.order, N), tau0, slc, slc2, eps, 1.0, mv, s, &est);
        slice_set_kernel<<<ebz(N), 256, 0, s>>>(r1, nk, r2, k, slc2, curcr);
        TTG_CHECK_LAUNCH();
      }
    };
    auto kstep = [&](int i) {
      if (P.diag) return kstep_diag(i);
      const LocalDims L = Ld(i);
      const i64 N = L.xsize();
      const double2 *p1 = phi[i], *p2 = phi[i + 1], *Ai = A_of(i);
      ZMatvecFn mv = [=](const double2* X, double2* Y, int t) { bfun3_z(L, p1, Ai, p2, X, Y, t, scratch, s); };
      ZMatvecFn mvT = [=](const double2* X, double2* Y, int t) {
        bfun3_transp_z(L, p1, Ai, p2, X, Y, t, scratch, s);
      };
      if (split) {
        // slot 0: the operator, slot 1: its adjoint (the norm estimate's)
        auto build = [&](int k) -> ZMatvecFn {
          const LocalDims Lk = k ? adjoint(L) : L;
          const bool adj = k == 1;
          realify_phi1_kernel<<<ebz(4 * Lk.ry1 * Lk.rx1 * Lk.ra1), 256, 0, s>>>(Lk.ry1, Lk.rx1, Lk.ra1, p1, rphi1[k], adj);
          realify_core_kernel<<<ebz(4 * Lk.ra1 * Lk.n * Lk.m * Lk.ra2), 256, 0, s>>>(Lk.ra1, Lk.n, Lk.m, Lk.ra2, Ai, rA[k], adj);
          realify_phi2_kernel<<<ebz(4 * Lk.rx2 * Lk.ra2 * Lk.ry2), 256, 0, s>>>(Lk.rx2, Lk.ra2, Lk.ry2, p2, rphi2[k], adj);
          TTG_CHECK_LAUNCH();
          MatvecFn smv;
          split_matvec_factory(Lreal(Lk), rphi1[k], rA[k], rphi2[k], kNvecSplit, smem[k],
                               split_bytes, s, &smv, k);
          const i64 Nk = Lk.xsize();
          return [=](const double2* X, double2* Y, int t) {
            for (int v0 = 0; v0 < t; v0 += kNvecSplit) {
              const int nv = std::min(kNvecSplit, t - v0);
              pack_x_kernel<<<ebz(Nk * nv), 256, 0, s>>>(Lk.rx1 * Lk.m, Lk.rx2, nv, X + Nk * v0, rx);
              TTG_CHECK_LAUNCH();
              smv(rx, ryv, nv);
              unpack_y_kernel<<<ebz(Nk * nv), 256, 0, s>>>(Lk.ry1, Lk.n * Lk.ry2, nv, ryv, Y + Nk * v0);
              TTG_CHECK_LAUNCH();
            }
          };
        };
        mv = build(0);
        if (!P.real_scheme) mvT = build(1);
      }
      // the real tt_ksl passes dmatvec as its own transpose (tt_ksl.f90:38-45)
      const double anorm = znormest_dev(w, N, 4, mv, P.real_scheme ? &mv : &mvT, counter, s, &est);
      zexp_mv_dev(w, N, P.order, tau0, cr[i], curcr, eps, anorm, mv, s, &est);
      if (split) split_matvec_check(s, P.real_scheme ? 1 : 2);
    };
    auto sstep = [&](i64 rx1, i64 rx2, i64 ra, i64 ry1, i64 ry2, const double2* ph1,
                     const double2* ph2, const double2* Rin) {
      const i64 N = rx1 * ry2;
      ZMatvecFn mv = [=](const double2* X, double2* Y, int t) {
        sfun_apply(rx1, rx2, ra, ry1, ry2, ph1, ph2, X, Y, t, scratch, s);
      };
      const double anorm = P.diag ? 1.0 : znormest_dev(w, N, 4, mv, nullptr, counter, s, &est);
      zexp_mv_dev(w, N, P.order, -tau0, Rin, Sout, eps, anorm, mv, s, &est);
    };
    if (P.real_scheme) {
      // tt_ksl.f90:312-393.  Backward i = d..1: K-step; for i < d the left QR
      // of the new core and the S-step of R on the bond (i, i+1), core i = Q S;
      // for i > 1 the right QR pushed into core i-1.  Forward i = 1..d: for
      // i < d the left QR and S-step first, then the K-step, then the left QR
      // pushed into core i+1.  tau0 = tau/2 throughout.
      for (int k = 1; k < d; ++k)
        TTG_REQUIRE(ry[k] <= n[k] * ry[k + 1],
                    "tt_ksl: every rank must pass the right-to-left QR unchanged (r_k <= n_k r_{k+1})");
      // QR of X (ry_i n_i x ry_{i+1}) in place, S-step of R, out = Q S
      auto left_s = [&](int i, double2* X, double2* out) {
        const i64 rows = ry[i] * n[i], r2 = ry[i + 1];
        qr_householder_z((int)rows, (int)r2, X, R, tau_ws, s);
        phi_left_z(Ld(i), phi[i], A_of(i), X, X, phitmp, scratch, s);
        sstep(r2, r2, P.ra[i + 1], r2, r2, phitmp, phi[i + 1], R);
        GemmZ g;
        g.M = (int)rows; g.N = (int)r2; g.K = (int)r2;
        g.A = X; g.sAm = 1; g.sAk = rows;
        g.B = Sout; g.sBk = 1; g.sBn = r2;
        g.C = out; g.sCm = 1; g.sCn = rows;
        gemm_z(g, s);
      };
      auto copy = [&](double2* dst, const double2* src, i64 count) {
        TTG_CUDA(cudaMemcpyAsync(dst, src, sizeof(double2) * count, cudaMemcpyDeviceToDevice, s));
      };
      // with d = 1 the backward K-step is never stored (crnew(1) is written
      // only under i < d or i > 1), so one call is the forward half step
      for (int i = d - 1; i >= 0 && d > 1; --i) {
        kstep(i);                                          // curcr
        const double2* cur = curcr;
        if (i < d - 1) {
          left_s(i, curcr, t2);
          cur = t2;
        }
        if (i > 0) {
          const i64 cols = n[i] * ry[i + 1], r1 = ry[i];
          transpose_z(r1, cols, cur, t1, s);               // cols x r1
          qr_householder_z((int)cols, (int)r1, t1, R, tau_ws, s);
          transpose_z(cols, r1, t1, cr[i], s);             // Q^T: r1 x cols
          transpose_z(r1, r1, R, Rt, s);
          GemmZ g;   // core_{i-1} = core_{i-1} R^T
          g.M = (int)(ry[i - 1] * n[i - 1]); g.N = (int)r1; g.K = (int)r1;
          g.A = cr[i - 1]; g.sAm = 1; g.sAk = ry[i - 1] * n[i - 1];
          g.B = Rt; g.sBk = 1; g.sBn = r1;
          g.C = t3; g.sCm = 1; g.sCn = ry[i - 1] * n[i - 1];
          gemm_z(g, s);
          copy(cr[i - 1], t3, ry[i - 1] * n[i - 1] * r1);
          phi_right_z(Ld(i), phi[i + 1], A_of(i), cr[i], cr[i], phi[i], scratch, s);
        } else {
          copy(cr[i], cur, Ld(i).xsize());
        }
      }
      for (int i = 0; i < d; ++i) {
        if (i < d - 1) {
          left_s(i, cr[i], t2);
          copy(cr[i], t2, Ld(i).xsize());
        }
        kstep(i);                                          // curcr
        if (i < d - 1) {
          const i64 rows = ry[i] * n[i], r2 = ry[i + 1];
          qr_householder_z((int)rows, (int)r2, curcr, R, tau_ws, s);
          copy(cr[i], curcr, rows * r2);
          GemmZ g;   // core_{i+1} = R core_{i+1}
          g.M = (int)r2; g.N = (int)(n[i + 1] * ry[i + 2]); g.K = (int)r2;
          g.A = R; g.sAm = 1; g.sAk = r2;
          g.B = cr[i + 1]; g.sBk = 1; g.sBn = r2;
          g.C = t2; g.sCm = 1; g.sCn = r2;
          gemm_z(g, s);
          copy(cr[i + 1], t2, r2 * n[i + 1] * ry[i + 2]);
          phi_left_z(Ld(i), phi[i], A_of(i), cr[i], cr[i], phi[i + 1], scratch, s);
        } else {
          copy(cr[i], curcr, Ld(i).xsize());
        }
      }
      if (P.verb > 0) fprintf(stderr, "tt_ksl: step %d done\n", step + 1);
      continue;
    }
    int i = d - 1, dir = -1, swp = 0;
    while (swp < 1) {
      kstep(i);
      if (dir < 0) {
        if (i > 0) {
          const i64 cols = n[i] * ry[i + 1];
          const i64 rnew = std::min(cols, ry[i]);
          TTG_REQUIRE(rnew == ry[i], "ztt_ksl: the S-step needs a rank-preserving QR");
          transpose_z(ry[i], cols, curcr, t1, s);                    // cols x ry_i
          qr_householder_z((int)cols, (int)ry[i], t1, R, tau_ws, s); // Q: cols x rnew
          transpose_z(cols, rnew, t1, cr[i], s);                     // rnew x cols
          transpose_z(rnew, ry[i], R, Rt, s);                        // ry_i x rnew
          LocalDims Lr{rnew, n[i], ry[i + 1], rnew, n[i], ry[i + 1], P.ra[i], P.ra[i + 1]};
          phi_right_z(Lr, phi[i + 1], A_of(i), cr[i], cr[i], phitmp, scratch, s);
          sstep(ry[i], ry[i], P.ra[i], rnew, rnew, phi[i], phitmp, Rt);
          GemmZ g;   // core_{i-1} = core_{i-1} * Stmp (ry_i x rnew)
          g.M = (int)(ry[i - 1] * n[i - 1]); g.N = (int)rnew; g.K = (int)ry[i];
          g.A = cr[i - 1]; g.sAm = 1; g.sAk = ry[i - 1] * n[i - 1];
          g.B = Sout; g.sBk = 1; g.sBn = ry[i];
          g.C = t2; g.sCm = 1; g.sCn = ry[i - 1] * n[i - 1];
          gemm_z(g, s);
          TTG_CUDA(cudaMemcpyAsync(cr[i - 1], t2, sizeof(double2) * ry[i - 1] * n[i - 1] * rnew,
                                   cudaMemcpyDeviceToDevice, s));
          ry[i] = rnew;
          TTG_CUDA(cudaMemcpyAsync(phi[i], phitmp, sizeof(double2) * rnew * P.ra[i] * rnew,
                                   cudaMemcpyDeviceToDevice, s));
        } else {
          TTG_CUDA(cudaMemcpyAsync(cr[i], curcr, sizeof(double2) * Ld(i).xsize(),
                                   cudaMemcpyDeviceToDevice, s));
        }
      } else {
        if (i < d - 1) {
          const i64 rows = ry[i] * n[i];
          const i64 rnew = std::min(rows, ry[i + 1]);
          TTG_REQUIRE(rnew == ry[i + 1], "ztt_ksl: the S-step needs a rank-preserving QR");
          qr_householder_z((int)rows, (int)ry[i + 1], curcr, R, tau_ws, s);
          TTG_CUDA(cudaMemcpyAsync(cr[i], curcr, sizeof(double2) * rows * rnew,
                                   cudaMemcpyDeviceToDevice, s));
          LocalDims Ll{ry[i], n[i], rnew, ry[i], n[i], rnew, P.ra[i], P.ra[i + 1]};
          phi_left_z(Ll, phi[i], A_of(i), cr[i], cr[i], phitmp, scratch, s);
          sstep(rnew, rnew, P.ra[i + 1], ry[i + 1], ry[i + 1], phitmp, phi[i + 1], R);
          GemmZ g;   // core_{i+1} = Stmp (rnew x ry_{i+1}) * core_{i+1}
          g.M = (int)rnew; g.N = (int)(n[i + 1] * ry[i + 2]); g.K = (int)ry[i + 1];
          g.A = Sout; g.sAm = 1; g.sAk = rnew;
          g.B = cr[i + 1]; g.sBk = 1; g.sBn = ry[i + 1];
          g.C = t2; g.sCm = 1; g.sCn = rnew;
          gemm_z(g, s);
          TTG_CUDA(cudaMemcpyAsync(cr[i + 1], t2, sizeof(double2) * rnew * n[i + 1] * ry[i + 2],
                                   cudaMemcpyDeviceToDevice, s));
          ry[i + 1] = rnew;
          TTG_CUDA(cudaMemcpyAsync(phi[i + 1], phitmp, sizeof(double2) * rnew * rnew * P.ra[i + 1],
                                   cudaMemcpyDeviceToDevice, s));
        } else {
          TTG_CUDA(cudaMemcpyAsync(cr[i], curcr, sizeof(double2) * Ld(i).xsize(),
                                   cudaMemcpyDeviceToDevice, s));
        }
      }
      if (dir > 0 && i == d - 1) {
        dir = -1;
        i = d - 1;
        swp++;
      } else if (dir < 0 && i == 0) {
        dir = 1;
        i = 0;
        if (P.typ == 1) break;
      } else {
        i += dir;
      }
    }
    if (P.verb > 0) fprintf(stderr, "ztt_ksl: step %d done\n", step + 1);
  }
  TTG_CUDA(cudaStreamSynchronize(s));
  i64 tot = 0;
  for (int k = 0; k < d; ++k) tot += ry[k] * n[k] * ry[k + 1];
  out_cores.resize(tot);
  i64 off = 0;
  for (int k = 0; k < d; ++k) {
    const i64 sz = ry[k] * n[k] * ry[k + 1];
    TTG_CUDA(cudaMemcpyAsync(out_cores.data() + off, cr[k], sizeof(double2) * sz,
                             cudaMemcpyDeviceToHost, s));
    off += sz;
  }
  TTG_CUDA(cudaStreamSynchronize(s));
  out_ry = ry;
}

}  // namespace ttg

using namespace ttg;

static void ksl_entry(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* m,
                      const ttg_int* ra, const double2* crA, const double2* crY0, ttg_int* ry,
                      double tau, int verb, int typ, int order, int method, ttg_int nsteps,
                      bool real) {
  TTG_CUDA(cudaSetDevice(ctx->device));
  TTG_REQUIRE(method == TTG_METHOD_PLAIN || method == TTG_METHOD_SPLIT,
              "ksl: method must be PLAIN (FP64) or SPLIT (BF16x3 K-step products)");
  TTG_REQUIRE(typ == 1 || typ == 2, "typ must be 1 (KSL) or 2 (symmetric KSL)");
  KslParams P;
  P.d = (int)d;
  P.n.assign(n, n + d);
  P.m.assign(m, m + d);
  P.ra.assign(ra, ra + d + 1);
  P.ry.assign(ry, ry + d + 1);
  P.crA = crA;
  P.crY0 = crY0;
  P.tau = tau;
  P.typ = typ;
  P.order = order > 0 ? order : 8;
  P.nsteps = nsteps > 0 ? (int)nsteps : 1;
  P.verb = verb;
  P.method = method;
  P.real_scheme = real;
  long long l0 = g_launches;
  ExpStats est;
  est.mxstep = ctx->lim_expsteps > 0 ? ctx->lim_expsteps : 500;
  est.strict = ctx->strict != 0;
  ctx->stat_capped = 0;
  std::vector<i64> ry_out;
  run_ksl(ctx, P, ctx->zresult_core, ry_out, est);
  ctx->stat_capped = est.capped;
  for (int k = 0; k <= d; ++k) ry[k] = ry_out[k];
  ctx->result_core.clear();
  if (real) {
    ctx->result_core.resize(ctx->zresult_core.size());
    for (size_t e = 0; e < ctx->zresult_core.size(); ++e) ctx->result_core[e] = ctx->zresult_core[e].real();
    ctx->zresult_core.clear();
  }
  ctx->stat_matvecs = est.nmult;
  ctx->stat_sweeps = P.nsteps;
  ctx->stat_res = 0.0;
  ctx->stat_launches = g_launches - l0;
}

extern "C" int ttg_ksl_z(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* m,
                         const ttg_int* ra, const double* crA, const double* crY0, ttg_int* ry,
                         double tau, ttg_int rmax, int verb, int typ, int order, int method,
                         ttg_int nsteps) {
  if (!ctx) return TTG_ERR_ARG;
  try {
    TTG_REQUIRE(d > 0 && n && m && ra && crA && crY0 && ry, "null argument");
    (void)rmax;   // read but unused by the reference as well (tt_ksl.f90:446)
    ksl_entry(ctx, d, n, m, ra, (const double2*)crA, (const double2*)crY0, ry, tau, verb, typ,
              order, method, nsteps, false);
  } catch (const ttg::Error& e) {
    ctx->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}

// tt_ksl (tt_ksl.f90:191-428): real operator and start, the real scheme's
// sweep, computed in complex arithmetic on real data (the imaginary parts
// stay zero); the real parts go to the real result.  typ is read but, as in
// the reference, the scheme is always the symmetric one.
extern "C" int ttg_ksl_d(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* m,
                         const ttg_int* ra, const double* crA, const double* crY0, ttg_int* ry,
                         double tau, ttg_int rmax, int verb, int typ, int order, int method,
                         ttg_int nsteps) {
  if (!ctx) return TTG_ERR_ARG;
  try {
    TTG_REQUIRE(d > 0 && n && m && ra && crA && crY0 && ry, "null argument");
    (void)rmax;   // read but unused by the reference as well (tt_ksl.f90:234-245)
    i64 na = 0, ny = 0;
    for (ttg_int k = 0; k < d; ++k) {
      TTG_REQUIRE(n[k] > 0 && m[k] > 0 && ra[k] > 0 && ry[k] > 0, "sizes must be positive");
      na += ra[k] * n[k] * m[k] * ra[k + 1];
      ny += ry[k] * n[k] * ry[k + 1];
    }
    std::vector<double2> zA(na), zY(ny);
    for (i64 e = 0; e < na; ++e) zA[e] = make_double2(crA[e], 0.0);
    for (i64 e = 0; e < ny; ++e) zY[e] = make_double2(crY0[e], 0.0);
    ksl_entry(ctx, d, n, m, ra, zA.data(), zY.data(), ry, tau, verb, typ, order, method, nsteps,
              true);
  } catch (const ttg::Error& e) {
    ctx->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}

// ztt_diag_ksl / dtt_diag_ksl (tt_diag_ksl.f90:315-804): KSL for operators
// diagonal in the physical index.  The real version runs the same scheme in
// complex arithmetic on real data (the imaginary parts stay zero) and returns
// the real parts.
static int diag_ksl_entry(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* ra,
                          const double2* crA, const double2* crY0, ttg_int* ry, double tau,
                          int verb, int typ, int order, ttg_int nsteps, bool real_out) {
  TTG_CUDA(cudaSetDevice(ctx->device));
  TTG_REQUIRE(typ == 1 || typ == 2, "typ must be 1 (KSL) or 2 (symmetric KSL)");
  KslParams P;
  P.d = (int)d;
  P.n.assign(n, n + d);
  P.m.assign(n, n + d);
  P.ra.assign(ra, ra + d + 1);
  P.ry.assign(ry, ry + d + 1);
  P.crA = crA;
  P.crY0 = crY0;
  P.tau = tau;
  P.typ = typ;
  P.order = order > 0 ? order : 8;
  P.nsteps = nsteps > 0 ? (int)nsteps : 1;
  P.verb = verb;
  P.diag = true;
  long long l0 = g_launches;
  ExpStats est;
  est.mxstep = ctx->lim_expsteps > 0 ? ctx->lim_expsteps : 500;
  est.strict = ctx->strict != 0;
  ctx->stat_capped = 0;
  std::vector<i64> ry_out;
  run_ksl(ctx, P, ctx->zresult_core, ry_out, est);
  ctx->stat_capped = est.capped;
  for (int k = 0; k <= d; ++k) ry[k] = ry_out[k];
  ctx->result_core.clear();
  if (real_out) {
    ctx->result_core.resize(ctx->zresult_core.size());
    for (size_t e = 0; e < ctx->zresult_core.size(); ++e) ctx->result_core[e] = ctx->zresult_core[e].real();
    ctx->zresult_core.clear();
  }
  ctx->stat_matvecs = est.nmult;
  ctx->stat_sweeps = P.nsteps;
  ctx->stat_res = 0.0;
  ctx->stat_launches = g_launches - l0;
  return TTG_OK;
}

extern "C" int ttg_diag_ksl_z(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* ra,
                              const double* crA, const double* crY0, ttg_int* ry, double tau,
                              ttg_int rmax, int verb, int typ, int order, ttg_int nsteps) {
  if (!ctx) return TTG_ERR_ARG;
  try {
    TTG_REQUIRE(d > 0 && n && ra && crA && crY0 && ry, "null argument");
    (void)rmax;   // read but unused by the reference as well (tt_diag_ksl.f90:600)
    return diag_ksl_entry(ctx, d, n, ra, (const double2*)crA, (const double2*)crY0, ry, tau, verb,
                          typ, order, nsteps, false);
  } catch (const ttg::Error& e) {
    ctx->last_error = e.msg;
    return e.code;
  }
}

extern "C" int ttg_diag_ksl_d(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* ra,
                              const double* crA, const double* crY0, ttg_int* ry, double tau,
                              ttg_int rmax, int verb, int typ, int order, ttg_int nsteps) {
  if (!ctx) return TTG_ERR_ARG;
  try {
    TTG_REQUIRE(d > 0 && n && ra && crA && crY0 && ry, "null argument");
    (void)rmax;
    i64 na = 0, ny = 0;
    for (ttg_int k = 0; k < d; ++k) {
      na += ra[k] * n[k] * ra[k + 1];
      ny += ry[k] * n[k] * ry[k + 1];
    }
    std::vector<double2> zA(na), zY(ny);
    for (i64 e = 0; e < na; ++e) zA[e] = make_double2(crA[e], 0.0);
    for (i64 e = 0; e < ny; ++e) zY[e] = make_double2(crY0[e], 0.0);
    return diag_ksl_entry(ctx, d, n, ra, zA.data(), zY.data(), ry, tau, verb, typ, order, nsteps,
                          true);
  } catch (const ttg::Error& e) {
    ctx->last_error = e.msg;
    return e.code;
  }
}
