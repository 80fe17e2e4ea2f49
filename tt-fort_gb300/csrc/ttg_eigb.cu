// Block-TT ALS eigensolver driver (tt_eigb, tt_eigb.f90:110-436) on the GPU.
//
// Every array of the sweep stays in HBM for the whole call: operator cores,
// TT cores (each with capacity rank_cap * n * rank_cap * B), interface
// matrices Phi, the Davidson basis and the SVD workspace are carved out of one
// allocation made before the first sweep.  The host keeps the reference's
// control flow (sweep order, turn points, stopping rule) and reads back only
// scalars: B eigenvalues and residual norms per Davidson iteration and the
// singular values that my_chop3 needs.
#include "ttg_davidson.cuh"
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <numeric>
#include <thread>

namespace ttg {

size_t chosen_bytes(i64 N, int B);
DavidsonStats chosen_solve(i64 N, int B, void* dav_mem, double* hbuf, void* jd_mem,
                           const MatvecFn& mv64, const MatvecFn& mvlow, const double* X0,
                           double tol, int max_matvecs, double* X, double* theta_host,
                           cudaStream_t s, DavTimer* timer, int* fp64_matvecs);

struct DevBlock {
  char* base = nullptr;
  size_t top = 0, cap = 0;
  ~DevBlock() { if (base) cudaFree(base); }
  void alloc(size_t bytes) {
    if (cudaMalloc(&base, bytes) != cudaSuccess) {
      base = nullptr;
      throw Error{TTG_ERR_NOMEM, "tt_eigb: device allocation failed"};
    }
    cap = bytes;
  }
  template <class T> T* take(size_t count) {
    size_t b = (count * sizeof(T) + 255) & ~size_t(255);
    if (top + b > cap) throw Error{TTG_ERR_NOMEM, "tt_eigb: device block exhausted"};
    T* p = (T*)(base + top);
    top += b;
    return p;
  }
};

struct PinnedBuf {
  double* p = nullptr;
  explicit PinnedBuf(size_t n) { TTG_CUDA(cudaMallocHost(&p, n * sizeof(double))); }
  ~PinnedBuf() { if (p) cudaFreeHost(p); }
};

static inline size_t al(size_t bytes) { return (bytes + 255) & ~size_t(255); }

struct EigbParams {
  int d;
  std::vector<i64> n, m, ra, ry;
  const double* crA;
  const double* crY0;
  double eps;
  i64 rmax;
  int B;
  int nswp;
  i64 max_full_size;
  int verb;
  int method;
};

struct EigbOutput {
  std::vector<double> lambda;
  std::vector<double> cores;
  std::vector<i64> ry;
  long long matvecs = 0;
  long long fp64_matvecs = 0;
  int sweeps = 0;
  double res = 0.0;
};

// TTG_PROFILE=1: synchronise after every phase and print where the time went
struct PhaseTimer {
  bool on = false;
  cudaStream_t s = nullptr;
  double t[8] = {0};
  std::chrono::steady_clock::time_point t0;
  void start() {
    if (!on) return;
    cudaStreamSynchronize(s);
    t0 = std::chrono::steady_clock::now();
  }
  void stop(int k) {
    if (!on) return;
    cudaStreamSynchronize(s);
    t[k] += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  DavTimer dav;
  void report() {
    if (!on) return;
    const char* nm[8] = {"qr-init", "dense", "davidson", "svd", "fold", "phi", "other", "mv"};
    for (int k = 0; k < 8; ++k) fprintf(stderr, "[ttg profile] %-9s %8.3f s\n", nm[k], t[k]);
    const char* dn[7] = {"init", "rr-eig", "ritz+res", "restart", "orth", "matvec", "h-update"};
    for (int k = 0; k < 7; ++k) fprintf(stderr, "[ttg profile]   dav %-9s %8.3f s\n", dn[k], dav.t[k]);
    fprintf(stderr, "[ttg profile]   dav iters %lld restarts %lld jacobi sweeps %lld\n", dav.iters,
            dav.restarts, dav.jac_sweeps);
    fprintf(stderr, "[ttg profile]   fp64 matvecs %lld of %lld\n", fp64_mv_report, all_mv_report);
  }
  long long fp64_mv_report = 0, all_mv_report = 0;
};

static void run_eigb(ttg_ctx* ctx, EigbParams P, EigbOutput& out) {
  cudaStream_t s = ctx->stream;
  PhaseTimer pt;
  pt.on = std::getenv("TTG_PROFILE") != nullptr;
  pt.s = s;
  const int d = P.d, B = P.B;
  auto& n = P.n;
  auto& ry = P.ry;
  TTG_REQUIRE(d >= 2, "tt_eigb: d must be >= 2");
  TTG_REQUIRE(ry[d] == B, "Inconsistent number of eigenvalues sought and initial guess last rank");
  TTG_REQUIRE(ry[0] == 1 && P.ra[0] == 1 && P.ra[d] == 1, "boundary ranks must be 1");
  TTG_REQUIRE(B >= 1 && B <= 16, "B must be in [1, 16]");
  for (int i = 0; i < d; ++i) TTG_REQUIRE(n[i] == P.m[i], "tt_eigb needs square cores (n == m)");
  const double eps2 = P.eps / std::sqrt((double)d);
  const double resid_damp = 10.0;
  // PRIMME's maxMatvecs (tt_eigb.f90:152,269), or the context's cap
  const int max_matvecs = ctx->lim_matvecs > 0 ? ctx->lim_matvecs : 500;
  ctx->stat_capped = 0;

  // operator offsets (compute_ps, matrix_util.f90:242-251)
  std::vector<i64> pa(d + 1, 0);
  for (int i = 0; i < d; ++i) pa[i + 1] = pa[i] + P.ra[i] * n[i] * P.m[i] * P.ra[i + 1];
  // rank capacities
  std::vector<i64> Rc(d + 1);
  Rc[0] = 1;
  Rc[d] = 1;
  for (int i = 1; i < d; ++i) Rc[i] = std::max(ry[i], P.rmax);
  std::vector<i64> capc(d), capphi(d + 1);
  i64 Nmax = 1, capmax = 1;
  for (int i = 0; i < d; ++i) {
    capc[i] = Rc[i] * n[i] * Rc[i + 1] * B;
    if (i == d - 1) capc[i] = std::max(capc[i], ry[d - 1] * n[d - 1] * B);
    capmax = std::max(capmax, capc[i]);
    Nmax = std::max(Nmax, Rc[i] * n[i] * Rc[i + 1]);
  }
  for (int i = 0; i <= d; ++i) capphi[i] = Rc[i] * Rc[i] * P.ra[i];
  size_t svdmax = 0;
  i64 rmaxsvd = 1;
  for (int i = 0; i < d; ++i) {
    int p1 = (int)(B * Rc[i]), q1 = (int)(n[i] * Rc[i + 1]);
    int p2 = (int)(Rc[i] * n[i]), q2 = (int)(Rc[i + 1] * B);
    svdmax = std::max({svdmax, svd_scratch(p1, q1), svd_scratch(p2, q2)});
    rmaxsvd = std::max<i64>(rmaxsvd, std::max(std::min(p1, q1), std::min(p2, q2)));
  }
  size_t bf_scr = 0, phi_scr = 0, split_bytes = 0;
  for (int i = 0; i < d; ++i) {
    LocalDims L{Rc[i], n[i], Rc[i + 1], Rc[i], n[i], Rc[i + 1], P.ra[i], P.ra[i + 1]};
    bf_scr = std::max(bf_scr, bfun3_f64_scratch(L, B));
    phi_scr = std::max(phi_scr, phi_f64_scratch(L));
    if (P.method == TTG_METHOD_SPLIT) split_bytes = std::max(split_bytes, split_matvec_bytes(L, B));
  }
  const i64 dense_max = std::min<i64>(P.max_full_size - 1, 512);
  const int maxb_cap = (int)std::min<i64>(std::max(4 * B, 32), Nmax);
  TTG_REQUIRE(maxb_cap <= 128, "davidson basis too large");

  size_t total = al(sizeof(double) * pa[d]);
  for (int i = 0; i < d; ++i) total += al(sizeof(double) * capc[i]);
  for (int i = 0; i <= d; ++i) total += al(sizeof(double) * capphi[i]);
  total += al(sizeof(double) * Nmax * B);          // curcr
  total += 2 * al(sizeof(double) * capmax);        // tmp, tmp2
  total += al(svdmax) + al(sizeof(double) * capmax) * 2 + al(sizeof(double) * rmaxsvd * 2);
  total += al(bf_scr) + al(phi_scr) + al(split_bytes);
  total += 2 * al(sizeof(double) * dense_max * dense_max) + al(sizeof(double) * 512) + al(256);
  total += al(syev_lowest_scratch((int)std::max<i64>(1, dense_max)));
  total += al(Davidson::bytes(Nmax, B, maxb_cap));
  const bool jd = P.method == TTG_METHOD_SPLIT || P.method == TTG_METHOD_JD64;
  if (jd) total += al(chosen_bytes(Nmax, B));
  const bool learned_prec = P.method == TTG_METHOD_PLAIN && ctx->learned && (ctx->learned_mode & 1);
  const bool record = P.method == TTG_METHOD_PLAIN && (ctx->learned_mode & 2);
  if (learned_prec) total += al(sizeof(double) * Nmax);
  total += 1 << 16;
  DevBlock mem;
  mem.alloc(total);
  double* dA = mem.take<double>(pa[d]);
  std::vector<double*> cr(d), phi(d + 1);
  for (int i = 0; i < d; ++i) cr[i] = mem.take<double>(capc[i]);
  for (int i = 0; i <= d; ++i) phi[i] = mem.take<double>(capphi[i]);
  double* curcr = mem.take<double>(Nmax * B);
  double* tmp = mem.take<double>(capmax);
  double* tmp2 = mem.take<double>(capmax);
  double* svd_scr = (double*)mem.take<char>(svdmax);
  double* sU = mem.take<double>(capmax);
  double* sVt = mem.take<double>(capmax);
  double* sS = mem.take<double>(rmaxsvd * 2);
  double* bfs = (double*)mem.take<char>(bf_scr);
  double* phs = (double*)mem.take<char>(phi_scr);
  void* split_mem = split_bytes ? (void*)mem.take<char>(split_bytes) : nullptr;
  double* dH = mem.take<double>(std::max<i64>(1, dense_max * dense_max));
  double* dV = mem.take<double>(std::max<i64>(1, dense_max * dense_max));
  double* dw = mem.take<double>(512);
  double* dscr = (double*)mem.take<char>(syev_lowest_scratch((int)std::max<i64>(1, dense_max)));
  int* dst = mem.take<int>(64);
  void* dav_mem = mem.take<char>(Davidson::bytes(Nmax, B, maxb_cap));
  void* jd_mem = jd ? (void*)mem.take<char>(chosen_bytes(Nmax, B)) : nullptr;
  double* ldiag = learned_prec ? mem.take<double>(Nmax) : nullptr;
  PinnedBuf hb(4096 + rmaxsvd * 2);
  double* hbuf = hb.p;

  // upload operator and start cores
  TTG_CUDA(cudaMemcpyAsync(dA, P.crA, sizeof(double) * pa[d], cudaMemcpyHostToDevice, s));
  {
    i64 off = 0;
    for (int i = 0; i < d; ++i) {
      i64 sz = ry[i] * n[i] * ry[i + 1];
      TTG_CUDA(cudaMemcpyAsync(cr[i], P.crY0 + off, sizeof(double) * sz, cudaMemcpyHostToDevice, s));
      off += sz;
    }
  }
  fill_f64(phi[0], 1, 1.0, s);
  fill_f64(phi[d], 1, 1.0, s);
  auto A_of = [&](int i) { return dA + pa[i]; };
  auto dimsL = [&](int i) {
    return LocalDims{ry[i], n[i], ry[i + 1], ry[i], n[i], ry[i + 1], P.ra[i], P.ra[i + 1]};
  };

  // QR orthogonalisation left to right, tt_eigb.f90:202-217
  pt.start();
  for (int i = 0; i < d; ++i) {
    i64 rows = ry[i] * n[i];
    i64 rnew = std::min(rows, ry[i + 1]);
    qr_householder((int)rows, (int)ry[i + 1], cr[i], tmp, tmp2, s);
    if (i < d - 1) {
      GemmF64 g;   // cr[i+1] = R (rnew x ry[i+1]) * cr[i+1] (ry[i+1] x n ry[i+2])
      g.M = (int)rnew; g.N = (int)(n[i + 1] * ry[i + 2]); g.K = (int)ry[i + 1];
      g.A = tmp; g.sAm = 1; g.sAk = rnew;
      g.B = cr[i + 1]; g.sBk = 1; g.sBn = ry[i + 1];
      g.C = tmp2; g.sCm = 1; g.sCn = rnew;
      gemm_f64(g, s);
      TTG_CUDA(cudaMemcpyAsync(cr[i + 1], tmp2, sizeof(double) * rnew * n[i + 1] * ry[i + 2],
                               cudaMemcpyDeviceToDevice, s));
      ry[i + 1] = rnew;
      phi_left_f64(dimsL(i), phi[i], A_of(i), cr[i], cr[i], phi[i + 1], phs, s);
    }
  }
  ry[d] = 1;
  pt.stop(0);

  int i = d - 1, dir = -1, swp = 1;
  double ermax = 0.0, fvold = 0.0, res = 0.0;
  std::vector<double> lam(B, 0.0);
  long long total_mv = 0, fp64_mv = 0;
  while (swp <= P.nswp) {
    const i64 N = ry[i] * n[i] * ry[i + 1];
    TTG_REQUIRE(N >= B, "local problem smaller than the block size");
    int nmv = 0;
    pt.start();
    if (N < P.max_full_size && N <= dense_max) {
      // dense branch: d2d_fullmat + dsyev, tt_eigb.f90:234-249
      fullmat_f64(ry[i], n[i], ry[i + 1], P.ra[i], P.ra[i + 1], phi[i], A_of(i), phi[i + 1], dH, s);
      syev_lowest_svd((int)N, B, dH, dw, dV, dscr, dst, s);
      TTG_CUDA(cudaMemcpyAsync(curcr, dV, sizeof(double) * N * B, cudaMemcpyDeviceToDevice, s));
      TTG_CUDA(cudaMemcpyAsync(hbuf, dw, sizeof(double) * B, cudaMemcpyDeviceToHost, s));
      TTG_CUDA(cudaStreamSynchronize(s));
      for (int j = 0; j < B; ++j) lam[j] = hbuf[j];
      res = 0.0;
      pt.stop(1);
    } else {
      LocalDims L = dimsL(i);
      const double* p1 = phi[i];
      const double* Ai = A_of(i);
      const double* p2 = phi[i + 1];
      MatvecFn mv = [=](const double* X, double* Y, int nv) { bfun3_f64(L, p1, Ai, p2, X, Y, nv, bfs, s); };
      MatvecFn mvlow;
      if (P.method == TTG_METHOD_SPLIT)
        split_matvec_factory(L, p1, Ai, p2, B, split_mem, split_bytes, s, &mvlow);
      if (P.method == TTG_METHOD_JD64) mvlow = mv;   // ablation: the same solver, FP64 products
      if (pt.on) {
        PhaseTimer* ptp = &pt;
        auto wrap = [ptp](MatvecFn inner) {
          return MatvecFn([inner, ptp](const double* X, double* Y, int nv) {
            cudaStreamSynchronize(ptp->s);
            auto a = std::chrono::steady_clock::now();
            inner(X, Y, nv);
            cudaStreamSynchronize(ptp->s);
            ptp->t[7] += std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
          });
        };
        mv = wrap(mv);
        if (mvlow) mvlow = wrap(mvlow);
      }
      DavidsonStats st;
      if (jd) {
        if (pt.on) pt.dav.s = s;
        int n64 = 0;
        st = chosen_solve(N, B, dav_mem, hbuf, jd_mem, mv, mvlow, cr[i], eps2 / resid_damp,
                          max_matvecs, curcr, lam.data(), s, pt.on ? &pt.dav : nullptr, &n64);
        fp64_mv += n64;
        if (P.method == TTG_METHOD_SPLIT) split_matvec_check(s);
      } else {
        const int maxb = (int)std::min<i64>(std::max(4 * B, 32), N);
        const int keep = std::min(B + std::max(1, B / 2), std::max(maxb - B, 1));
        Davidson dav(N, B, maxb, keep, dav_mem, hbuf, s);
        if (pt.on) { pt.dav.s = s; dav.timer = &pt.dav; }
        // learned preconditioner (no reference counterpart): the Davidson
        // expansions use it; the FP64 residual test still judges convergence
        if (learned_prec) dav.prec = make_learned_prec(ctx->learned, L, p1, Ai, p2, ldiag, s);
        st = dav.solve(mv, cr[i], eps2 / resid_damp, max_matvecs, curcr, lam.data());
        fp64_mv += st.matvecs;
        if (record) learned_record(ctx, L, p1, Ai, p2, cr[i], curcr, B, mv, s);
      }
      nmv = st.matvecs;
      res = st.res;
      if (!st.converged) {
        // the reference tolerates PRIMME's -3 (maxMatvecs reached) and goes
        // on with the current block (tt_eigb.f90:285-288)
        ++ctx->stat_capped;
        if (ctx->strict)
          throw Error{TTG_ERR_NOCONV, "tt_eigb: local eigensolve at core " + std::to_string(i) +
                                          " reached the matvec cap (" +
                                          std::to_string(max_matvecs) + ") before its tolerance"};
      }
      pt.stop(2);
    }
    double fv = 0.0;
    for (int j = 0; j < B; ++j) fv += lam[j];
    double erloc = (fvold - fv) / std::fabs(fv);
    ermax = std::max(ermax, erloc);
    total_mv += nmv;
    fvold = fv;
    if (P.verb > 0)
      fprintf(stderr, "swp: %d i: [%d/%d] loc_size: %lld matvecs: %d res: %.3e ermax: %.3e\n", swp,
              i + 1, d, (long long)N, nmv, res, ermax);

    if (dir < 0 && i > 0) {
      // tt_eigb.f90:305-356
      const int p = (int)(B * ry[i]), q = (int)(n[i] * ry[i + 1]);
      const int r = std::min(p, q);
      pt.start();
      transpose_f64(N, B, curcr, tmp, s);                // (B ry_i) x (n ry_{i+1})
      svd_jacobi(p, q, tmp, sU, sS, sVt, svd_scr, dst, s);
      TTG_CUDA(cudaMemcpyAsync(hbuf, sS, sizeof(double) * r, cudaMemcpyDeviceToHost, s));
      TTG_CUDA(cudaStreamSynchronize(s));
      pt.stop(3);
      pt.start();
      i64 nn = std::min<i64>(ttg_my_chop3(r, hbuf, eps2), P.rmax);
      copy_rows_f64(r, nn, q, sVt, cr[i], s);             // core i = Vt(1:nn, :)
      scale_cols_f64(p, nn, sU, p, sS, s);               // U(:, 1:nn) diag(s)
      transpose_f64(B, ry[i] * nn, sU, tmp, s);          // ry_i x nn x B
      GemmF64 g;   // cr[i-1] (ry_{i-1} n_{i-1} x nn B) = cr[i-1] * Ut
      g.M = (int)(ry[i - 1] * n[i - 1]); g.N = (int)(nn * B); g.K = (int)ry[i];
      g.A = cr[i - 1]; g.sAm = 1; g.sAk = ry[i - 1] * n[i - 1];
      g.B = tmp; g.sBk = 1; g.sBn = ry[i];
      g.C = tmp2; g.sCm = 1; g.sCn = ry[i - 1] * n[i - 1];
      gemm_f64(g, s);
      TTG_CUDA(cudaMemcpyAsync(cr[i - 1], tmp2, sizeof(double) * ry[i - 1] * n[i - 1] * nn * B,
                               cudaMemcpyDeviceToDevice, s));
      ry[i] = nn;
      pt.stop(4);
      pt.start();
      phi_right_f64(dimsL(i), phi[i + 1], A_of(i), cr[i], cr[i], phi[i], phs, s);
      pt.stop(5);
    }
    if (dir > 0 && i < d - 1) {
      // tt_eigb.f90:357-394
      const int p = (int)(ry[i] * n[i]), q = (int)(ry[i + 1] * B);
      const int r = std::min(p, q);
      pt.start();
      svd_jacobi(p, q, curcr, sU, sS, sVt, svd_scr, dst, s);
      TTG_CUDA(cudaMemcpyAsync(hbuf, sS, sizeof(double) * r, cudaMemcpyDeviceToHost, s));
      TTG_CUDA(cudaStreamSynchronize(s));
      pt.stop(3);
      pt.start();
      i64 nn = std::min<i64>(ttg_my_chop3(r, hbuf, eps2), P.rmax);
      TTG_CUDA(cudaMemcpyAsync(cr[i], sU, sizeof(double) * p * nn, cudaMemcpyDeviceToDevice, s));
      copy_rows_f64(r, nn, q, sVt, tmp, s);               // Vt(1:nn,:)  nn x (ry_{i+1} B)
      scale_rows_f64(nn, q, tmp, nn, sS, s);              // S Vt
      transpose_f64(nn * ry[i + 1], B, tmp, tmp2, s);    // B x nn x ry_{i+1}
      GemmF64 g;   // cur (B nn x n ry_{i+2}) = SVt (B nn x ry_{i+1}) * cr[i+1]
      g.M = (int)(B * nn); g.N = (int)(n[i + 1] * ry[i + 2]); g.K = (int)ry[i + 1];
      g.A = tmp2; g.sAm = 1; g.sAk = B * nn;
      g.B = cr[i + 1]; g.sBk = 1; g.sBn = ry[i + 1];
      g.C = tmp; g.sCm = 1; g.sCn = B * nn;
      gemm_f64(g, s);
      transpose_f64(B, nn * n[i + 1] * ry[i + 2], tmp, cr[i + 1], s);
      ry[i + 1] = nn;
      pt.stop(4);
      pt.start();
      phi_left_f64(dimsL(i), phi[i], A_of(i), cr[i], cr[i], phi[i + 1], phs, s);
      pt.stop(5);
    }
    if (dir > 0 && i == d - 2) {
      dir = -1;
      i = d - 1;
      if (P.verb > 0) {
        i64 rm = *std::max_element(ry.begin(), ry.begin() + d);
        fprintf(stderr, "swp: %d er = %.3e rmax:%lld\n", swp, ermax, (long long)rm);
      }
      swp++;
      if (ermax < P.eps) break;
      ermax = 0.0;
    } else if (dir < 0 && i == 1) {
      dir = 1;
      i = 0;
    } else {
      i += dir;
    }
  }
  ry[d] = B;
  TTG_CUDA(cudaStreamSynchronize(s));
  i64 tot = 0;
  for (int k = 0; k < d; ++k) tot += ry[k] * n[k] * ry[k + 1];
  out.cores.resize(tot);
  i64 off = 0;
  for (int k = 0; k < d; ++k) {
    i64 sz = ry[k] * n[k] * ry[k + 1];
    TTG_CUDA(cudaMemcpyAsync(out.cores.data() + off, cr[k], sizeof(double) * sz,
                             cudaMemcpyDeviceToHost, s));
    off += sz;
  }
  TTG_CUDA(cudaStreamSynchronize(s));
  pt.fp64_mv_report = fp64_mv;
  pt.all_mv_report = total_mv;
  pt.report();
  out.lambda = lam;
  out.ry = ry;
  out.matvecs = total_mv;
  out.fp64_matvecs = fp64_mv;
  out.sweeps = swp - 1;
  out.res = res;
}

}  // namespace ttg

using namespace ttg;

extern "C" int ttg_eigb(ttg_ctx* ctx, ttg_int d, const ttg_int* n, const ttg_int* m,
                        const ttg_int* ra, const double* crA, const double* crY0, ttg_int* ry,
                        double eps, ttg_int rmax, double* lambda, ttg_int B, ttg_int nswp,
                        ttg_int max_full_size, int verb, int method) {
  if (!ctx) return TTG_ERR_ARG;
  try {
    TTG_CUDA(cudaSetDevice(ctx->device));
    TTG_REQUIRE(d > 0 && n && m && ra && crA && crY0 && ry && lambda, "null argument");
    TTG_REQUIRE(method == TTG_METHOD_PLAIN || method == TTG_METHOD_SPLIT ||
                    method == TTG_METHOD_JD64,
                "unknown method");
    EigbParams P;
    P.d = (int)d;
    P.n.assign(n, n + d);
    P.m.assign(m, m + d);
    P.ra.assign(ra, ra + d + 1);
    P.ry.assign(ry, ry + d + 1);
    P.crA = crA;
    P.crY0 = crY0;
    P.eps = eps;
    P.rmax = rmax;
    P.B = (int)B;
    P.nswp = (int)(nswp > 0 ? nswp : 20);
    P.max_full_size = max_full_size > 0 ? max_full_size : 2000;
    P.verb = verb;
    P.method = method;
    long long l0 = g_launches;
    EigbOutput out;
    run_eigb(ctx, P, out);
    for (int k = 0; k <= d; ++k) ry[k] = out.ry[k];
    for (int k = 0; k < B; ++k) lambda[k] = out.lambda[k];
    ctx->result_core = std::move(out.cores);
    ctx->zresult_core.clear();
    ctx->stat_matvecs = out.matvecs;
    ctx->stat_sweeps = out.sweeps;
    ctx->stat_res = out.res;
    ctx->stat_launches = g_launches - l0;
  } catch (const ttg::Error& e) {
    ctx->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}

// ---------------------------------------------------------------------------
// Batched eigen sweeps: many independent chains (no counterpart in the
// reference, whose tt_eigb solves one chain per call).  A single chain's
// sweep is sequential, so a batch is spread over worker threads, each with
// its own context and non-blocking stream; the chains' kernels overlap on
// the GPU.  Chains are taken longest first (estimated cost d * rmax^3 * B).
// ---------------------------------------------------------------------------
struct ttg_batch {
  ttg_ctx* ctx = nullptr;
  int nworkers = 1;
  struct Job {
    int d = 0;
    std::vector<i64> n, m, ra, ry;
    std::vector<double> crA, crY0;
    double eps = 0.0;
    i64 rmax = 0;
    int B = 1, nswp = 20, method = 0;
    i64 mfs = 2000;
    // results
    int status = 1;           // 1: not run
    std::string msg;
    EigbOutput out;
    double seconds = 0.0;
  };
  std::vector<Job> jobs;
};

extern "C" int ttg_batch_create(ttg_ctx* ctx, int nworkers, ttg_batch** out) {
  if (!ctx || !out || nworkers < 1 || nworkers > 256) return TTG_ERR_ARG;
  ttg_batch* b = new ttg_batch();
  b->ctx = ctx;
  b->nworkers = nworkers;
  *out = b;
  return TTG_OK;
}

extern "C" int ttg_batch_destroy(ttg_batch* b) {
  if (!b) return TTG_ERR_ARG;
  delete b;
  return TTG_OK;
}

extern "C" int ttg_batch_add_eigb(ttg_batch* b, ttg_int d, const ttg_int* n, const ttg_int* m,
                                  const ttg_int* ra, const double* crA, const double* crY0,
                                  const ttg_int* ry, double eps, ttg_int rmax, ttg_int B,
                                  ttg_int nswp, ttg_int max_full_size, int method, ttg_int* index) {
  if (!b) return TTG_ERR_ARG;
  ttg_ctx* c = b->ctx;
  try {
    TTG_REQUIRE(d > 0 && n && m && ra && crA && crY0 && ry && B > 0, "batch: null or bad argument");
    TTG_REQUIRE(method == TTG_METHOD_PLAIN || method == TTG_METHOD_SPLIT, "unknown method");
    TTG_REQUIRE(ry[d] == B, "batch: ry[d] must equal B");
    ttg_batch::Job j;
    j.d = (int)d;
    j.n.assign(n, n + d);
    j.m.assign(m, m + d);
    j.ra.assign(ra, ra + d + 1);
    j.ry.assign(ry, ry + d + 1);
    i64 na = 0, ny = 0;
    for (int k = 0; k < d; ++k) {
      na += ra[k] * n[k] * m[k] * ra[k + 1];
      ny += ry[k] * n[k] * ry[k + 1];
    }
    j.crA.assign(crA, crA + na);
    j.crY0.assign(crY0, crY0 + ny);
    j.eps = eps;
    j.rmax = rmax;
    j.B = (int)B;
    j.nswp = (int)(nswp > 0 ? nswp : 20);
    j.mfs = max_full_size > 0 ? max_full_size : 2000;
    j.method = method;
    b->jobs.push_back(std::move(j));
    if (index) *index = (ttg_int)b->jobs.size() - 1;
  } catch (const ttg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  }
  return TTG_OK;
}

// Runs every chain that has not run yet.  Returns TTG_OK when all succeeded,
// else the first failing chain's status (each chain's own status and message
// are kept: ttg_batch_result).
extern "C" int ttg_batch_run(ttg_batch* b) {
  if (!b) return TTG_ERR_ARG;
  ttg_ctx* c = b->ctx;
  std::vector<int> order;
  for (int i = 0; i < (int)b->jobs.size(); ++i)
    if (b->jobs[i].status == 1) order.push_back(i);
  auto cost = [&](int i) {
    const auto& j = b->jobs[i];
    const double r = (double)std::max<i64>(1, j.rmax);
    return (double)j.d * r * r * r * j.B;
  };
  std::stable_sort(order.begin(), order.end(), [&](int a, int z) { return cost(a) > cost(z); });
  std::atomic<size_t> next{0};
  const int nw = std::max(1, std::min<int>(b->nworkers, (int)order.size()));
  auto worker = [&]() {
    ttg_ctx* wc = nullptr;
    const int rc0 = ttg_create(c->device, &wc);
    while (true) {
      const size_t q = next.fetch_add(1);
      if (q >= order.size()) break;
      auto& j = b->jobs[order[q]];
      if (rc0 != TTG_OK) {
        j.status = TTG_ERR_CUDA;
        j.msg = "batch: worker context creation failed";
        continue;
      }
      try {
        TTG_CUDA(cudaSetDevice(wc->device));
        EigbParams P;
        P.d = j.d;
        P.n = j.n; P.m = j.m; P.ra = j.ra; P.ry = j.ry;
        P.crA = j.crA.data();
        P.crY0 = j.crY0.data();
        P.eps = j.eps;
        P.rmax = j.rmax;
        P.B = j.B;
        P.nswp = j.nswp;
        P.max_full_size = j.mfs;
        P.verb = 0;
        P.method = j.method;
        const auto t0 = std::chrono::steady_clock::now();
        run_eigb(wc, P, j.out);
        j.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        j.status = TTG_OK;
      } catch (const ttg::Error& e) {
        j.status = e.code;
        j.msg = e.msg;
      }
    }
    if (wc) ttg_destroy(wc);
  };
  std::vector<std::thread> th;
  for (int w = 0; w < nw; ++w) th.emplace_back(worker);
  for (auto& t : th) t.join();
  for (int i : order)
    if (b->jobs[i].status != TTG_OK) {
      c->last_error = "batch chain " + std::to_string(i) + ": " + b->jobs[i].msg;
      return b->jobs[i].status;
    }
  return TTG_OK;
}

// lambda (B), ry (d+1), ncore = number of core elements, stats; status of the
// chain (TTG_OK, 1 = not run, < 0 = its error)
extern "C" int ttg_batch_result(const ttg_batch* b, ttg_int i, double* lambda, ttg_int* ry,
                                ttg_int* ncore, ttg_int* matvecs, double* seconds, int* status) {
  if (!b || i < 0 || i >= (ttg_int)b->jobs.size()) return TTG_ERR_ARG;
  const auto& j = b->jobs[i];
  if (status) *status = j.status;
  if (j.status != TTG_OK) return TTG_OK;
  if (lambda) for (int k = 0; k < j.B; ++k) lambda[k] = j.out.lambda[k];
  if (ry) for (int k = 0; k <= j.d; ++k) ry[k] = j.out.ry[k];
  if (ncore) *ncore = (ttg_int)j.out.cores.size();
  if (matvecs) *matvecs = j.out.matvecs;
  if (seconds) *seconds = j.seconds;
  return TTG_OK;
}

extern "C" int ttg_batch_cores(const ttg_batch* b, ttg_int i, double* out, ttg_int nelem) {
  if (!b || !out || i < 0 || i >= (ttg_int)b->jobs.size()) return TTG_ERR_ARG;
  const auto& j = b->jobs[i];
  if (j.status != TTG_OK || nelem != (ttg_int)j.out.cores.size()) return TTG_ERR_ARG;
  std::copy(j.out.cores.begin(), j.out.cores.end(), out);
  return TTG_OK;
}

// ---------------------------------------------------------------------------
// The local eigensolve of tt_eigb on its own: the call tt_eigb.f90:252-283
// makes to PRIMME (dprimme with initSize = B, the current block as start,
// maxMatvecs and eps as given), on device operands.  It lets a caller (or a
// test) run the library's local solver against the reference's PRIMME on
// the same local problem.
// ---------------------------------------------------------------------------
extern "C" int ttg_local_eig(ttg_ctx* ctx, ttg_int r1, ttg_int n, ttg_int r2, ttg_int ra1,
                             ttg_int ra2, const double* phi1, const double* A,
                             const double* phi2, double* X, ttg_int B, double tol,
                             ttg_int max_matvecs, int method, double* lambda, double* res,
                             ttg_int* matvecs) {
  if (!ctx) return TTG_ERR_ARG;
  try {
    TTG_CUDA(cudaSetDevice(ctx->device));
    TTG_REQUIRE(r1 > 0 && n > 0 && r2 > 0 && ra1 > 0 && ra2 > 0, "all sizes must be positive");
    TTG_REQUIRE(phi1 && A && phi2 && X && lambda, "null argument");
    TTG_REQUIRE(B >= 1 && B <= 16, "B must be in [1, 16]");
    TTG_REQUIRE(method == TTG_METHOD_PLAIN || method == TTG_METHOD_SPLIT ||
                    method == TTG_METHOD_JD64,
                "unknown method");
    const i64 N = r1 * n * r2;
    TTG_REQUIRE(N < (1ll << 31), "local problem too large");
    TTG_REQUIRE(N >= B, "local problem smaller than the block size");
    cudaStream_t s = ctx->stream;
    LocalDims L{r1, n, r2, r1, n, r2, ra1, ra2};
    const int maxb = (int)std::min<i64>(std::max<i64>(4 * B, 32), N);
    const bool jd = method != TTG_METHOD_PLAIN;
    const size_t split_bytes = method == TTG_METHOD_SPLIT ? split_matvec_bytes(L, (int)B) : 0;
    size_t total = al(bfun3_f64_scratch(L, (int)B)) + al(Davidson::bytes(N, (int)B, maxb)) +
                   al(sizeof(double) * N * B) + al(split_bytes) + (1 << 16);
    if (jd) total += al(chosen_bytes(N, (int)B));
    DevBlock mem;
    mem.alloc(total);
    double* bfs = (double*)mem.take<char>(bfun3_f64_scratch(L, (int)B));
    void* dav_mem = mem.take<char>(Davidson::bytes(N, (int)B, maxb));
    double* X0 = mem.take<double>(N * B);
    void* split_mem = split_bytes ? (void*)mem.take<char>(split_bytes) : nullptr;
    void* jd_mem = jd ? (void*)mem.take<char>(chosen_bytes(N, (int)B)) : nullptr;
    PinnedBuf hb(4096);
    TTG_CUDA(cudaMemcpyAsync(X0, X, sizeof(double) * N * B, cudaMemcpyDeviceToDevice, s));
    MatvecFn mv = [=](const double* x, double* y, int nv) {
      bfun3_f64(L, phi1, A, phi2, x, y, nv, bfs, s);
    };
    const int maxmv = max_matvecs > 0 ? (int)std::min<ttg_int>(max_matvecs, 1 << 30) : 500;
    std::vector<double> lam(B, 0.0);
    DavidsonStats st;
    if (jd) {
      MatvecFn mvlow = mv;
      if (method == TTG_METHOD_SPLIT)
        split_matvec_factory(L, phi1, A, phi2, (int)B, split_mem, split_bytes, s, &mvlow);
      int n64 = 0;
      st = chosen_solve(N, (int)B, dav_mem, hb.p, jd_mem, mv, mvlow, X0, tol, maxmv, X,
                        lam.data(), s, nullptr, &n64);
      if (method == TTG_METHOD_SPLIT) split_matvec_check(s);
    } else {
      const int keep = std::min((int)B + std::max(1, (int)B / 2), std::max(maxb - (int)B, 1));
      Davidson dav(N, (int)B, maxb, keep, dav_mem, hb.p, s);
      st = dav.solve(mv, X0, tol, maxmv, X, lam.data());
    }
    TTG_CUDA(cudaStreamSynchronize(s));
    for (int j = 0; j < B; ++j) lambda[j] = lam[j];
    if (res) *res = st.res;
    if (matvecs) *matvecs = st.matvecs;
    ctx->stat_capped = st.converged ? 0 : 1;
    if (!st.converged && ctx->strict)
      throw Error{TTG_ERR_NOCONV, "ttg_local_eig: reached the matvec cap before its tolerance"};
  } catch (const ttg::Error& e) {
    ctx->last_error = e.msg;
    return e.code;
  } catch (const std::exception& e) {
    ctx->last_error = e.what();
    return TTG_ERR_ARG;
  }
  return TTG_OK;
}
