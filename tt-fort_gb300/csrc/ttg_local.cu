// Plain (FP64 / complex128) local operator and interface updates.
//
//   bfun3      y = Phi1 * A * Phi2 * x            ttals.f90:9-32   (dbfun3)
//   phi_left   Phi1' = sum Phi1 y A x             ttals.f90:203-227 (dphi_left)
//   phi_right  Phi2' = sum x Phi2 A y             ttals.f90:150-173 (dphi_right)
//   phi2_*     Y'X projections without A          ttals.f90:260-314
//   fullmat    dense local matrix                 tt_eigb.f90:88-105 (d2d_fullmat)
//   z*         complex versions, y conjugated     ttals.f90:34-57,85-108,176-256
//
// Each product is three GEMMs.  The reference transposes its intermediates
// between the GEMMs (dtransp, ttals.f90:22,26); here the intermediates are
// laid out so that every GEMM reads and writes them with unit stride:
//   T1[b1, j, a2, c2]   = x * Phi2              (rx1*m  x ra2*ry2)
//   T2[b1, a1, i, c2]   = A (x) T1, one GEMM per c2
//   y [c1, i, c2]       = Phi1 * T2             (ry1 x n*ry2)
// so the transposes cost nothing.  All GEMMs go through gemm_f64 / gemm_z.
#include "ttg_common.cuh"

namespace ttg {

size_t bfun3_f64_scratch(const LocalDims& L, int nvec) {
  return (size_t)(L.t1size() + L.t2size()) * nvec * sizeof(double);
}

size_t phi_f64_scratch(const LocalDims& L) {
  i64 a = std::max(L.t1size(), L.rx1 * L.ra1 * L.n * L.ry2);
  i64 b = std::max(L.t2size(), L.rx1 * L.m * L.ra2 * L.ry2);
  return (size_t)(a + b) * sizeof(double) * 2;   // room for complex too
}

template <class G, class T>
static void stage1(G& g, const LocalDims& L, const T* x, const T* phi2, T* T1, int nvec) {
  // T1 (rx1*m x ra2*ry2) = x (rx1*m x rx2) * phi2 (rx2 x ra2*ry2)
  g.M = (int)(L.rx1 * L.m); g.N = (int)(L.ra2 * L.ry2); g.K = (int)L.rx2;
  g.A = x;    g.sAm = 1; g.sAk = L.rx1 * L.m;
  g.B = phi2; g.sBk = 1; g.sBn = L.rx2;
  g.C = T1;   g.sCm = 1; g.sCn = L.rx1 * L.m;
  g.nb1 = 1; g.nb2 = nvec;
  g.bA2 = L.xsize(); g.bB2 = 0; g.bC2 = L.t1size();
}

template <class G, class T>
static void stage2(G& g, const LocalDims& L, const T* A, const T* T1, T* T2, int nvec) {
  // per (c2, vec): T2[b1,(a1,i)] = sum_(j,a2) A[(a1,i),(j,a2)] T1[b1,(j,a2)]
  g.M = (int)(L.ra1 * L.n); g.N = (int)L.rx1; g.K = (int)(L.m * L.ra2);
  g.A = A;  g.sAm = 1; g.sAk = L.ra1 * L.n;
  g.B = T1; g.sBk = L.rx1; g.sBn = 1;
  g.C = T2; g.sCm = L.rx1; g.sCn = 1;
  g.nb1 = (int)L.ry2; g.nb2 = nvec;
  g.bA1 = 0; g.bA2 = 0;
  g.bB1 = L.rx1 * L.m * L.ra2; g.bB2 = L.t1size();
  g.bC1 = L.rx1 * L.ra1 * L.n; g.bC2 = L.t2size();
}

template <class G, class T>
static void stage3(G& g, const LocalDims& L, const T* phi1, const T* T2, T* y, int nvec) {
  // y (ry1 x n*ry2) = phi1 (ry1 x rx1*ra1) * T2 (rx1*ra1 x n*ry2)
  g.M = (int)L.ry1; g.N = (int)(L.n * L.ry2); g.K = (int)(L.rx1 * L.ra1);
  g.A = phi1; g.sAm = 1; g.sAk = L.ry1;
  g.B = T2;   g.sBk = 1; g.sBn = L.rx1 * L.ra1;
  g.C = y;    g.sCm = 1; g.sCn = L.ry1;
  g.nb1 = 1; g.nb2 = nvec;
  g.bA2 = 0; g.bB2 = L.t2size(); g.bC2 = L.ysize();
}

void bfun3_f64(const LocalDims& L, const double* phi1, const double* A, const double* phi2,
               const double* x, double* y, int nvec, double* scratch, cudaStream_t s) {
  double* T1 = scratch;
  double* T2 = scratch + L.t1size() * nvec;
  { GemmF64 g; stage1(g, L, x, phi2, T1, nvec); gemm_f64(g, s); }
  { GemmF64 g; stage2(g, L, A, T1, T2, nvec); gemm_f64(g, s); }
  { GemmF64 g; stage3(g, L, phi1, T2, y, nvec); gemm_f64(g, s); }
}

void bfun3_z(const LocalDims& L, const double2* phi1, const double2* A, const double2* phi2,
             const double2* x, double2* y, int nvec, double2* scratch, cudaStream_t s) {
  double2* T1 = scratch;
  double2* T2 = scratch + L.t1size() * nvec;
  { GemmZ g; stage1(g, L, x, phi2, T1, nvec); gemm_z(g, s); }
  { GemmZ g; stage2(g, L, A, T1, T2, nvec); gemm_z(g, s); }
  { GemmZ g; stage3(g, L, phi1, T2, y, nvec); gemm_z(g, s); }
}

// Adjoint product (zbfun3_transp, ttals.f90:85-108): x has the y layout
// (ry1, n, ry2), output y has the x layout (rx1, m, rx2); y = B^H x.
void bfun3_transp_z(const LocalDims& L, const double2* phi1, const double2* A,
                    const double2* phi2, const double2* x, double2* y, int nvec,
                    double2* scratch, cudaStream_t s) {
  const i64 p1 = L.rx1 * L.ra1 * L.n * L.ry2;     // R1[b1,a1,i,c2]
  const i64 p2 = L.rx1 * L.m * L.ra2 * L.ry2;     // R2[b1,j,a2,c2]
  double2* R1 = scratch;
  double2* R2 = scratch + p1 * nvec;
  {
    GemmZ g;   // R1[(b1,a1),(i,c2)] = sum_c1 conj(phi1[c1,(b1,a1)]) x[c1,(i,c2)]
    g.M = (int)(L.rx1 * L.ra1); g.N = (int)(L.n * L.ry2); g.K = (int)L.ry1;
    g.A = phi1; g.sAm = L.ry1; g.sAk = 1; g.conjA = true;
    g.B = x; g.sBk = 1; g.sBn = L.ry1;
    g.C = R1; g.sCm = 1; g.sCn = L.rx1 * L.ra1;
    g.nb2 = nvec; g.bB2 = L.ysize(); g.bC2 = p1;
    gemm_z(g, s);
  }
  {
    GemmZ g;   // per (c2, vec): R2[b1,(j,a2)] = sum_p conj(A[p,(j,a2)]) R1[b1,p]
    g.M = (int)(L.m * L.ra2); g.N = (int)L.rx1; g.K = (int)(L.ra1 * L.n);
    g.A = A; g.sAm = L.ra1 * L.n; g.sAk = 1; g.conjA = true;
    g.B = R1; g.sBk = L.rx1; g.sBn = 1;
    g.C = R2; g.sCm = L.rx1; g.sCn = 1;
    g.nb1 = (int)L.ry2; g.nb2 = nvec;
    g.bB1 = L.rx1 * L.ra1 * L.n; g.bB2 = p1;
    g.bC1 = L.rx1 * L.m * L.ra2; g.bC2 = p2;
    gemm_z(g, s);
  }
  {
    GemmZ g;   // y[(b1,j), b2] = sum_(a2,c2) R2[(b1,j),(a2,c2)] conj(phi2[b2,(a2,c2)])
    g.M = (int)(L.rx1 * L.m); g.N = (int)L.rx2; g.K = (int)(L.ra2 * L.ry2);
    g.A = R2; g.sAm = 1; g.sAk = L.rx1 * L.m;
    g.B = phi2; g.sBk = L.rx2; g.sBn = 1; g.conjB = true;
    g.C = y; g.sCm = 1; g.sCn = L.rx1 * L.m;
    g.nb2 = nvec; g.bA2 = p2; g.bC2 = L.xsize();
    gemm_z(g, s);
  }
}

template <class G, class T>
static void phi_right_impl(const LocalDims& L, const T* phi2_old, const T* A, const T* x,
                           const T* y, T* phi2_new, T* scratch, bool conj_y, cudaStream_t s,
                           void (*gemm)(const G&, cudaStream_t)) {
  T* T1 = scratch;
  T* T2 = scratch + L.t1size();
  { G g; stage1(g, L, x, phi2_old, T1, 1); gemm(g, s); }
  { G g; stage2(g, L, A, T1, T2, 1); gemm(g, s); }
  {
    // phi2_new (rx1*ra1 x ry1) = T2 (rx1*ra1 x n*ry2) * y^T (n*ry2 x ry1)
    G g;
    g.M = (int)(L.rx1 * L.ra1); g.N = (int)L.ry1; g.K = (int)(L.n * L.ry2);
    g.A = T2; g.sAm = 1; g.sAk = L.rx1 * L.ra1;
    g.B = y; g.sBk = L.ry1; g.sBn = 1;
    g.C = phi2_new; g.sCm = 1; g.sCn = L.rx1 * L.ra1;
    if constexpr (sizeof(T) == 16) g.conjB = conj_y;
    gemm(g, s);
  }
}

template <class G, class T>
static void phi_left_impl(const LocalDims& L, const T* phi1_old, const T* A, const T* x,
                          const T* y, T* phi1_new, T* scratch, bool conj_y, cudaStream_t s,
                          void (*gemm)(const G&, cudaStream_t)) {
  const i64 psz = L.rx1 * L.ra1 * L.n * L.ry2;   // P[b1,a1,i,c2]
  T* P = scratch;
  T* Q = scratch + psz;                           // Q[b1,j,a2,c2]
  {
    G g;   // P[(b1,a1),(i,c2)] = sum_c1 phi1_old[c1,(b1,a1)] y[c1,(i,c2)]
    g.M = (int)(L.rx1 * L.ra1); g.N = (int)(L.n * L.ry2); g.K = (int)L.ry1;
    g.A = phi1_old; g.sAm = L.ry1; g.sAk = 1;
    g.B = y; g.sBk = 1; g.sBn = L.ry1;
    g.C = P; g.sCm = 1; g.sCn = L.rx1 * L.ra1;
    if constexpr (sizeof(T) == 16) g.conjB = conj_y;
    gemm(g, s);
  }
  {
    G g;   // per c2: Q[b1,(j,a2)] = sum_(a1,i) A[(a1,i),(j,a2)] P[b1,(a1,i)]
    g.M = (int)(L.m * L.ra2); g.N = (int)L.rx1; g.K = (int)(L.ra1 * L.n);
    g.A = A; g.sAm = L.ra1 * L.n; g.sAk = 1;
    g.B = P; g.sBk = L.rx1; g.sBn = 1;
    g.C = Q; g.sCm = L.rx1; g.sCn = 1;
    g.nb1 = (int)L.ry2; g.bB1 = L.rx1 * L.ra1 * L.n; g.bC1 = L.rx1 * L.m * L.ra2;
    gemm(g, s);
  }
  {
    G g;   // per a2: phi1_new[c2, b2] = sum_(b1,j) Q[(b1,j), a2, c2] x[(b1,j), b2]
    g.M = (int)L.ry2; g.N = (int)L.rx2; g.K = (int)(L.rx1 * L.m);
    g.A = Q; g.sAm = L.rx1 * L.m * L.ra2; g.sAk = 1;
    g.B = x; g.sBk = 1; g.sBn = L.rx1 * L.m;
    g.C = phi1_new; g.sCm = 1; g.sCn = L.ry2;
    g.nb1 = (int)L.ra2; g.bA1 = L.rx1 * L.m; g.bC1 = L.ry2 * L.rx2;
    gemm(g, s);
  }
}

void phi_right_f64(const LocalDims& L, const double* phi2_old, const double* A,
                   const double* x, const double* y, double* phi2_new, double* scratch,
                   cudaStream_t s) {
  phi_right_impl<GemmF64, double>(L, phi2_old, A, x, y, phi2_new, scratch, false, s, gemm_f64);
}
void phi_left_f64(const LocalDims& L, const double* phi1_old, const double* A,
                  const double* x, const double* y, double* phi1_new, double* scratch,
                  cudaStream_t s) {
  phi_left_impl<GemmF64, double>(L, phi1_old, A, x, y, phi1_new, scratch, false, s, gemm_f64);
}
void phi_right_z(const LocalDims& L, const double2* phi2_old, const double2* A,
                 const double2* x, const double2* y, double2* phi2_new, double2* scratch,
                 cudaStream_t s) {
  phi_right_impl<GemmZ, double2>(L, phi2_old, A, x, y, phi2_new, scratch, true, s, gemm_z);
}
void phi_left_z(const LocalDims& L, const double2* phi1_old, const double2* A,
                const double2* x, const double2* y, double2* phi1_new, double2* scratch,
                cudaStream_t s) {
  phi_left_impl<GemmZ, double2>(L, phi1_old, A, x, y, phi1_new, scratch, true, s, gemm_z);
}

void phi2_left_f64(i64 rx1, i64 rx2, i64 ry1, i64 n, i64 ry2, const double* phi1_old,
                   const double* x, const double* y, double* phi1_new, double* scratch,
                   cudaStream_t s) {
  // res1 (rx1 x n*ry2) = phi1_old^T (rx1 x ry1) * y (ry1 x n*ry2)    ttals.f90:309
  {
    GemmF64 g;
    g.M = (int)rx1; g.N = (int)(n * ry2); g.K = (int)ry1;
    g.A = phi1_old; g.sAm = ry1; g.sAk = 1;
    g.B = y; g.sBk = 1; g.sBn = ry1;
    g.C = scratch; g.sCm = 1; g.sCn = rx1;
    gemm_f64(g, s);
  }
  // phi1 (ry2 x rx2) = res1^T ((rx1 n) x ry2)^T * x (rx1 n x rx2)    ttals.f90:311
  {
    GemmF64 g;
    g.M = (int)ry2; g.N = (int)rx2; g.K = (int)(rx1 * n);
    g.A = scratch; g.sAm = rx1 * n; g.sAk = 1;
    g.B = x; g.sBk = 1; g.sBn = rx1 * n;
    g.C = phi1_new; g.sCm = 1; g.sCn = ry2;
    gemm_f64(g, s);
  }
}

void phi2_right_f64(i64 rx1, i64 rx2, i64 ry1, i64 n, i64 ry2, const double* phi2_old,
                    const double* x, const double* y, double* phi2_new, double* scratch,
                    cudaStream_t s) {
  // res1 (rx1 n x ry2) = x (rx1 n x rx2) * phi2_old (rx2 x ry2)       ttals.f90:273
  {
    GemmF64 g;
    g.M = (int)(rx1 * n); g.N = (int)ry2; g.K = (int)rx2;
    g.A = x; g.sAm = 1; g.sAk = rx1 * n;
    g.B = phi2_old; g.sBk = 1; g.sBn = rx2;
    g.C = scratch; g.sCm = 1; g.sCn = rx1 * n;
    gemm_f64(g, s);
  }
  // phi2 (rx1 x ry1) = res1 (rx1 x n ry2) * y^T (n ry2 x ry1)          ttals.f90:275
  {
    GemmF64 g;
    g.M = (int)rx1; g.N = (int)ry1; g.K = (int)(n * ry2);
    g.A = scratch; g.sAm = 1; g.sAk = rx1;
    g.B = y; g.sBk = ry1; g.sBn = 1;
    g.C = phi2_new; g.sCm = 1; g.sCn = rx1;
    gemm_f64(g, s);
  }
}

// B[(c1,i,c2),(b1,j,b2)] = sum_{a1,a2} phi1[c1,b1,a1] A[a1,i,j,a2] phi2[b2,a2,c2]
__global__ void fullmat_kernel(i64 rx1, i64 m, i64 rx2, i64 ra1, i64 ra2,
                               const double* __restrict__ phi1, const double* __restrict__ A,
                               const double* __restrict__ phi2, double* __restrict__ Bm) {
  const i64 N = rx1 * m * rx2;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < N * N;
       e += (i64)gridDim.x * blockDim.x) {
    i64 row = e % N, col = e / N;
    i64 c1 = row % rx1, i = (row / rx1) % m, c2 = row / (rx1 * m);
    i64 b1 = col % rx1, j = (col / rx1) % m, b2 = col / (rx1 * m);
    double acc = 0.0;
    for (i64 a2 = 0; a2 < ra2; ++a2) {
      double p2 = phi2[b2 + rx2 * (a2 + ra2 * c2)];
      if (p2 == 0.0) continue;
      double t = 0.0;
      for (i64 a1 = 0; a1 < ra1; ++a1)
        t += phi1[c1 + rx1 * (b1 + rx1 * a1)] * A[a1 + ra1 * (i + m * (j + m * a2))];
      acc += t * p2;
    }
    Bm[e] = acc;
  }
}

void fullmat_f64(i64 rx1, i64 m, i64 rx2, i64 ra1, i64 ra2, const double* phi1,
                 const double* A, const double* phi2, double* Bmat, cudaStream_t s) {
  i64 N = rx1 * m * rx2;
  int blocks = (int)std::min<i64>(4096, (N * N + 255) / 256);
  fullmat_kernel<<<blocks, 256, 0, s>>>(rx1, m, rx2, ra1, ra2, phi1, A, phi2, Bmat);
  TTG_CHECK_LAUNCH();
}

}  // namespace ttg
