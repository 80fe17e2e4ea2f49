"""Dense local operators of the ALS sweep, restated from the reference.

Test infrastructure only (see ``oracle/__init__.py``).  Each function keeps
the reference's GEMM/transpose order so that rounding behaves alike.

Layouts (column-major, as in the reference):
  x     (rx1, m, rx2)         b1, j, b2
  y     (ry1, n, ry2)         c1, i, c2
  A     (ra1, n, m, ra2)      a1, i, j, a2
  phi1  (ry1, rx1, ra1)       c1, b1, a1
  phi2  (rx2, ra2, ry2)       b2, a2, c2
"""
import numpy as np
import scipy.linalg as sla


def F(a, *shape):
    """View a flat column-major buffer with the given Fortran shape."""
    return np.reshape(a, shape, order="F")


def flat(a):
    return np.ravel(a, order="F")


def dtransp(n, m, a):
    """``dtransp`` matrix_util.f90:152-170: (n x m) -> (m x n), flat."""
    return flat(F(a[: n * m], n, m).T)


def compute_ps(d, r, n):
    """``compute_ps`` matrix_util.f90:242-251, 0-based offsets (ps[0] = 0)."""
    ps = np.zeros(d + 1, dtype=np.int64)
    for i in range(d):
        ps[i + 1] = ps[i] + r[i] * n[i] * r[i + 1]
    return ps


def my_chop3(s, eps):
    """``my_chop3`` matrix_util.f90:254-275 (relative Frobenius truncation).

    Returns the rank kept: the smallest i such that the tail sum of squares
    s(i+1..n) stays below (eps*||s||)^2, plus one, capped at n.
    """
    n = len(s)
    nrm = np.linalg.norm(s)
    nrm = (nrm * eps) * (nrm * eps)
    cursum = 0.0
    i = n
    while i > 0:
        cursum += s[i - 1] * s[i - 1]
        if cursum > nrm:
            break
        i -= 1
    return min(i + 1, n)


def dqr(n, m, a):
    """``dqr`` matrix_util.f90:37-61: Householder QR (dgeqrf + dorgqr).

    Returns (Q, R) with Q the first min(n, m) columns (n x rnew, flat) and R
    (rnew x m, flat, upper triangular), LAPACK sign convention.
    """
    A = F(a[: n * m], n, m)
    q, r = sla.qr(A, mode="economic")
    return flat(q), flat(r)


def zqr(n, m, a):
    """``zqr`` matrix_util.f90:64-90 (zgeqrf + zungqr)."""
    return dqr(n, m, a)


def bfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, x):
    """``dbfun3`` ttals.f90:9-32 / ``zbfun3`` :34-57: y = Phi1 * A * Phi2 * x."""
    res1 = F(x, rx1 * m, rx2) @ F(phi2, rx2, ra2 * ry2)          # b1,j,a2,c2
    res1 = dtransp(rx1, m * ra2 * ry2, flat(res1))                  # j,a2,c2,b1
    res2 = F(A, ra1 * n, m * ra2) @ F(res1, m * ra2, ry2 * rx1)   # a1,i,c2,b1
    res2 = dtransp(ra1 * n * ry2, rx1, flat(res2))                  # b1,a1,i,c2
    y = F(phi1, ry1, rx1 * ra1) @ F(res2, rx1 * ra1, n * ry2)     # c1,i,c2
    return flat(y)


def bfun3_block(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, X, nvec):
    """``primme_matvec`` tt_eigb.f90:15-27: bfun3 applied to nvec vectors."""
    sx = rx1 * m * rx2
    return np.concatenate([bfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2,
                                 X[k * sx:(k + 1) * sx]) for k in range(nvec)])


def zbfun3_transp(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, x):
    """``zbfun3_transp`` ttals.f90:85-108 (x has the y layout ry1,n,ry2).

    Computes conj(B^H-ish product) exactly as the reference writes it:
    res1 = x^H phi1, transposes, times A, times phi2^T, then conjugates.
    """
    res1 = F(x, ry1, n * ry2).conj().T @ F(phi1, ry1, rx1 * ra1)  # n*ry2 x rx1*ra1
    res1 = dtransp(n, ry2 * rx1 * ra1, flat(res1))                 # ry2,rx1,ra1,n
    res2 = F(res1, ry2 * rx1, ra1 * n) @ F(A, ra1 * n, m * ra2)    # ry2,rx1,m,ra2
    res2 = dtransp(ry2, rx1 * m * ra2, flat(res2))                 # rx1,m,ra2,ry2
    y = F(res2, rx1 * m, ra2 * ry2) @ F(phi2, rx2, ra2 * ry2).T   # rx1*m x rx2
    return flat(y).conj()


def phi_right(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi2_old, A, x, y, conj=False):
    """``dphi_right`` ttals.f90:150-173 / ``zphi_right`` :176-200.

    Output phi2 (rx1, ra1, ry1) = sum x(b1,j,b2) phi2(b2,a2,c2) A(a1,i,j,a2) y(c1,i,c2).
    ``conj`` conjugates y (the complex version).
    """
    yy = np.conj(y) if conj else y
    res1 = F(x, rx1 * m, rx2) @ F(phi2_old, rx2, ra2 * ry2)        # b1,j,a2,c2
    res1 = dtransp(rx1, m * ra2 * ry2, flat(res1))                  # j,a2,c2,b1
    res2 = F(A, ra1 * n, m * ra2) @ F(res1, m * ra2, ry2 * rx1)   # a1,i,c2,b1
    res2 = dtransp(ra1, n * ry2 * rx1, flat(res2))                  # i,c2,b1,a1
    phi = F(yy, ry1, n * ry2) @ F(res2, n * ry2, rx1 * ra1)        # c1,b1,a1
    return dtransp(ry1, rx1 * ra1, flat(phi))                       # b1,a1,c1


def phi_left(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1_old, A, x, y, conj=False):
    """``dphi_left`` ttals.f90:203-227 / ``zphi_left`` :229-256.

    Output phi1 (ry2, rx2, ra2) = sum phi1(c1,b1,a1) y(c1,i,c2) A(a1,i,j,a2) x(b1,j,b2).
    """
    yy = np.conj(y) if conj else y
    res1 = F(phi1_old, ry1, rx1 * ra1).T @ F(yy, ry1, n * ry2)     # b1,a1,i,c2
    res1 = dtransp(rx1, ra1 * n * ry2, flat(res1))                  # a1,i,c2,b1
    res2 = F(res1, ra1 * n, ry2 * rx1).T @ F(A, ra1 * n, m * ra2)  # c2,b1,j,a2
    res2 = dtransp(ry2, rx1 * m * ra2, flat(res2))                  # b1,j,a2,c2
    phi = F(res2, rx1 * m, ra2 * ry2).T @ F(x, rx1 * m, rx2)       # a2,c2,b2
    return dtransp(ra2, ry2 * rx2, flat(phi))                       # c2,b2,a2


def phi2_left(rx1, rx2, ry1, n, ry2, phi1_old, x, y):
    """``dphi2_left`` ttals.f90:296-314: phi1 (ry2, rx2) = y' x projection."""
    res1 = F(phi1_old, ry1, rx1).T @ F(y, ry1, n * ry2)            # b1,i,c2
    return flat(F(res1, rx1 * n, ry2).T @ F(x, rx1 * n, rx2))


def phi2_right(rx1, rx2, ry1, n, ry2, phi2_old, x, y):
    """``dphi2_right`` ttals.f90:260-277: phi2 (rx1, ry1)."""
    res1 = F(x, rx1 * n, rx2) @ F(phi2_old, rx2, ry2)              # b1,j,c2
    return flat(F(res1, rx1, n * ry2) @ F(y, ry1, n * ry2).T)


def fullmat(rx1, m, rx2, ra1, ra2, phi1, A, phi2):
    """``d2d_fullmat`` tt_eigb.f90:88-105: dense local matrix.

    Returns B (N x N) with N = rx1*m*rx2, rows (c1,i,c2), columns (b1,j,b2).
    """
    P1 = F(phi1, rx1, rx1, ra1)
    Ac = F(A, ra1, m, m, ra2)
    P2 = F(phi2, rx2, ra2, rx2)
    Bm = np.einsum("cba,aijd,edf->cifbje", P1, Ac, P2, optimize=True)
    N = rx1 * m * rx2
    return Bm.reshape(N, N, order="F")
