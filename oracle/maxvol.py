"""maxvol row selection restated (oracle).

Test infrastructure only (see ``oracle/__init__.py``).  Follows ``maxvol0_d``
(maxvol.f90:27-119), the start-from-scratch path of ``maxvol_d``
(maxvol.f90:197-288) with a tall ``a`` (m >= n):

  * z = a; LU with partial pivoting of the m x n matrix (dgetrf)      :47-49
  * b = inverse of the leading n x n block of the pivoted matrix,
    taken from its LU factors without further pivoting (dgetri with
    the identity pivot vector)                                         :52-54
  * p = the rows the interchanges move to the top                     :56-60
  * z = a b, so z[p, :] = I                                            :61
  * up to 1024 times: per column the first row of largest |z| (idamax),
    the first column of the largest of those (maxloc); stop when it is
    below 1 + tol or already the selected row; else replace p(j) by i
    and update z by the rank-1 formula, forcing row i to e_j           :66-90

Indices are 0-based here (the reference's are 1-based).
"""
import numpy as np
import scipy.linalg as sla

TOL_DEF = 1e-2
MAXITER = 1 << 10


def maxvol(a, tol=TOL_DEF, maxiter=MAXITER):
    """Returns (p, z, iters) for a tall m x n matrix a (m >= n)."""
    a = np.asarray(a, dtype=np.float64)
    m, n = a.shape
    if m < n:
        raise ValueError("maxvol: wide matrices are not permitted")
    lu, piv = sla.lu_factor(a.copy(order="F"), check_finite=False)   # dgetrf(m, n)
    L = np.tril(lu[:n, :n], -1) + np.eye(n)
    U = np.triu(lu[:n, :n])
    b = np.linalg.inv(L @ U)           # dgetri with identity pivots: inverse of L U
    per = np.arange(m)
    for i in range(n):                 # per(i) <-> per(p(i))
        ip = per[i]
        per[i] = per[piv[i]]
        per[piv[i]] = ip
    p = per[:n].copy()
    z = a @ b
    it = 0
    for it in range(1, maxiter + 1):
        q = np.argmax(np.abs(z), axis=0)           # idamax: first maximum
        v = np.abs(z[q, np.arange(n)])
        j = int(np.argmax(v))                       # maxloc: first maximum
        i = int(q[j])
        amax = abs(z[i, j])
        if amax < 1.0 + tol or p[j] == i:
            break
        ip = p[j]
        p[j] = i
        u = z[:, j].copy()
        vv = z[ip, :] - z[i, :]
        zinv = 1.0 / z[i, j]
        z += np.outer(u, zinv * vv)
        z[i, :] = 0.0
        z[i, j] = 1.0
    return p, z, it


def maxvol_contract(a, p, z, tol=TOL_DEF):
    """max |z| <= 1 + tol, z[p, :] = I and z = a inv(a[p, :])."""
    n = a.shape[1]
    ok_bound = np.max(np.abs(z)) <= 1.0 + tol + 1e-12
    ok_id = np.allclose(z[p, :], np.eye(n), atol=1e-12)
    ok_z = np.allclose(z, a @ np.linalg.inv(a[p, :]), rtol=1e-8, atol=1e-8)
    return ok_bound and ok_id and ok_z
