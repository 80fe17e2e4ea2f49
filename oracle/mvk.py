"""``tt_mvk4`` of tt_adapt_als.f90 restated (oracle): the AMEn matvec.

Test infrastructure only (see ``oracle/__init__.py``).  Approximates
y = A x in the TT format by alternating projections (tt_adapt_als.f90:67-500):

  * eps2 = eps / sqrt(d); the start y (crY0, ranks ry) is orthogonalised
    left to right by QR, building the interfaces phi = Y'AX of shape
    (ry, rx, ra) with dphi_left                                        :190-223
  * sweeps start at the right end going left; at core i the projected core
    is curcr = dbfun3(phi_i, A_i, phi_{i+1}, x_i) and
    err = |cr_i - curcr| / |curcr|                                    :241-262
  * going right (i < d): with kickrank > 0 an SVD of curcr (ry1 n x ry2)
    truncated by my_chop3(eps2), the singular values folded into V^T; the
    right-going kick is switched off in the reference (commented out), so
    none is added; with kickrank <= 0 a QR.  The factor R goes into core
    i+1, then dphi_left                                               :269-345
  * going left (i > 1): with kickrank > 0 an SVD of curcr (ry1 x n ry2)
    truncated by my_chop3(eps2), the kick: min(kickrank, n ry2) vectors of
    the incremental Cholesky (duchol_fort 'N') of dbfun3_right(A_i, phi_{i+1},
    x_i), appended to V, QR, R folded; with kickrank <= 0 a QR of the
    transpose.  R^T goes into core i-1, then dphi_right                :351-434
  * at the two ends the projected core is stored; at the right end a sweep
    is counted and the loop stops when the sweep's err_max < eps         :437-473

The reference's rmax only sizes its work arrays (ranks above it overflow
them); here the kept ranks are capped at rmax.
"""
import numpy as np

from .ops import F, flat, dtransp, bfun3, phi_left, phi_right, dqr, my_chop3
from .als import bfun3_right, uchol


def tt_mvk4(d, n, m, rx, ra, crA, crX, crY0, ry, eps, rmax, kickrank=5, nswp=20):
    """Returns dict(cores, ry, sweeps, err_max)."""
    n = [int(v) for v in n]
    m = [int(v) for v in m]
    rx = [int(v) for v in rx]
    ra = [int(v) for v in ra]
    ry = [int(v) for v in ry]
    eps2 = eps / np.sqrt(d)
    pa = np.concatenate([[0], np.cumsum([ra[k] * n[k] * m[k] * ra[k + 1] for k in range(d)])])
    px = np.concatenate([[0], np.cumsum([rx[k] * m[k] * rx[k + 1] for k in range(d)])])
    A = [np.asarray(crA[pa[k]:pa[k + 1]]) for k in range(d)]
    X = [np.asarray(crX[px[k]:px[k + 1]]) for k in range(d)]
    cr = []
    off = 0
    for k in range(d):
        sz = ry[k] * n[k] * ry[k + 1]
        cr.append(np.array(crY0[off:off + sz], dtype=np.float64))
        off += sz
    phi = [np.ones(1) for _ in range(d + 1)]

    def bf(i):
        return bfun3(rx[i], m[i], rx[i + 1], ry[i], n[i], ry[i + 1], ra[i], ra[i + 1],
                     phi[i], A[i], phi[i + 1], X[i])

    def upd_left(i):
        phi[i + 1] = phi_left(rx[i], m[i], rx[i + 1], ry[i], n[i], ry[i + 1], ra[i], ra[i + 1],
                              phi[i], A[i], X[i], cr[i])

    def upd_right(i):
        phi[i] = phi_right(rx[i], m[i], rx[i + 1], ry[i], n[i], ry[i + 1], ra[i], ra[i + 1],
                           phi[i + 1], A[i], X[i], cr[i])

    for i in range(d - 1):
        rnew = min(ry[i] * n[i], ry[i + 1])
        q, R = dqr(ry[i] * n[i], ry[i + 1], cr[i])
        cr[i] = q
        cr[i + 1] = flat(F(R, rnew, ry[i + 1]) @ F(cr[i + 1], ry[i + 1], n[i + 1] * ry[i + 2]))
        ry[i + 1] = rnew
        upd_left(i)

    err_max = 0.0
    i = d - 1
    direction = -1
    swp = 1
    while swp <= nswp:
        curcr = bf(i)
        err = np.linalg.norm(cr[i] - curcr) / np.linalg.norm(curcr)
        err_max = max(err_max, err)
        if direction > 0 and i < d - 1:
            m_ = ry[i] * n[i]
            rnew = min(ry[i + 1], m_)
            if kickrank > 0:
                U, s, Vt = np.linalg.svd(F(curcr, m_, ry[i + 1]), full_matrices=False)
                nn = min(my_chop3(s, eps2), rmax)
                Um = U[:, :nn]
                Rm = s[:nn, None] * Vt[:nn, :]
                rnew = nn
            else:
                q, Rq = dqr(m_, ry[i + 1], curcr)
                Um = F(q, m_, rnew)
                Rm = F(Rq, rnew, ry[i + 1])
            cr[i] = flat(Um)
            cr[i + 1] = flat(Rm @ F(cr[i + 1], ry[i + 1], n[i + 1] * ry[i + 2]))
            ry[i + 1] = rnew
            upd_left(i)
        if direction < 0 and i > 0:
            m_ = n[i] * ry[i + 1]
            rnew = min(m_, ry[i])
            if kickrank > 0:
                U, s, Vt = np.linalg.svd(F(curcr, ry[i], m_), full_matrices=False)
                nn = min(my_chop3(s, eps2), rmax)
                Cm = Vt[:nn, :].T                                     # m_ x nn
                Rm = s[:nn, None] * U[:, :nn].T                       # nn x ry1
                full = bfun3_right(rx[i], m[i], rx[i + 1], ry[i], n[i], ry[i + 1], ra[i],
                                   ra[i + 1], A[i], phi[i + 1], X[i])
                du, mm = uchol("N", rx[i] * ra[i], m_, full, min(kickrank, m_))
                Cm = np.hstack([Cm, du[:, :mm]])
                Rm = np.vstack([Rm, np.zeros((mm, ry[i]))])
                rnew = min(m_, nn + mm)
                q, Rq = dqr(m_, nn + mm, flat(Cm))
                Cm = F(q, m_, rnew)
                Rm = F(Rq, rnew, nn + mm) @ Rm
            else:
                q, Rq = dqr(m_, ry[i], dtransp(ry[i], m_, curcr))
                Cm = F(q, m_, rnew)
                Rm = F(Rq, rnew, ry[i])
            cr[i] = flat(Cm.T)
            cr[i - 1] = flat(F(cr[i - 1], ry[i - 1] * n[i - 1], ry[i]) @ Rm.T)
            ry[i] = rnew
            upd_right(i)
        if direction > 0 and i == d - 1:
            cr[i] = curcr
            direction = -1
            i += 1
            swp += 1
            if err_max < eps:
                break
            err_max = 0.0
        if direction < 0 and i == 0:
            cr[i] = curcr
            direction = 1
            i -= 1
        i += direction
    cores = np.concatenate([cr[k][:ry[k] * n[k] * ry[k + 1]] for k in range(d)])
    return {"cores": cores, "ry": ry, "sweeps": min(swp, nswp), "err_max": err_max}
