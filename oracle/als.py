"""``tt_amen_solve`` of tt_adapt_als.f90 restated (oracle).

Test infrastructure only (see ``oracle/__init__.py``).  This is the flat-array
AMEn of tt_adapt_als.f90:513-1132, a different algorithm from ``dtt_amen_solve``
(ttamen.f90, ``oracle/amen.py``):

  * eps2 = eps / sqrt(d); left-to-right QR of x with the interfaces
    phiA = X'AX and phiy = X'Y                                     :591-644
  * alternating half sweeps, starting at the right end going left; a sweep
    is counted at the right end                                      :648-1111
  * local step: rhs from phiy, residual r = A x - rhs, and when
    tau = eps2 / (2 |r|/|rhs|) < 1 a Householder GMRES(nrestart) x niters
    correction (dgmresr_hh_fort, tt_linalg.f90:651-845) with tolerance
    tau, x -= dx                                                     :655-797
  * truncation: SVD, then the residual-based rank scan from the top
    (the kept rank is one more than the first rank, counting down, whose
    residual exceeds both 2 res_new and eps2), then the kick: kickrank
    vectors of an incremental Cholesky (duchol_fort, tt_linalg.f90:540-642)
    of [Y-projection, A-projection] appended to the kept block, QR, and
    the R factor pushed into the neighbour                           :807-1018
  * when a whole half sweep ends with res_max < eps the kick is switched
    off (kickrank = -1) and the next end of a half sweep stops       :1066-1105

Preconditioners: 'n' (none, the default) and the block-Jacobi 'c', 'l', 'r'
of djac_gen / djac_apply (``oracle/jac.py``), regenerated for every local
system that GMRES solves (:746-769); GMRES is right-preconditioned, i.e. it
solves (A P) z = r and the correction is P z (tt_linalg.f90:689-690,733-735;
tt_adapt_als.f90:776-781).

One detail is kept as the reference has it: ``dbfun3_left``
(tt_linalg.f90:242-253) transposes Phi1 into a work array but multiplies
with Phi1 itself, reading its (ry1, rx1, ra1) memory as an (ra1*ry1) x rx1
matrix; the left kick uses that product.
"""
import numpy as np
import scipy.linalg as sla

from .ops import F, flat, dtransp, bfun3, phi_left, phi_right, phi2_left, phi2_right, dqr
from .amen import gmres_hh
from .jac import jac_gen, jac_apply


def bfun3_left(rx1, m, rx2, ry1, n, ra1, ra2, phi1, A, x):
    """dbfun3_left as written (see the module docstring): (ry1 n) x (rx2 ra2)."""
    res2 = F(phi1, ra1 * ry1, rx1) @ F(x, rx1, m * rx2)              # (a1,c1),(j,b2)
    res1 = F(res2, ra1, ry1, m, rx2).transpose(0, 2, 1, 3)           # a1,j,c1,b2
    Ap = F(A, ra1, n, m, ra2).transpose(0, 2, 1, 3)                  # a1,j,i,a2
    y = F(flat(res1), ra1 * m, ry1 * rx2).T @ F(flat(Ap), ra1 * m, n * ra2)   # (c1,b2),(i,a2)
    y = F(flat(y), ry1, rx2, n, ra2).transpose(0, 2, 1, 3)           # c1,i,b2,a2
    return flat(y)


def bfun3_right(rx1, m, rx2, ry1, n, ry2, ra1, ra2, A, phi2, x):
    """dbfun3_right tt_linalg.f90:210-240: (rx1 ra1) x (n ry2)."""
    res1 = F(x, rx1 * m, rx2) @ F(phi2, rx2, ra2 * ry2)              # b1,j,a2,c2
    res1 = dtransp(rx1, m * ra2 * ry2, flat(res1))                   # j,a2,c2,b1
    res2 = F(A, ra1 * n, m * ra2) @ F(res1, m * ra2, ry2 * rx1)      # a1,i,c2,b1
    return dtransp(ra1 * n * ry2, rx1, flat(res2))                    # b1,a1,i,c2


def uchol(trans, m, n, dA, numvec):
    """duchol_fort (tt_linalg.f90:540-642).  trans 'T': dA is n x m; 'N': m x n.
    Returns (du (n x real_numvec), real_numvec)."""
    A = F(dA, n, m) if trans == "T" else F(dA, m, n).T               # n x m either way
    du = np.zeros((n, numvec))
    lam = np.zeros(numvec)
    ddiag = np.sum(A * A, axis=1)
    cnt = 0
    broke = False
    while cnt < numvec:
        maxi = int(np.argmax(np.abs(ddiag)))                          # idamax
        du[:, cnt] = A @ A[maxi, :]
        for j in range(cnt):
            du[:, cnt] -= lam[j] * du[maxi, j] * du[:, j]
        maxa = np.sqrt(abs(du[maxi, cnt]))
        if maxa < 1e-300:
            broke = True
            break
        du[:, cnt] /= maxa
        ddiag = ddiag - du[:, cnt] ** 2
        k = cnt + 1
        q, r = sla.qr(du[:, :k], mode="economic")
        dx = r[:, k - 1].copy()
        du[:, :k] = q
        dv = np.outer(dx, dx) + np.diag(lam[:k])
        w, v = np.linalg.eigh(dv)
        lam[:k] = w
        du[:, :k] = du[:, :k] @ v
        cnt += 1
    # the Fortran loop index: the failing step when the loop exits early
    real = cnt + 1 if broke else numvec
    return du[:, :real], real


def tt_amen_solve(d, n, m, ry, ra, crA, crY, crX0, rx, eps, kickrank=4, nswp=20, nrestart=40,
                  niters=2, prec="n"):
    """Restatement of tt_amen_solve (tt_adapt_als.f90:513).  Returns a dict
    with ``cores`` (result_core layout), ``rx``, ``sweeps``, ``res_max`` (of
    the last finished half sweep) and ``matvecs``."""
    n = [int(v) for v in n]
    ry = [int(v) for v in ry]
    ra = [int(v) for v in ra]
    rx = [int(v) for v in rx]
    eps2 = eps / np.sqrt(d)
    pa = np.concatenate([[0], np.cumsum([ra[k] * n[k] * n[k] * ra[k + 1] for k in range(d)])])
    py = np.concatenate([[0], np.cumsum([ry[k] * n[k] * ry[k + 1] for k in range(d)])])
    A = [np.asarray(crA[pa[k]:pa[k + 1]]) for k in range(d)]
    Y = [np.asarray(crY[py[k]:py[k + 1]]) for k in range(d)]
    cr = []
    off = 0
    for k in range(d):
        sz = rx[k] * n[k] * rx[k + 1]
        cr.append(np.array(crX0[off:off + sz], dtype=np.float64))
        off += sz
    phiA = [np.ones(1) for _ in range(d + 1)]
    phiy = [np.ones(1) for _ in range(d + 1)]

    def mvk(i, x):
        return bfun3(rx[i], n[i], rx[i + 1], rx[i], n[i], rx[i + 1], ra[i], ra[i + 1],
                     phiA[i], A[i], phiA[i + 1], x)

    def upd_left(i):
        phiA[i + 1] = phi_left(rx[i], n[i], rx[i + 1], rx[i], n[i], rx[i + 1], ra[i], ra[i + 1],
                               phiA[i], A[i], cr[i], cr[i])
        phiy[i + 1] = phi2_left(ry[i], ry[i + 1], rx[i], n[i], rx[i + 1], phiy[i], Y[i], cr[i])

    def upd_right(i):
        phiA[i] = phi_right(rx[i], n[i], rx[i + 1], rx[i], n[i], rx[i + 1], ra[i], ra[i + 1],
                            phiA[i + 1], A[i], cr[i], cr[i])
        phiy[i] = phi2_right(ry[i], ry[i + 1], rx[i], n[i], rx[i + 1], phiy[i + 1], Y[i], cr[i])

    # initial QR, left to right
    for i in range(d - 1):
        rnew = min(rx[i] * n[i], rx[i + 1])
        q, R = dqr(rx[i] * n[i], rx[i + 1], cr[i])
        cr[i] = q
        cr[i + 1] = flat(F(R, rnew, rx[i + 1]) @ F(cr[i + 1], rx[i + 1], n[i + 1] * rx[i + 2]))
        rx[i + 1] = rnew
        upd_left(i)

    err_max = 0.0
    res_max = 0.0
    last_res = 0.0
    i = d - 1
    direction = -1
    swp = 1
    kick = kickrank
    nmv = 0
    while swp <= nswp:
        if direction < 0:
            work = F(Y[i], ry[i] * n[i], ry[i + 1]) @ F(phiy[i + 1], ry[i + 1], rx[i + 1])
            kick_y = F(flat(work), ry[i], n[i] * rx[i + 1])
            rhs = flat(F(phiy[i], rx[i], ry[i]) @ kick_y)
        else:
            work = F(phiy[i], rx[i], ry[i]) @ F(Y[i], ry[i], n[i] * ry[i + 1])
            kick_y = F(flat(work), rx[i] * n[i], ry[i + 1])
            rhs = flat(kick_y @ F(phiy[i + 1], ry[i + 1], rx[i + 1]))
        nn = rx[i] * n[i] * rx[i + 1]
        r0 = mvk(i, cr[i]) - rhs
        nmv += 1
        norm_rhs = np.linalg.norm(rhs)
        err = np.linalg.norm(r0) / norm_rhs
        res_max = max(res_max, err)
        tau = eps2 / (err * 2.0)
        if tau < 1.0:
            if prec.lower() in ("c", "l", "r"):
                jacs = jac_gen(prec, rx[i], n[i], rx[i + 1], ra[i], ra[i + 1], phiA[i], A[i],
                               phiA[i + 1])
                pj = lambda v: jac_apply(prec, rx[i], n[i], rx[i + 1], jacs, v)  # noqa: E731
                z, k_mv, _ = gmres_hh(lambda v: mvk(i, pj(v)), r0, min(nrestart, nn), tau, niters)
                dx = pj(z)
            else:
                dx, k_mv, _ = gmres_hh(lambda v: mvk(i, v), r0, min(nrestart, nn), tau, niters)
            nmv += k_mv
            cr[i] = cr[i] - dx
            res_new = np.linalg.norm(mvk(i, cr[i]) - rhs) / norm_rhs
            nmv += 1
            err = np.linalg.norm(dx) / np.linalg.norm(cr[i])
            err_max = max(err_max, err)
        else:
            res_new = err
        curcr = cr[i].copy()
        if direction > 0 and i < d - 1:
            m_ = rx[i] * n[i]
            rnew = min(rx[i + 1], m_)
            if kick > 0 or kick == -1:
                U, s, Vt = np.linalg.svd(F(curcr, m_, rx[i + 1]), full_matrices=False)
                Rm = s[:, None] * Vt                                      # rnew x rx2
                kept = 0
                for cand in range(rnew - 1, 0, -1):
                    w = flat(U[:, :cand] @ Rm[:cand, :])
                    e = np.linalg.norm(mvk(i, w) - rhs) / norm_rhs
                    nmv += 1
                    if e > res_new * 2.0 and e > eps2:
                        kept = cand
                        break
                nn_k = kept + 1
                Um = U[:, :nn_k]
                Rm = Rm[:nn_k, :]
                rnew = nn_k
                if kick > 0:
                    tA = bfun3_left(rx[i], n[i], rx[i + 1], rx[i], n[i], ra[i], ra[i + 1],
                                    phiA[i], A[i], cr[i])
                    kb = np.hstack([kick_y, F(tA, m_, rx[i + 1] * ra[i + 1])])
                    du, mm = uchol("T", rx[i + 1] * ra[i + 1] + ry[i + 1], m_, flat(kb),
                                   min(kick, m_))
                    Um = np.hstack([Um, du[:, :mm]])
                    Rm = np.vstack([Rm, np.zeros((mm, rx[i + 1]))])
                    rnew = min(m_, nn_k + mm)
                    q, Rq = dqr(m_, nn_k + mm, flat(Um))
                    Um = F(q, m_, rnew)
                    Rm = F(Rq, rnew, nn_k + mm) @ Rm
            else:
                q, Rq = dqr(m_, rx[i + 1], curcr)
                Um = F(q, m_, rnew)
                Rm = F(Rq, rnew, rx[i + 1])
            cr[i] = flat(Um)
            cr[i + 1] = flat(Rm @ F(cr[i + 1], rx[i + 1], n[i + 1] * rx[i + 2]))
            rx[i + 1] = rnew
            upd_left(i)
        if direction < 0 and i > 0:
            m_ = n[i] * rx[i + 1]
            rnew = min(m_, rx[i])
            if kick > 0 or kick == -1:
                U, s, Vt = np.linalg.svd(F(curcr, rx[i], m_), full_matrices=False)
                Lm = U * s[None, :]                                       # rx1 x rnew
                kept = 0
                for cand in range(rnew - 1, 0, -1):
                    w = flat(Lm[:, :cand] @ Vt[:cand, :])
                    e = np.linalg.norm(mvk(i, w) - rhs) / norm_rhs
                    nmv += 1
                    if e > res_new * 2.0 and e > eps2:
                        kept = cand
                        break
                nn_k = kept + 1
                Cm = Vt[:nn_k, :].T                                       # m_ x nn
                Rm = Lm[:, :nn_k].T                                       # nn x rx1
                rnew = nn_k
                if kick > 0:
                    tA = bfun3_right(rx[i], n[i], rx[i + 1], rx[i], n[i], rx[i + 1], ra[i],
                                     ra[i + 1], A[i], phiA[i + 1], cr[i])
                    kb = np.vstack([F(flat(kick_y), ry[i], m_), F(tA, rx[i] * ra[i], m_)])
                    du, mm = uchol("N", rx[i] * ra[i] + ry[i], m_, flat(kb), min(kick, m_))
                    Cm = np.hstack([Cm, du[:, :mm]])
                    Rm = np.vstack([Rm, np.zeros((mm, rx[i]))])
                    rnew = min(m_, nn_k + mm)
                    q, Rq = dqr(m_, nn_k + mm, flat(Cm))
                    Cm = F(q, m_, rnew)
                    Rm = F(Rq, rnew, nn_k + mm) @ Rm
            else:
                q, Rq = dqr(m_, rx[i], flat(F(curcr, rx[i], m_).T))
                Cm = F(q, m_, rnew)
                Rm = F(Rq, rnew, rx[i])
            cr[i] = flat(Cm.T)
            cr[i - 1] = flat(F(cr[i - 1], rx[i - 1] * n[i - 1], rx[i]) @ Rm.T)
            rx[i] = rnew
            upd_right(i)
        if (direction > 0 and i == d - 1) or (direction < 0 and i == 0):
            last_res = res_max
        if direction > 0 and i == d - 1:
            direction = -1
            i += 1
            if kick < 0:
                break
            if res_max < eps:
                kick = -1
            swp += 1
            err_max = 0.0
            res_max = 0.0
        if direction < 0 and i == 0:
            if kick < 0:
                break
            if res_max < eps:
                kick = -1
            direction = 1
            i -= 1
            err_max = 0.0
            res_max = 0.0
        i += direction
    cores = np.concatenate([cr[k][:rx[k] * n[k] * rx[k + 1]] for k in range(d)])
    return {"cores": cores, "rx": rx, "sweeps": min(swp, nswp), "res_max": last_res,
            "matvecs": nmv}
