"""AMEn linear solver ``dtt_amen_solve`` restated (oracle).

Test infrastructure only (see ``oracle/__init__.py``).  Follows ttamen.f90:29-252:

  * defaults kickrank 4, nswp 20, local_iters 2, local_restart 40,
    trunc_norm 1 (residual), max_full_size 50                    ttamen.f90:52-59
  * real_tol = tol / sqrt(d-1) / resid_damp (2)                 ttamen.f90:64-65
  * right-to-left QR of x (and of the enrichment z) with the
    projections X'AX, X'Y, Z'AX, Z'Y                            ttamen.f90:84-108
  * left-to-right: local residual, local solve (dense dgesv below
    max_full_size, Householder GMRES otherwise), residual-based
    truncation (dtt_trunc, ttnodeop.f90:227-302), enrichment of the core
    with the projected residual and update of z                  ttamen.f90:112-227
  * stop when the largest local residual is below tol           ttamen.f90:239-243
with ``dtt_qr`` (ttnodeop.f90:18-78, ``ort0`` ort.f90:17-82), ``dtt_enrich``
(:143-182), ``dtt_YAX`` (:385-448) and ``d2d_gmresr`` (ttlocsolve.f90:509-682).
The enrichment TT z starts from N(0,1) cores drawn from the splitmix64 /
Box-Muller stream ``sm_normals`` (the reference draws them from the
clock-seeded Fortran generator); the CUDA library uses the same stream.
"""
import numpy as np
import scipy.linalg as sla

from .ops import F, flat, dtransp, bfun3, phi_left, phi_right, phi2_left, phi2_right, fullmat

RESID_DAMP = 2.0


def sm_normals(seed, count):
    """Standard normals from splitmix64 uniforms in (0, 1] (Box-Muller)."""
    i = np.arange(count, dtype=np.uint64)
    base = np.uint64(seed) * np.uint64(1000003)

    def uni(k):
        with np.errstate(over="ignore"):
            z = k * np.uint64(0x9E3779B97F4A7C15)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        return ((z >> np.uint64(11)).astype(np.float64) + 1.0) * 2.0 ** -53

    with np.errstate(over="ignore"):
        u1 = uni(base + np.uint64(2) * i + np.uint64(1))
        u2 = uni(base + np.uint64(2) * i + np.uint64(2))
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


class TT:
    def __init__(self, n, r, cores):
        self.n = list(n)
        self.r = list(r)
        self.c = [np.array(c, dtype=np.float64) for c in cores]

    @staticmethod
    def from_flat(n, r, flatcores):
        cores, off = [], 0
        for k in range(len(n)):
            sz = r[k] * n[k] * r[k + 1]
            cores.append(np.array(flatcores[off:off + sz], dtype=np.float64))
            off += sz
        return TT(n, r, cores)

    def flat(self):
        return np.concatenate([self.c[k][:self.r[k] * self.n[k] * self.r[k + 1]]
                               for k in range(len(self.n))])


def ort0(U):
    """ort0_d (ort.f90:17-82): Q, R of a tall matrix; a wide one keeps itself
    as R and an identity block as Q."""
    m, n = U.shape
    if m < n:
        R = np.zeros((n, n))
        R[:m, :] = U
        Q = np.zeros((m, n))
        Q[:, :m] = np.eye(m)
        return Q, R
    q, r = sla.qr(U, mode="economic")
    return q, r


def tt_qr(x, k, dir_):
    """dtt_qr (ttnodeop.f90:18-78) on core k (0-based)."""
    n, r = x.n, x.r
    if dir_ > 0:
        m, rr, p = r[k] * n[k], r[k + 1], n[k + 1] * r[k + 2]
        U = F(x.c[k], m, rr)
        Q, R = ort0(U)
        rnew = min(rr, m)
        nnod = F(x.c[k + 1], rr, p)
        x.c[k] = flat(Q[:, :rnew])
        x.c[k + 1] = flat(R[:rnew, :] @ nnod)
        r[k + 1] = rnew
    else:
        m, rr, p = n[k] * r[k + 1], r[k], r[k - 1] * n[k - 1]
        U = F(dtransp(rr, m, x.c[k]), m, rr)
        Q, R = ort0(U)
        rnew = min(rr, m)
        nnod = F(x.c[k - 1], p, rr)
        x.c[k] = dtransp(m, rnew, flat(Q[:, :rnew]))
        x.c[k - 1] = flat(nnod @ R[:rnew, :].T)
        r[k] = rnew


def tt_enrich(x, k, rho, left):
    """dtt_enrich (ttnodeop.f90:143-182) with a left block of rho columns."""
    n, r = x.n, x.r
    knod = F(x.c[k], r[k] * n[k], r[k + 1])
    nnod = F(x.c[k + 1], r[k + 1], n[k + 1] * r[k + 2])
    x.c[k] = flat(np.hstack([knod, F(left, r[k] * n[k], rho)]))
    x.c[k + 1] = flat(np.vstack([nnod, np.zeros((rho, n[k + 1] * r[k + 2]))]))
    r[k + 1] += rho


def yax(phi_old, y, x, k, dir_, A=None, ra=None):
    """dtt_YAX (ttnodeop.f90:385-448): projections Y'AX (with A) or Y'X."""
    if A is not None:
        args = (x.r[k], x.n[k], x.r[k + 1], y.r[k], y.n[k], y.r[k + 1], ra[k], ra[k + 1])
        if dir_ > 0:
            return phi_left(*args, phi_old, A, x.c[k], y.c[k])
        return phi_right(*args, phi_old, A, x.c[k], y.c[k])
    if dir_ > 0:
        return phi2_left(x.r[k], x.r[k + 1], y.r[k], x.n[k], y.r[k + 1], phi_old, x.c[k], y.c[k])
    return phi2_right(x.r[k], x.r[k + 1], y.r[k], x.n[k], y.r[k + 1], phi_old, x.c[k], y.c[k])


def gmres_hh(mv, rhs, nrestart, tol, niters):
    """d2d_gmresr (ttlocsolve.f90:509-682), no preconditioner: Householder
    GMRES(nrestart) for mv(sol) = rhs, niters restarts, relative tol."""
    sz = len(rhs)
    nr = min(sz, nrestart)
    sol = np.zeros(sz)
    U = np.zeros((sz, nr + 1))
    R = np.zeros((nr + 1, nr + 1))
    JJ = np.zeros((2, nr + 1))
    tau = np.zeros(nr + 1)
    nrmrhs = None
    curres = 1.0
    total = 0
    for it in range(niters):
        w = mv(sol) - rhs
        total += 1
        nrmr = np.linalg.norm(w)
        if it == 0:
            nrmrhs = nrmr
        if nrmr == 0.0:
            break
        dbeta = nrmr
        if w[0] < 0:
            dbeta = -dbeta
        w[0] += dbeta
        tau[0] = -dbeta
        w = w / np.linalg.norm(w)
        U[:, 0] = w
        j_last = 0
        for j in range(nr):            # 1-based j+1
            j_last = j
            w = -2.0 * U[j, j] * U[:, j]
            w[j] += 1.0
            for i in range(j - 1, -1, -1):
                w = w - 2.0 * (U[:, i] @ w) * U[:, i]
            w = w / np.linalg.norm(w)
            w = mv(w)
            total += 1
            for i in range(j + 1):
                w = w - 2.0 * (U[:, i] @ w) * U[:, i]
            if j + 1 < sz:
                U[:j + 1, j + 1] = 0.0
                tail = w[j + 1:].copy()
                dalpha = np.linalg.norm(tail)
                if dalpha != 0.0:
                    if w[j + 1] < 0:
                        dalpha = -dalpha
                    tail[0] += dalpha
                    U[j + 1:, j + 1] = tail / np.linalg.norm(tail)
                    w[j + 1] = -dalpha
                    w[j + 2:] = 0.0
                else:
                    U[j + 1:, j + 1] = tail
            for i in range(j):
                d0 = w[i]
                w[i] = JJ[0, i] * w[i] + JJ[1, i] * w[i + 1]
                w[i + 1] = -JJ[1, i] * d0 + JJ[0, i] * w[i + 1]
            if j + 1 < sz:
                dalpha = np.hypot(w[j], w[j + 1])
                JJ[0, j] = w[j] / dalpha
                JJ[1, j] = w[j + 1] / dalpha
                tau[j + 1] = -JJ[1, j] * tau[j]
                tau[j] = JJ[0, j] * tau[j]
                w[j] = dalpha
                w[j + 1] = 0.0
            R[:j + 1, j] = w[:j + 1]
            curres = abs(tau[j + 1]) / nrmrhs
            if curres < tol:
                break
        jj = j_last + 1
        y = sla.solve_triangular(R[:jj, :jj], tau[:jj], lower=False)
        w = -2.0 * U[jj - 1, jj - 1] * y[jj - 1] * U[:, jj - 1]
        w[jj - 1] += y[jj - 1]
        for i in range(jj - 2, -1, -1):
            w[i] += y[i]
            w = w - 2.0 * (U[:, i] @ w) * U[:, i]
        sol = sol - w
        if curres < tol:
            break
    return sol, total, curres


def tt_amen_solve(d, n, ra, crA, ry, crY, rx, crX0, tol, kickrank=4, nswp=20, local_iters=2,
                  local_restart=40, trunc_norm=1, max_full_size=50, seed=0, verb=0):
    """Restatement of dtt_amen_solve; returns dict(cores, rx, sweeps, res_max)."""
    n = list(map(int, n)); ra = list(map(int, ra))
    off = np.zeros(d + 1, dtype=np.int64)
    for k in range(d):
        off[k + 1] = off[k] + ra[k] * n[k] * n[k] * ra[k + 1]
    Ac = [np.asarray(crA[off[k]:off[k + 1]], dtype=np.float64) for k in range(d)]
    x = TT.from_flat(n, list(map(int, rx)), crX0)
    y = TT.from_flat(n, list(map(int, ry)), crY)
    real_tol = tol / np.sqrt(d - 1) / RESID_DAMP
    one = np.ones(1)
    pxax = [None] * (d + 1); pxy = [None] * (d + 1)
    pxax[0] = pxax[d] = one; pxy[0] = pxy[d] = one
    kick = kickrank
    if kick > 0:
        zr = [1] + [kick] * (d - 1) + [1]
        z = TT.from_flat(n, zr, sm_normals(seed, sum(zr[k] * n[k] * zr[k + 1] for k in range(d))))
        pzax = [None] * (d + 1); pzy = [None] * (d + 1)
        pzax[0] = pzax[d] = one; pzy[0] = pzy[d] = one
    nmv = 0
    swp_done = 0
    res_max = 0.0
    for swp in range(1, nswp + 1):
        swp_done = swp
        for k in range(d - 1, 0, -1):
            if kick > 0 and swp > 1:
                zk = bfun3(x.r[k], n[k], x.r[k + 1], z.r[k], n[k], z.r[k + 1], ra[k], ra[k + 1],
                           pzax[k], Ac[k], pzax[k + 1], x.c[k])
                t = F(pzy[k], z.r[k], y.r[k]) @ F(y.c[k], y.r[k], n[k] * y.r[k + 1])
                rhs = F(flat(t), z.r[k] * n[k], y.r[k + 1]) @ F(pzy[k + 1], y.r[k + 1], z.r[k + 1])
                z.c[k] = zk - flat(rhs)
            tt_qr(x, k, -1)
            pxax[k] = yax(pxax[k + 1], x, x, k, -1, Ac[k], ra)
            pxy[k] = yax(pxy[k + 1], x, y, k, -1)
            if kick > 0:
                tt_qr(z, k, -1)
                pzax[k] = yax(pzax[k + 1], z, x, k, -1, Ac[k], ra)
                pzy[k] = yax(pzy[k + 1], z, y, k, -1)
        res_max = 0.0
        err_max = 0.0
        for k in range(d):
            rx1, rx2 = x.r[k], x.r[k + 1]
            N = rx1 * n[k] * rx2
            t = F(pxy[k], rx1, y.r[k]) @ F(y.c[k], y.r[k], n[k] * y.r[k + 1])
            rhs = flat(F(flat(t), rx1 * n[k], y.r[k + 1]) @ F(pxy[k + 1], y.r[k + 1], rx2))
            mv = lambda v: bfun3(rx1, n[k], rx2, rx1, n[k], rx2, ra[k], ra[k + 1], pxax[k], Ac[k],
                                 pxax[k + 1], v)
            resid = mv(x.c[k]) - rhs
            nmv += 1
            err = np.linalg.norm(resid) / np.linalg.norm(rhs)
            res_max = max(res_max, err)
            if err > real_tol:
                if N < max_full_size:
                    Bm = fullmat(rx1, n[k], rx2, ra[k], ra[k + 1], pxax[k], Ac[k], pxax[k + 1])
                    sol = np.linalg.solve(Bm, resid)
                else:
                    sol, cnt, _ = gmres_hh(mv, resid, local_restart, real_tol / err, local_iters)
                    nmv += cnt
                x.c[k] = x.c[k] - sol
                err_max = max(err_max, np.linalg.norm(sol) / np.linalg.norm(x.c[k]))
                resid = mv(x.c[k]) - rhs
                nmv += 1
                err = np.linalg.norm(resid) / np.linalg.norm(rhs)
            if k < d - 1:
                if kick > 0:
                    if trunc_norm == 1:
                        err = max(err, real_tol * RESID_DAMP)
                        xnew, c = trunc_resid(x, k, err, Ac, ra, pxax, rhs)
                        nmv += c
                    else:
                        xnew = trunc_chop(x, k, real_tol * RESID_DAMP)
                    sol = bfun3(rx1, n[k], rx2, rx1, n[k], z.r[k + 1], ra[k], ra[k + 1], pxax[k],
                                Ac[k], pzax[k + 1], xnew)
                    zk = bfun3(rx1, n[k], rx2, z.r[k], n[k], z.r[k + 1], ra[k], ra[k + 1], pzax[k],
                               Ac[k], pzax[k + 1], xnew)
                    t = F(pxy[k], rx1, y.r[k]) @ F(y.c[k], y.r[k], n[k] * y.r[k + 1])
                    sol = sol - flat(F(flat(t), rx1 * n[k], y.r[k + 1]) @ F(pzy[k + 1], y.r[k + 1], z.r[k + 1]))
                    t = F(pzy[k], z.r[k], y.r[k]) @ F(y.c[k], y.r[k], n[k] * y.r[k + 1])
                    z.c[k] = zk - flat(F(flat(t), z.r[k] * n[k], y.r[k + 1]) @ F(pzy[k + 1], y.r[k + 1], z.r[k + 1]))
                    tt_enrich(x, k, z.r[k + 1], sol)
                    tt_qr(x, k, +1)
                    tt_qr(z, k, +1)
                    pzax[k + 1] = yax(pzax[k], z, x, k, +1, Ac[k], ra)
                    pzy[k + 1] = yax(pzy[k], z, y, k, +1)
                else:
                    tt_qr(x, k, +1)
                pxax[k + 1] = yax(pxax[k], x, x, k, +1, Ac[k], ra)
                pxy[k + 1] = yax(pxy[k], x, y, k, +1)
        if verb:
            print(f"amen swp {swp} max_dx {err_max:.3e} max_res {res_max:.3e} max_rank {max(x.r)}")
        if trunc_norm == 1 and res_max < tol:
            break
        if trunc_norm != 1 and err_max < tol:
            break
    return {"cores": x.flat(), "rx": list(x.r), "sweeps": swp_done, "res_max": res_max,
            "matvecs": nmv}


def _svd(knod):
    u, s, vt = sla.svd(knod, full_matrices=False, lapack_driver="gesvd")
    return u, s, vt.T


def trunc_resid(x, k, tol, Ac, ra, pxax, rhs):
    """dtt_trunc dir=+1 with the residual criterion (ttnodeop.f90:227-302)."""
    n, r = x.n, x.r
    m, rr, p = r[k] * n[k], r[k + 1], n[k + 1] * r[k + 2]
    knod = F(x.c[k], m, rr)
    u, s, v = _svd(knod)
    rmin = min(rr, m)
    v = v * s
    norm_rhs = np.linalg.norm(rhs)
    rnew = rmin - 1
    cnt = 0
    while rnew >= 1:
        core = flat(u[:, :rnew] @ v[:, :rnew].T)
        res = bfun3(r[k], n[k], rr, r[k], n[k], rr, ra[k], ra[k + 1], pxax[k], Ac[k], pxax[k + 1],
                    core) - rhs
        cnt += 1
        if np.linalg.norm(res) / norm_rhs > tol:
            break
        rnew -= 1
    rnew += 1
    nnod = F(x.c[k + 1], rr, p)
    x.c[k] = flat(u[:, :rnew])
    x.c[k + 1] = flat(v[:, :rnew].T @ nnod)
    xnew = flat(u[:, :rnew] @ v[:, :rnew].T)
    r[k + 1] = rnew
    return xnew, cnt


def trunc_chop(x, k, tol):
    """dtt_trunc dir=+1 with the Frobenius criterion (chop, svd.f90:86-111)."""
    n, r = x.n, x.r
    m, rr, p = r[k] * n[k], r[k + 1], n[k + 1] * r[k + 2]
    u, s, v = _svd(F(x.c[k], m, rr))
    v = v * s
    rnew = len(s)
    nrm = np.linalg.norm(s)
    bound = tol * tol * nrm * nrm
    er = s[rnew - 1] ** 2
    while er < bound:
        rnew -= 1
        er += s[rnew - 1] ** 2
    nnod = F(x.c[k + 1], rr, p)
    x.c[k] = flat(u[:, :rnew])
    x.c[k + 1] = flat(v[:, :rnew].T @ nnod)
    xnew = flat(u[:, :rnew] @ v[:, :rnew].T)
    r[k + 1] = rnew
    return xnew
