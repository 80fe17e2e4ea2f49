"""Projector-splitting (KSL) time step ``ztt_ksl`` restated (oracle).

Test infrastructure only (see ``oracle/__init__.py``).  Follows
tt_ksl.f90:431-668:

  * QR left->right of cores 1..d-1 with zphi_left updates   tt_ksl.f90:528-550
  * tau0 = tau/2 for the symmetric scheme (typ = 2)          tt_ksl.f90:557-561
  * backward half sweep i = d..1: K-step exp(+tau0 A_loc) on core i, then
    (i > 1) QR of the transposed core, zphi_right, S-step exp(-tau0 S) of
    the transposed R factor, folded into core i-1            tt_ksl.f90:569-599
  * forward half sweep i = 1..d: K-step, then (i < d) QR, zphi_left, S-step
    folded into core i+1                                     tt_ksl.f90:600-625
  * every exponential through zexp_mv (Krylov order 8, tol 1e-8) with the
    Higham 1-norm estimate as anorm (usenrm = 1)
The S operator (sfun_ksl, tt_ksl.f90:142-152) maps S (rx1 x rx2) to
phi1 (ry1 x rx1*ra) * [S phi2 (rx2 x ra*ry2)]; it is consistent only when the
QR keeps the rank, which is the case for the reference's own inputs.
"""
import numpy as np

from .ops import F, flat, dtransp, compute_ps, bfun3, zbfun3_transp, phi_left, phi_right
from .expokit import zexp_mv
from .normest import znormest, Seed


def zqr_lapack(n, m, a):
    """zqr (matrix_util.f90:64-90): zgeqrf + zungqr, LAPACK reflector signs."""
    import scipy.linalg as sla
    q, r = sla.qr(F(np.asarray(a, dtype=np.complex128)[: n * m], n, m), mode="economic")
    return flat(q), flat(r)


def sfun(rx1, rx2, ra, ry1, ry2, phi1, phi2):
    def mv(Sx):
        res1 = F(Sx, rx1, rx2) @ F(phi2, rx2, ra * ry2)              # rx1, ra, ry2
        return flat(F(phi1, ry1, rx1 * ra) @ F(flat(res1), rx1 * ra, ry2))
    return mv


def _cols(fn):
    def apply(X):
        return np.column_stack([fn(X[:, j]) for j in range(X.shape[1])])
    return apply


def ztt_ksl(d, n, m, ra, crA, crY0, ry, tau, rmax, typ=2, order=8, verb=0):
    """One KSL time step.  Returns dict(cores, ry, stats)."""
    n = list(map(int, n)); m = list(map(int, m)); ra = list(map(int, ra))
    ry = list(map(int, ry))
    crA = np.asarray(crA, dtype=np.complex128)
    eps = 1e-8
    pa = compute_ps(d, ra, [n[i] * m[i] for i in range(d)])
    Acore = [crA[pa[i]:pa[i + 1]] for i in range(d)]
    cr = []
    off = 0
    for i in range(d):
        sz = ry[i] * n[i] * ry[i + 1]
        cr.append(np.array(crY0[off:off + sz], dtype=np.complex128))
        off += sz
    phi = [None] * (d + 1)
    phi[0] = np.ones(1, dtype=np.complex128)
    phi[d] = np.ones(1, dtype=np.complex128)
    for i in range(d - 1):
        rnew = min(ry[i] * n[i], ry[i + 1])
        q, r = zqr_lapack(ry[i] * n[i], ry[i + 1], cr[i])
        cr[i] = q
        cr[i + 1] = flat(F(r, rnew, ry[i + 1]) @ F(cr[i + 1], ry[i + 1], n[i + 1] * ry[i + 2]))
        ry[i + 1] = rnew
        phi[i + 1] = phi_left(ry[i], m[i], ry[i + 1], ry[i], n[i], ry[i + 1], ra[i], ra[i + 1],
                              phi[i], Acore[i], cr[i], cr[i], conj=True)
    seed = Seed()
    tau0 = tau / 2 if typ == 2 else tau
    stats = {"exp_calls": 0, "nmult": 0, "normest": []}

    def kstep(i):
        r1, r2 = ry[i], ry[i + 1]
        N = r1 * n[i] * r2
        args = (r1, n[i], r2, r1, n[i], r2, ra[i], ra[i + 1], phi[i], Acore[i], phi[i + 1])
        mv = lambda x: bfun3(*args, x)
        mvT = lambda x: zbfun3_transp(*args, x)
        anorm = znormest(N, 4, _cols(mv), _cols(mvT), seed)
        w, st = zexp_mv(N, order, tau0, cr[i], eps, anorm, mv)
        stats["exp_calls"] += 1
        stats["nmult"] += st["nmult"]
        stats["normest"].append(anorm)
        return w

    def sstep(rx1, rx2, rr, ry1, ry2, p1, p2, R):
        mv = sfun(rx1, rx2, rr, ry1, ry2, p1, p2)
        N = rx1 * ry2
        anorm = znormest(N, 4, _cols(mv), None, seed)
        w, st = zexp_mv(N, order, -tau0, R, eps, anorm, mv)
        stats["exp_calls"] += 1
        stats["nmult"] += st["nmult"]
        stats["normest"].append(anorm)
        return w

    i, dir_, swp = d - 1, -1, 0
    while swp < 1:
        curcr = kstep(i)
        if dir_ < 0:
            if i > 0:
                ct = dtransp(ry[i], n[i] * ry[i + 1], curcr)          # (n r2) x r1
                rnew = min(n[i] * ry[i + 1], ry[i])
                q, r = zqr_lapack(n[i] * ry[i + 1], ry[i], ct)
                core = dtransp(n[i] * ry[i + 1], rnew, q)             # rnew x (n r2)
                cr[i] = core
                R = dtransp(rnew, ry[i], r)                           # r1 x rnew
                phitmp = phi_right(rnew, n[i], ry[i + 1], rnew, n[i], ry[i + 1], ra[i], ra[i + 1],
                                   phi[i + 1], Acore[i], core, core, conj=True)
                if rnew != ry[i]:
                    raise ValueError("KSL S-step needs a rank-preserving QR")
                Stmp = sstep(ry[i], ry[i], ra[i], rnew, rnew, phi[i], phitmp, R)
                cr[i - 1] = flat(F(cr[i - 1], ry[i - 1] * n[i - 1], ry[i]) @ F(Stmp, ry[i], rnew))
                ry[i] = rnew
                phi[i] = phitmp
            else:
                cr[i] = curcr
        else:
            if i < d - 1:
                q, r = zqr_lapack(ry[i] * n[i], ry[i + 1], curcr)
                rnew = min(ry[i] * n[i], ry[i + 1])
                cr[i] = q
                phitmp = phi_left(ry[i], n[i], rnew, ry[i], n[i], rnew, ra[i], ra[i + 1],
                                  phi[i], Acore[i], q, q, conj=True)
                if rnew != ry[i + 1]:
                    raise ValueError("KSL S-step needs a rank-preserving QR")
                Stmp = sstep(rnew, rnew, ra[i + 1], ry[i + 1], ry[i + 1], phitmp, phi[i + 1], r)
                cr[i + 1] = flat(F(Stmp, rnew, ry[i + 1]) @ F(cr[i + 1], ry[i + 1], n[i + 1] * ry[i + 2]))
                ry[i + 1] = rnew
                phi[i + 1] = phitmp
            else:
                cr[i] = curcr
        if dir_ > 0 and i == d - 1:
            dir_, i = -1, d - 1
            swp += 1
        elif dir_ < 0 and i == 0:
            dir_, i = 1, 0
            if typ == 1:
                break
        else:
            i += dir_
    cores = np.concatenate([cr[k][:ry[k] * n[k] * ry[k + 1]] for k in range(d)])
    return {"cores": cores, "ry": ry, "stats": stats}


def tt_ksl_real(d, n, m, ra, crA, crY0, ry, tau, rmax, order=8, usenrm=1):
    """One step of the real-valued ``tt_ksl`` (tt_ksl.f90:191-428), a
    different scheme from ``ztt_ksl``: always symmetric (tau/2 everywhere),
    and one sweep = a backward half sweep i = d..1 (K-step on core i; for
    i < d the S-step on the bond (i, i+1) from the left QR factor of the new
    core, folded back into core i; for i > 1 the right QR of core i pushed into
    core i-1) followed by a forward half sweep i = 1..d (for i < d the S-step
    of the left QR of core i, then the K-step; for i < d the left QR pushed
    into core i+1).

    Norm estimates as the reference calls them: the K-step passes ``dmatvec``
    as its own transpose (tt_ksl.f90:38-45), and the S-step's
    ``dsfun_matvec_transp`` writes its product into its input, so
    ``normest_higham`` continues with the sign vectors themselves (identity,
    as the complex S-step); the estimator is the one-sided Higham iteration
    of ``oracle/normest.py`` (the reference's real DLACN1 with its own random
    signs gives other estimates; they only move the Krylov step sizes).
    usenrm 2 takes anorm = 1.  The reference's ``dsfun_matvec`` multiplies
    with the undeclared ``ONE`` and ``ZERO`` (tt_ksl.f90:122-130); this
    restatement uses 1 and 0, the values that code means.  Computed in complex
    arithmetic on real data; returns dict(cores (real), ry).  The ranks are
    fixed; they must pass the QR steps unchanged (r_{k+1} <= r_k n_k after
    the left-to-right QR, r_k <= n_k r_{k+1})."""
    n = list(map(int, n)); m = list(map(int, m)); ra = list(map(int, ra))
    ry = list(map(int, ry))
    crA = np.asarray(crA, dtype=np.complex128)
    eps = 1e-8
    pa = compute_ps(d, ra, [n[i] * m[i] for i in range(d)])
    Acore = [crA[pa[i]:pa[i + 1]] for i in range(d)]
    cr = []
    off = 0
    for i in range(d):
        sz = ry[i] * n[i] * ry[i + 1]
        cr.append(np.array(crY0[off:off + sz], dtype=np.complex128))
        off += sz
    phi = [None] * (d + 1)
    phi[0] = np.ones(1, dtype=np.complex128)
    phi[d] = np.ones(1, dtype=np.complex128)
    for i in range(d - 1):
        rnew = min(ry[i] * n[i], ry[i + 1])
        q, r = zqr_lapack(ry[i] * n[i], ry[i + 1], cr[i])
        cr[i] = q
        cr[i + 1] = flat(F(r, rnew, ry[i + 1]) @ F(cr[i + 1], ry[i + 1], n[i + 1] * ry[i + 2]))
        ry[i + 1] = rnew
        phi[i + 1] = phi_left(ry[i], m[i], ry[i + 1], ry[i], n[i], ry[i + 1], ra[i], ra[i + 1],
                              phi[i], Acore[i], cr[i], cr[i], conj=True)
    for i in range(d - 1):
        if ry[i] * n[i] < ry[i + 1] or n[i + 1] * ry[i + 2] < ry[i + 1]:
            raise ValueError("tt_ksl needs ranks its QR steps keep")
    seed = Seed()
    t2 = tau / 2

    def kexp(i, x):
        r1, r2 = ry[i], ry[i + 1]
        N = r1 * n[i] * r2
        mv = lambda v: bfun3(r1, n[i], r2, r1, n[i], r2, ra[i], ra[i + 1], phi[i], Acore[i],  # noqa: E731
                             phi[i + 1], v)
        anorm = 1.0 if usenrm == 2 else znormest(N, 4, _cols(mv), _cols(mv), seed)
        w, _ = zexp_mv(N, order, t2, x, eps, anorm, mv)
        return w

    def sexp(i, ph1, R):
        r = ry[i + 1]
        mv = sfun(r, r, ra[i + 1], r, r, ph1, phi[i + 1])
        anorm = 1.0 if usenrm == 2 else znormest(r * r, 4, _cols(mv), None, seed)
        w, _ = zexp_mv(r * r, order, -t2, R, eps, anorm, mv)
        return w

    def left_s(i, core):
        # QR of core i (ry_i n_i x ry_{i+1}), S-step of R, core i = Q S
        r1, r2 = ry[i], ry[i + 1]
        q, R = zqr_lapack(r1 * n[i], r2, core)
        ph = phi_left(r1, m[i], r2, r1, n[i], r2, ra[i], ra[i + 1], phi[i], Acore[i], q, q,
                      conj=True)
        S = sexp(i, ph, R)
        return flat(F(q, r1 * n[i], r2) @ F(S, r2, r2))

    # backward half sweep; with d = 1 neither branch stores the K-step, so
    # the reference's result is the forward half step alone
    for i in range(d - 1, -1, -1):
        curcr = kexp(i, cr[i])
        if i < d - 1:
            curcr = left_s(i, curcr)
            cr[i] = curcr
        if i > 0:
            r1, r2 = ry[i], ry[i + 1]
            ct = dtransp(r1, n[i] * r2, curcr)                        # (n r2) x r1
            q, R = zqr_lapack(n[i] * r2, r1, ct)
            cr[i] = dtransp(n[i] * r2, r1, q)                         # r1 x (n r2)
            cr[i - 1] = flat(F(cr[i - 1], ry[i - 1] * n[i - 1], r1) @ F(R, r1, r1).T)
            phi[i] = phi_right(r1, m[i], r2, r1, n[i], r2, ra[i], ra[i + 1], phi[i + 1],
                               Acore[i], cr[i], cr[i], conj=True)
    # forward half sweep
    for i in range(d):
        curcr = left_s(i, cr[i]) if i < d - 1 else cr[i]
        cr[i] = kexp(i, curcr)
        if i < d - 1:
            r1, r2 = ry[i], ry[i + 1]
            q, R = zqr_lapack(r1 * n[i], r2, cr[i])
            cr[i] = q
            cr[i + 1] = flat(F(R, r2, r2) @ F(cr[i + 1], r2, n[i + 1] * ry[i + 2]))
            phi[i + 1] = phi_left(r1, m[i], r2, r1, n[i], r2, ra[i], ra[i + 1], phi[i],
                                  Acore[i], cr[i], cr[i], conj=True)
    cores = np.concatenate([cr[k][:ry[k] * n[k] * ry[k + 1]] for k in range(d)])
    return {"cores": cores.real.copy(), "ry": ry}


def _slice(a, r1, n, r2, k):
    return flat(F(a, r1, n, r2)[:, k, :])


def phi_diag_left(ry1, n, ry2, ra1, ra2, phi, A, x):
    """zphi_diag_left (tt_diag_ksl.f90:269-284): sum over the slices k of
    zphi_left with m = n = 1."""
    out = 0
    for k in range(n):
        out = out + phi_left(ry1, 1, ry2, ry1, 1, ry2, ra1, ra2, phi, _slice(A, ra1, n, ra2, k),
                             _slice(x, ry1, n, ry2, k), _slice(x, ry1, n, ry2, k), conj=True)
    return out


def phi_diag_right(ry1, n, ry2, ra1, ra2, phi, A, x):
    """zphi_diag_right (tt_diag_ksl.f90:286-301)."""
    out = 0
    for k in range(n):
        out = out + phi_right(ry1, 1, ry2, ry1, 1, ry2, ra1, ra2, phi, _slice(A, ra1, n, ra2, k),
                              _slice(x, ry1, n, ry2, k), _slice(x, ry1, n, ry2, k), conj=True)
    return out


def ztt_diag_ksl(d, n, ra, crA, crY0, ry, tau, rmax, typ=2, order=8):
    """One step of ztt_diag_ksl (tt_diag_ksl.f90:560-804), the KSL scheme for
    an operator diagonal in the physical index (cores A(a1, i, a2)).

    As ztt_ksl, except: every K-step runs one Krylov exponential per slice
    k = 1..n of the core (the local operator is bfun3 with m = n = 1 and the
    slice A(:, k, :)); the interfaces are the slice sums zphi_diag_left/right;
    every exponential takes anorm = 1 (the reference's norm estimates are
    commented out).  dtt_diag_ksl (:315-558) is the same scheme in real
    arithmetic; for real data this function gives it with zero imaginary
    parts.  Returns dict(cores, ry)."""
    n = list(map(int, n)); ra = list(map(int, ra)); ry = list(map(int, ry))
    crA = np.asarray(crA, dtype=np.complex128)
    eps = 1e-8
    pa = compute_ps(d, ra, n)
    Acore = [crA[pa[i]:pa[i + 1]] for i in range(d)]
    cr = []
    off = 0
    for i in range(d):
        sz = ry[i] * n[i] * ry[i + 1]
        cr.append(np.array(crY0[off:off + sz], dtype=np.complex128))
        off += sz
    phi = [None] * (d + 1)
    phi[0] = np.ones(1, dtype=np.complex128)
    phi[d] = np.ones(1, dtype=np.complex128)
    for i in range(d - 1):
        rnew = min(ry[i] * n[i], ry[i + 1])
        q, r = zqr_lapack(ry[i] * n[i], ry[i + 1], cr[i])
        cr[i] = q
        cr[i + 1] = flat(F(r, rnew, ry[i + 1]) @ F(cr[i + 1], ry[i + 1], n[i + 1] * ry[i + 2]))
        ry[i + 1] = rnew
        phi[i + 1] = phi_diag_left(ry[i], n[i], ry[i + 1], ra[i], ra[i + 1], phi[i], Acore[i], cr[i])
    tau0 = tau / 2 if typ == 2 else tau

    def kstep(i):
        r1, r2 = ry[i], ry[i + 1]
        N = r1 * r2
        out = np.zeros((r1, n[i], r2), dtype=np.complex128, order="F")
        for k in range(n[i]):
            Ak = _slice(Acore[i], ra[i], n[i], ra[i + 1], k)
            mv = lambda x: bfun3(r1, 1, r2, r1, 1, r2, ra[i], ra[i + 1], phi[i], Ak, phi[i + 1], x)  # noqa: E731,B023
            w, _ = zexp_mv(N, min(order, N), tau0, _slice(cr[i], r1, n[i], r2, k), eps, 1.0, mv)
            out[:, k, :] = F(w, r1, r2)
        return flat(out)

    def sstep(rx1, rx2, rr, ry1, ry2, p1, p2, R):
        mv = sfun(rx1, rx2, rr, ry1, ry2, p1, p2)
        w, _ = zexp_mv(rx1 * ry2, order, -tau0, R, eps, 1.0, mv)
        return w

    i, dir_, swp = d - 1, -1, 0
    while swp < 1:
        curcr = kstep(i)
        if dir_ < 0:
            if i > 0:
                ct = dtransp(ry[i], n[i] * ry[i + 1], curcr)
                rnew = min(n[i] * ry[i + 1], ry[i])
                q, r = zqr_lapack(n[i] * ry[i + 1], ry[i], ct)
                core = dtransp(n[i] * ry[i + 1], rnew, q)
                cr[i] = core
                R = dtransp(rnew, ry[i], r)
                phitmp = phi_diag_right(rnew, n[i], ry[i + 1], ra[i], ra[i + 1], phi[i + 1],
                                        Acore[i], core)
                if rnew != ry[i]:
                    raise ValueError("KSL S-step needs a rank-preserving QR")
                Stmp = sstep(ry[i], ry[i], ra[i], rnew, rnew, phi[i], phitmp, R)
                cr[i - 1] = flat(F(cr[i - 1], ry[i - 1] * n[i - 1], ry[i]) @ F(Stmp, ry[i], rnew))
                ry[i] = rnew
                phi[i] = phitmp
            else:
                cr[i] = curcr
        else:
            if i < d - 1:
                q, r = zqr_lapack(ry[i] * n[i], ry[i + 1], curcr)
                rnew = min(ry[i] * n[i], ry[i + 1])
                cr[i] = q
                phitmp = phi_diag_left(ry[i], n[i], rnew, ra[i], ra[i + 1], phi[i], Acore[i], q)
                if rnew != ry[i + 1]:
                    raise ValueError("KSL S-step needs a rank-preserving QR")
                Stmp = sstep(rnew, rnew, ra[i + 1], ry[i + 1], ry[i + 1], phitmp, phi[i + 1], r)
                cr[i + 1] = flat(F(Stmp, rnew, ry[i + 1]) @ F(cr[i + 1], ry[i + 1], n[i + 1] * ry[i + 2]))
                ry[i + 1] = rnew
                phi[i + 1] = phitmp
            else:
                cr[i] = curcr
        if dir_ > 0 and i == d - 1:
            dir_, i = -1, d - 1
            swp += 1
        elif dir_ < 0 and i == 0:
            dir_, i = 1, 0
            if typ == 1:
                break
        else:
            i += dir_
    cores = np.concatenate([cr[k][:ry[k] * n[k] * ry[k + 1]] for k in range(d)])
    return {"cores": cores, "ry": ry}


def tt_full(d, n, ry, cores):
    """Dense vector (earlier modes fastest) of a TT with ry[0] = ry[d] = 1."""
    off = 0
    cur = np.ones((1, 1), dtype=np.result_type(cores.dtype, np.float64))
    for i in range(d):
        sz = ry[i] * n[i] * ry[i + 1]
        c = F(cores[off:off + sz], ry[i], n[i] * ry[i + 1])
        off += sz
        cur = (cur @ c).reshape(-1, ry[i + 1], order="F")
    return cur[:, 0]
