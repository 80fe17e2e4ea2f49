"""Krylov exponential (Expokit ZGEXPV / ZGPADM) restated in numpy (oracle).

Test infrastructure only (see ``oracle/__init__.py``).

``zgpadm``  follows expm/expokit.f:767-940 (ZGPADM): irreducible (ideg,ideg)
            Pade approximant of exp(tH) with scaling and squaring, the scale
            chosen from the infinity norm of tH.
``zgexpv``  follows expm/expokit.f:2403-2793 (ZGEXPV): Arnoldi with modified
            Gram-Schmidt (m steps), happy-breakdown tolerance 1e-7, local
            error estimate from the last two entries of exp(tH_{m+2}) e_1,
            step rejection and the step-size rule with delta = 1.2,
            gamma = 0.9, step sizes rounded to two significant digits,
            mxstep = 500.
``zexp_mv`` follows expm/explib.f90:53-125: m1 = min(m, n); 1x1 problems
            use the matvec of 1; the start vector is normalised.
"""
import math

import numpy as np


def zgpadm(ideg, m, t, H):
    """exp(t H) for a small dense m x m complex matrix (ZGPADM)."""
    H = np.asarray(H, dtype=np.complex128)[:m, :m]
    hnorm = np.abs(H).sum(axis=1).max()
    hnorm = abs(t * hnorm)
    if hnorm == 0.0:
        raise ValueError("null H in input of ZGPADM")
    ns = max(0, int(math.log(hnorm) / math.log(2.0)) + 2)
    scale = t / float(2 ** ns)
    scale2 = scale * scale
    # Pade coefficients
    i, j = ideg + 1, 2 * ideg + 1
    coef = [1.0 + 0j]
    for k in range(1, ideg + 1):
        coef.append(coef[k - 1] * float(i - k) / float(k * (j - k)))
    H2 = scale2 * (H @ H)
    I = np.eye(m, dtype=np.complex128)
    P = coef[ideg - 1] * I
    Q = coef[ideg] * I
    iodd = 1
    k = ideg - 1
    while True:
        used = Q if iodd else P
        F = used @ H2
        F = F + coef[k - 1] * I
        if iodd:
            Q = F
        else:
            P = F
        iodd = 1 - iodd
        k -= 1
        if k <= 0:
            break
    if iodd:
        Q = scale * (Q @ H)
    else:
        P = scale * (P @ H)
    Q = Q - P
    E = np.linalg.solve(Q, P)
    E = 2.0 * E + I
    if ns == 0 and iodd:
        return -E
    for _ in range(ns):
        E = E @ E
    return E


def _nint(x):
    """Fortran NINT: nearest integer, halves away from zero."""
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


def _round2(x):
    """Expokit's step rounding: keep about two significant digits."""
    sqr1 = math.sqrt(0.1)
    p1 = 10.0 ** (_nint(math.log10(x) - sqr1) - 1)
    return math.trunc(x / p1 + 0.55) * p1


def zgexpv(n, m, t, v, tol, anorm, matvec, mxstep=500):
    """w = exp(t A) v by Krylov steps (ZGEXPV).  Returns (w, stats)."""
    ideg = 6
    delta, gamma = 1.2, 0.9
    eps = np.finfo(float).eps
    if tol <= eps:
        tol = math.sqrt(eps)
    rndoff = eps * anorm
    break_tol = 1.0e-7
    sgn = math.copysign(1.0, t)
    t_out = abs(t)
    w = np.array(v, dtype=np.complex128)
    beta = np.linalg.norm(w)
    vnorm = beta
    xm = 1.0 / m
    p2 = tol * (((m + 1) / 2.72) ** (m + 1)) * math.sqrt(2.0 * 3.14 * (m + 1))
    t_new = (1.0 / anorm) * (p2 / (4.0 * beta * anorm)) ** xm
    t_new = _round2(t_new)
    t_now = 0.0
    nstep = nmult = nreject = 0
    mh = m + 2
    while t_now < t_out:
        nstep += 1
        t_step = min(t_out - t_now, t_new)
        V = np.zeros((n, m + 1), dtype=np.complex128)
        Hm = np.zeros((mh, mh), dtype=np.complex128)
        V[:, 0] = w / beta
        k1 = 2
        mbrkdwn = m
        avnorm = 0.0
        breakdown = False
        for j in range(m):
            nmult += 1
            p = matvec(V[:, j])
            for i in range(j + 1):
                hij = np.vdot(V[:, i], p)
                p = p - hij * V[:, i]
                Hm[i, j] = hij
            hj1j = np.linalg.norm(p)
            if hj1j <= break_tol:
                k1 = 0
                mbrkdwn = j + 1
                t_step = t_out - t_now
                breakdown = True
                break
            Hm[j + 1, j] = hj1j
            V[:, j + 1] = p / hj1j
        if not breakdown:
            nmult += 1
            avnorm = np.linalg.norm(matvec(V[:, m]))
        Hm[m + 1, m] = 1.0
        while True:
            mx = mbrkdwn + k1
            E = zgpadm(ideg, mx, sgn * t_step, Hm)
            if k1 == 0:
                err_loc = tol
            else:
                p1 = abs(E[m, 0]) * beta
                p2 = abs(E[m + 1, 0]) * beta * avnorm
                if p1 > 10.0 * p2:
                    err_loc = p2
                    xm = 1.0 / m
                elif p1 > p2:
                    err_loc = (p1 * p2) / (p1 - p2)
                    xm = 1.0 / m
                else:
                    err_loc = p1
                    xm = 1.0 / (m - 1)
            if k1 != 0 and err_loc > delta * t_step * tol:
                t_step = gamma * t_step * (t_step * tol / err_loc) ** xm
                t_step = _round2(t_step)
                nreject += 1
                continue
            break
        mx = mbrkdwn + max(0, k1 - 1)
        w = beta * (V[:, :mx] @ E[:mx, 0])
        beta = np.linalg.norm(w)
        t_new = gamma * t_step * (t_step * tol / err_loc) ** xm
        t_new = _round2(t_new)
        t_now += t_step
        if nstep >= mxstep:
            break
    return w, {"nmult": nmult, "nstep": nstep, "nreject": nreject}


def zexp_mv(n, m, tau, v, tol, anorm, matvec):
    """zexp_mv (explib.f90:53-125)."""
    m1 = min(m, n)
    if m1 == 1:
        a = matvec(np.ones(1, dtype=np.complex128))[0]
        return np.array([v[0] * np.exp(a * tau)]), {"nmult": 1, "nstep": 1, "nreject": 0}
    nrm = np.linalg.norm(v)
    if nrm > 0:
        w, st = zgexpv(n, m1, tau, np.asarray(v) / nrm, tol, anorm, matvec)
        return w * nrm, st
    return np.zeros(n, dtype=np.complex128), {"nmult": 0, "nstep": 0, "nreject": 0}
