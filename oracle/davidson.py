"""Block generalized-Davidson (GD+k) local eigensolver, oracle twin.

Test infrastructure only (see ``oracle/__init__.py``).  The reference solves
each local eigenproblem of ``tt_eigb`` with the vendored PRIMME started from
the current block (``initSize = B``), tolerance eps/sqrt(d)/10 relative to the
estimated norm of the operator, ``maxBasisSize = 100``,
``minRestartSize = min(B+1, N-1)``, ``maxMatvecs = 500``
(tt_eigb.f90:252-283).  PRIMME's GD+k restart keeps the current Ritz vectors
plus the previous iteration's Ritz vectors (primme/restart_d.c:120) and its
default convergence test is ||r|| <= eps * max|theta| (primme_interface.c).
This restatement runs that method with block expansion (every unconverged
residual is added per iteration), block classical Gram-Schmidt with Cholesky
QR, twice (BCGS2), for the basis, and a dense Rayleigh-Ritz solve.

The device solver of the CUDA library executes these exact steps in the same
order, so this module is also the step-by-step twin that checks it.
"""
import numpy as np
import scipy.linalg as sla

CHOL_DROP = 1e-14     # relative pivot below which a new direction is dropped
RESTART_DROP = 1e-10  # norm below which a previous Ritz direction is dropped


def chol_drop(G, tol=CHOL_DROP):
    """Cholesky of a Gram matrix that skips dependent columns.

    Returns (kept, Minv) with T[:, kept] @ Minv orthonormal when G = T^T T.
    """
    t = G.shape[0]
    L = np.zeros((t, t))
    kept = []
    for j in range(t):
        gjj = G[j, j]
        d = gjj - sum(L[j, k] ** 2 for k in kept)
        if not (gjj > 0) or d <= tol * gjj:
            continue
        L[j, j] = np.sqrt(d)
        for i in range(j + 1, t):
            L[i, j] = (G[i, j] - sum(L[i, k] * L[j, k] for k in kept)) / L[j, j]
        kept.append(j)
    Lk = L[np.ix_(kept, kept)]
    Minv = sla.solve_triangular(Lk, np.eye(len(kept)), lower=True).T if kept else np.zeros((0, 0))
    return kept, Minv


def orth_block(V, T):
    """BCGS2: project out V, Cholesky-QR; twice.  Drops dependent columns."""
    for _ in range(2):
        if V is not None and V.shape[1]:
            T = T - V @ (V.T @ T)
        kept, Minv = chol_drop(T.T @ T)
        T = T[:, kept] @ Minv
        if T.shape[1] == 0:
            break
    return T


def restart_coeffs(S, kr, Sprev, maxkc):
    """Coefficients of the GD+k restart: [S[:, :kr], orth(Sprev)] (MGS, twice),
    at most ``maxkc`` columns so that one expansion vector still fits."""
    k = S.shape[0]
    C = [S[:, j].copy() for j in range(kr)]
    if Sprev is not None:
        for b in range(Sprev.shape[1]):
            if len(C) >= maxkc:
                break
            p = np.zeros(k)
            p[:Sprev.shape[0]] = Sprev[:, b]
            for _ in range(2):
                for c in C:
                    p = p - c * (c @ p)
            nrm = np.linalg.norm(p)
            if nrm > RESTART_DROP:
                C.append(p / nrm)
    return np.column_stack(C)


def davidson(matvec, X0, B, tol, maxb=None, max_matvecs=500, keep=None):
    """Lowest B eigenpairs of a symmetric operator given by ``matvec(X)``.

    ``matvec`` maps an (N, k) array to (N, k).  Returns (theta, X, resnorms,
    matvecs, iterations).
    """
    N = X0.shape[0]
    maxb, keep = davidson_sizes(N, B, maxb, keep)
    V = orth_block(None, np.array(X0, dtype=np.float64))
    W = matvec(V)
    nmv = V.shape[1]
    H = V.T @ W
    H = 0.5 * (H + H.T)
    anorm = 0.0
    Sprev = None
    it = 0
    while True:
        it += 1
        k = V.shape[1]
        theta, S = sla.eigh(H)
        anorm = max(anorm, abs(theta[0]), abs(theta[-1]))
        nb = min(B, k)
        X = V @ S[:, :nb]
        AX = W @ S[:, :nb]
        R = AX - X * theta[:nb]
        rn = np.linalg.norm(R, axis=0)
        conv = rn <= tol * anorm
        if conv.all() or nmv >= max_matvecs or k >= N:
            return theta[:nb], X, rn, nmv, it
        T = R[:, ~conv]
        if k + T.shape[1] > maxb:
            kr = min(keep, k)
            C = restart_coeffs(S, kr, Sprev, maxb - 1)
            V = V @ C
            W = W @ C
            H = C.T @ H @ C
            H = 0.5 * (H + H.T)
            Sprev = None
            k = V.shape[1]
            T = T[:, :max(1, min(T.shape[1], maxb - k))]
        else:
            Sprev = S[:, :nb].copy()
        T = orth_block(V, T)
        if T.shape[1] == 0:
            return theta[:nb], X, rn, nmv, it
        WT = matvec(T)
        nmv += T.shape[1]
        t = T.shape[1]
        Hn = np.zeros((k + t, k + t))
        Hn[:k, :k] = H
        Hn[:k, k:] = V.T @ WT
        Hn[k:, :k] = Hn[:k, k:].T
        Tw = T.T @ WT
        Hn[k:, k:] = 0.5 * (Tw + Tw.T)
        H = Hn
        V = np.hstack([V, T])
        W = np.hstack([W, WT])


def davidson_sizes(N, B, maxb=None, keep=None):
    """Basis limits shared with the device solver."""
    if maxb is None:
        maxb = max(4 * B, 32)
    maxb = min(maxb, N)
    if keep is None:
        keep = min(B + max(1, B // 2), max(maxb - B, 1))
    return maxb, keep
