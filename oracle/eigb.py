"""Block-TT ALS eigensolver ``tt_eigb`` restated on the CPU (oracle).

Test infrastructure only (see ``oracle/__init__.py``).  Follows
tt_eigb.f90:110-436 step by step:

  * QR orthogonalisation left->right with Phi-left updates   tt_eigb.f90:202-217
  * ry(d+1) := 1, sweep starts at i = d going left           tt_eigb.f90:220-230
  * local solve: dense ``dsyev`` below ``max_full_size``      tt_eigb.f90:234-249
    otherwise an iterative solver started from the current block with the
    reference's tolerance eps/sqrt(d)/10 relative to ||A||   tt_eigb.f90:252-290
    (the reference uses the vendored PRIMME GD+k; ``oracle/davidson.py``
    restates that method with block expansion)
  * stopping rule on the relative change of sum(lambda)      tt_eigb.f90:293-295
  * SVD of the block, ``my_chop3`` + rmax, fold into the neighbour core and
    Phi update (dir < 0)                                     tt_eigb.f90:305-356
    (dir > 0)                                                tt_eigb.f90:357-394
  * turn points and sweep counter                            tt_eigb.f90:397-411
"""
import numpy as np
import scipy.linalg as sla

from .ops import F, flat, dtransp, compute_ps, my_chop3, dqr, bfun3_block, phi_left, \
    phi_right, fullmat
from .davidson import davidson


def local_eig(rx1, n, rx2, ra1, ra2, phi1, A, phi2, X0, B, tol, max_full_size, maxmv=500,
              maxb=None, local_solver=None):
    """Lowest B eigenpairs of the local operator; returns (lam, V, res, nmv).
    local_solver (optional): (mv, X0, B, tol, max_matvecs) -> (lam, V, res,
    nmv) in place of oracle/davidson.py, e.g. oracle/primme.py's PRIMME."""
    N = rx1 * n * rx2
    if N < max_full_size:
        H = fullmat(rx1, n, rx2, ra1, ra2, phi1, A, phi2)
        w, v = sla.eigh(H)          # dsyev('V','U') equivalent
        return w[:B].copy(), v[:, :B].copy(), 0.0, 0
    count = [0]

    def mv(X):
        X = np.asarray(X).reshape(N, -1, order="F")
        count[0] += X.shape[1]
        out = bfun3_block(rx1, n, rx2, rx1, n, rx2, ra1, ra2, phi1, A, phi2, flat(X), X.shape[1])
        return F(out, N, X.shape[1])

    if local_solver is not None:
        return local_solver(mv, np.array(X0, copy=True), B, tol, maxmv)
    lam, V, rn, nmv, _ = davidson(mv, np.array(X0, copy=True), B, tol, maxb=maxb,
                                  max_matvecs=maxmv)
    return lam, V, float(np.linalg.norm(rn)), nmv


def tt_eigb(d, n, m, ra, crA, crY0, ry, eps, rmax, B, nswp=20, max_full_size=2000,
            verb=0, resid_damp=10.0, local_solver=None, record=None):
    """Restatement of ``tt_eigb`` (tt_eigb.f90:110).

    Arguments follow the Fortran signature with 0-based Python lists.  Returns
    a dict with ``lambda`` (B,), ``cores`` (flat, result_core layout), ``ry``
    (d+1, ry[d] = B), ``sweeps``, ``matvecs`` and the last local residual.
    local_solver replaces the iterative local eigensolver (see local_eig);
    record (a list) receives every iterative local problem as a dict
    (dims, phi1, A, phi2, X0, tol) before it is solved.
    """
    n = list(map(int, n)); m = list(map(int, m)); ra = list(map(int, ra))
    ry = list(map(int, ry))
    assert ry[d] == B, "Inconsistent number of eigenvalues sought and initial guess last rank"
    eps2 = eps / np.sqrt(d)
    pa = compute_ps(d, ra, [n[i] * m[i] for i in range(d)])
    Acore = [crA[pa[i]:pa[i + 1]] for i in range(d)]
    cr = []
    off = 0
    for i in range(d):
        sz = ry[i] * n[i] * ry[i + 1]
        cr.append(np.array(crY0[off:off + sz], dtype=np.float64))
        off += sz
    phi = [None] * (d + 1)
    phi[0] = np.ones(1)
    phi[d] = np.ones(1)
    # QR sweep, tt_eigb.f90:202-217
    for i in range(d):
        rnew = min(ry[i] * n[i], ry[i + 1])
        q, r = dqr(ry[i] * n[i], ry[i + 1], cr[i])
        cr[i] = q
        if i < d - 1:
            cr[i + 1] = flat(F(r, rnew, ry[i + 1]) @ F(cr[i + 1], ry[i + 1], n[i + 1] * ry[i + 2]))
            ry[i + 1] = rnew
            phi[i + 1] = phi_left(ry[i], m[i], ry[i + 1], ry[i], n[i], ry[i + 1], ra[i], ra[i + 1],
                                  phi[i], Acore[i], cr[i], cr[i])
    ry[d] = 1
    i = d - 1
    dir_ = -1
    swp = 1
    ermax = 0.0
    fvold = 0.0
    lam = np.zeros(B)
    total_mv = 0
    res = 0.0
    history = []
    while swp <= nswp:
        N = ry[i] * n[i] * ry[i + 1]
        X0 = F(cr[i][:N * B], N, B)
        if record is not None and N >= max_full_size:
            record.append({"dims": (ry[i], n[i], ry[i + 1], ra[i], ra[i + 1]),
                           "phi1": phi[i].copy(), "A": Acore[i].copy(), "phi2": phi[i + 1].copy(),
                           "X0": X0.copy(), "tol": eps2 / resid_damp})
        lam, V, res, nmv = local_eig(ry[i], n[i], ry[i + 1], ra[i], ra[i + 1], phi[i], Acore[i],
                                     phi[i + 1], X0, B, eps2 / resid_damp, max_full_size,
                                     local_solver=local_solver)
        curcr = flat(V)
        fv = float(np.sum(lam))
        erloc = (fvold - fv) / abs(fv)
        ermax = max(ermax, erloc)
        total_mv += nmv
        fvold = fv
        if verb:
            print(f"swp {swp} i {i + 1} N {N} mv {nmv} res {res:.3e} ermax {ermax:.3e}")
        if dir_ < 0 and i > 0:
            Mt = F(dtransp(N, B, curcr), B * ry[i], n[i] * ry[i + 1])
            U, s, VT = sla.svd(Mt, full_matrices=False, lapack_driver="gesvd")
            nn = min(my_chop3(s, eps2), rmax)
            Us = U[:, :nn] * s[:nn]
            cr[i] = flat(VT[:nn, :])
            Ut = dtransp(B, ry[i] * nn, flat(Us))          # ry(i) x nn x B
            cr[i - 1] = flat(F(cr[i - 1], ry[i - 1] * n[i - 1], ry[i]) @ F(Ut, ry[i], nn * B))
            ry[i] = nn
            phi[i] = phi_right(ry[i], n[i], ry[i + 1], ry[i], n[i], ry[i + 1], ra[i], ra[i + 1],
                               phi[i + 1], Acore[i], cr[i], cr[i])
        if dir_ > 0 and i < d - 1:
            M = F(curcr, ry[i] * n[i], ry[i + 1] * B)
            U, s, VT = sla.svd(M, full_matrices=False, lapack_driver="gesvd")
            nn = min(my_chop3(s, eps2), rmax)
            cr[i] = flat(U[:, :nn])
            SV = flat(s[:nn, None] * VT[:nn, :])             # nn x (ry(i+1) B)
            SVt = dtransp(nn * ry[i + 1], B, SV)             # B x nn x ry(i+1)
            cur = F(SVt, B * nn, ry[i + 1]) @ F(cr[i + 1], ry[i + 1], n[i + 1] * ry[i + 2])
            cr[i + 1] = dtransp(B, nn * n[i + 1] * ry[i + 2], flat(cur))
            ry[i + 1] = nn
            phi[i + 1] = phi_left(ry[i], n[i], ry[i + 1], ry[i], n[i], ry[i + 1], ra[i], ra[i + 1],
                                  phi[i], Acore[i], cr[i], cr[i])
        if dir_ > 0 and i == d - 2:
            dir_ = -1
            i = d - 1
            history.append(ermax)
            swp += 1
            if ermax < eps:
                break
            ermax = 0.0
        elif dir_ < 0 and i == 1:
            dir_ = 1
            i = 0
        else:
            i += dir_
    ry[d] = B
    cores = np.concatenate([cr[k][:ry[k] * n[k] * ry[k + 1]] for k in range(d)])
    return {"lambda": np.array(lam), "cores": cores, "ry": ry, "sweeps": swp - 1,
            "matvecs": total_mv, "res": res, "history": history}


def tt_full_block(d, n, ry, cores):
    """Expand a TT block (ry[d] = B) into a dense (prod(n), B) matrix (small d)."""
    off = 0
    cur = np.ones((1, 1))
    for i in range(d):
        sz = ry[i] * n[i] * ry[i + 1]
        c = F(cores[off:off + sz], ry[i], n[i] * ry[i + 1])
        off += sz
        cur = (cur @ c).reshape(-1, ry[i + 1], order="F")
    return cur
