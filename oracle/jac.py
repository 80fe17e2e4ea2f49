"""Block-Jacobi preconditioners of the local AMEn system (oracle).

Test infrastructure only (see ``oracle/__init__.py``).  Restates ``djac_gen``
(tt_linalg.f90:363-494) and ``djac_apply`` (tt_linalg.f90:497-531), the
preconditioners ``prec = 'c' | 'l' | 'r'`` of ``tt_amen_solve``
(tt_adapt_als.f90:746-779).  Each keeps a part of the local operator
B[(c1,i,c2),(b1,j,b2)] = sum Phi1[c1,b1,a1] A[a1,i,j,a2] Phi2[b2,a2,c2]
and inverts it block by block:

  'c'  the diagonals of Phi1 and Phi2 only: one n x n block per (b1, b2),
       M[i, j] = sum d1[b1,a1] A[a1,i,j,a2] d2[b2,a2], with
       d1[b,a1] = Phi1[b,b,a1] and d2[b,a2] = Phi2[b,a2,b];
       jacs (n, n, rx2, rx1), block (b2, b1) at offset n^2 (b2 + rx2 b1)
  'l'  all of Phi1, the diagonal of Phi2: one (rx1 n)^2 block per b2 with
       rows (c1, i) and columns (b1, j); jacs (rx1 n, rx1 n, rx2)
  'r'  the diagonal of Phi1, all of Phi2: one (n rx2)^2 block per b1 with
       rows (i, c2) and columns (j, b2); jacs (n rx2, n rx2, rx1)

Every block is inverted by LU with partial pivoting (``dgesv`` against the
identity).  ``jac_apply`` multiplies each block with its part of x, so it
maps x (rx1, n, rx2) to y of the same layout.
"""
import numpy as np

from .ops import F, flat


def _diag1(phi1, rx1, ra1):
    P1 = F(phi1, rx1, rx1, ra1)
    return np.einsum("bba->ba", P1)                     # rx1 x ra1


def _diag2(phi2, rx2, ra2):
    P2 = F(phi2, rx2, ra2, rx2)
    return np.einsum("bab->ba", P2)                     # rx2 x ra2


def jac_gen(ptype, rx1, n, rx2, ra1, ra2, phi1, A, phi2):
    """``djac_gen``: the inverted blocks as the flat jacs array."""
    A4 = F(A, ra1, n, n, ra2)
    p = ptype.lower()
    if p == "c":
        M = np.einsum("ba,aijc,dc->ijdb", _diag1(phi1, rx1, ra1), A4, _diag2(phi2, rx2, ra2))
        blocks = M.reshape(n, n, rx2 * rx1, order="F")
    elif p == "l":
        P1 = F(phi1, rx1, rx1, ra1)
        M = np.einsum("xya,aijc,dc->xiyjd", P1, A4, _diag2(phi2, rx2, ra2))
        k = rx1 * n
        blocks = M.reshape(k, k, rx2, order="F")
    elif p == "r":
        P2 = F(phi2, rx2, ra2, rx2)
        M = np.einsum("ba,aijc,ecf->ifjeb", _diag1(phi1, rx1, ra1), A4, P2)
        k = n * rx2
        blocks = M.reshape(k, k, rx1, order="F")
    else:
        raise ValueError("prec must be 'c', 'l' or 'r'")
    inv = np.empty_like(blocks)
    for q in range(blocks.shape[2]):
        inv[:, :, q] = np.linalg.solve(blocks[:, :, q], np.eye(blocks.shape[0]))
    return flat(inv)


def jac_apply(ptype, rx1, n, rx2, jacs, x):
    """``djac_apply``: y = blockdiag(jacs) x, x and y of layout (rx1, n, rx2)."""
    p = ptype.lower()
    X = F(x, rx1, n, rx2)
    if p == "c":
        J = F(jacs, n, n, rx2, rx1)
        Y = np.einsum("ijdb,bjd->bid", J, X)
    elif p == "l":
        k = rx1 * n
        J = F(jacs, k, k, rx2)
        Y = np.einsum("rcd,cd->rd", J, X.reshape(k, rx2, order="F")).reshape(rx1, n, rx2,
                                                                                  order="F")
    elif p == "r":
        k = n * rx2
        J = F(jacs, k, k, rx1)
        Y = np.einsum("rcb,bc->br", J, X.reshape(rx1, k, order="F")).reshape(rx1, n, rx2,
                                                                                  order="F")
    else:
        raise ValueError("prec must be 'c', 'l' or 'r'")
    return flat(Y)


def jac_size(ptype, rx1, n, rx2):
    p = ptype.lower()
    if p == "c":
        return n * n * rx2 * rx1
    if p == "l":
        return (rx1 * n) ** 2 * rx2
    return (n * rx2) ** 2 * rx1
