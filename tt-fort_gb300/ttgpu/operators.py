"""Input builders for the sweep workloads: TT-matrices (operators) and TT blocks.

All cores are flat column-major buffers in the reference layout:
  TT-matrix core i   A(a1, i_row, j_col, a2), shape (ra_i, n_i, m_i, ra_{i+1})
  TT (block) core i  X(r_i, n_i, r_{i+1}),    the last rank carries the block
These are the ``crA`` / ``crY0`` arrays that ``tt_eigb`` (tt_eigb.f90:110),
``ztt_ksl`` (tt_ksl.f90:431) and ``tt_amen_solve`` (tt_adapt_als.f90:513) take.
"""
import numpy as np


def _flat(a):
    return np.ravel(a, order="F")


def xxz_mpo(d, delta=1.0, J=1.0):
    """Open-boundary spin-1/2 XXZ chain  H = sum_k J(SxSx + SySy) + delta SzSz.

    With delta = 1 this is the Heisenberg chain of the reference fixture
    ``Heisen_20.sdv`` (same operator, same boundary ranks [1,4,5,...,5,4,1]).
    Returns (n, m, ra, crA) with n = m = 2.
    """
    I = np.eye(2)
    Sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    Sm = Sp.T.copy()
    Sz = np.diag([0.5, -0.5])
    W = np.zeros((5, 2, 2, 5))
    W[0, :, :, 0] = I
    W[0, :, :, 1] = Sp
    W[0, :, :, 2] = Sm
    W[0, :, :, 3] = Sz
    W[1, :, :, 4] = 0.5 * J * Sm
    W[2, :, :, 4] = 0.5 * J * Sp
    W[3, :, :, 4] = delta * Sz
    W[4, :, :, 4] = I
    # bond k (between sites k and k+1) keeps states reachable from the left
    # and able to reach the right end
    fixed = []
    for k in range(d):
        left = [0] if k == 0 else _bond_states(k, d)
        right = [4] if k == d - 1 else _bond_states(k + 1, d)
        fixed.append(W[np.ix_(left, [0, 1], [0, 1], right)])
    ra = [1] + [len(_bond_states(k, d)) for k in range(1, d)] + [1]
    crA = np.concatenate([_flat(c) for c in fixed])
    return [2] * d, [2] * d, ra, crA


def _bond_states(k, d):
    """MPO states alive on bond k (1 <= k <= d-1)."""
    s = [0, 1, 2, 3, 4]
    if k == 1:
        s = [0, 1, 2, 3]          # nothing can be finished after one site
    if k == d - 1:
        s = [x for x in s if x != 0]  # the last site cannot start a pair
    return s


def laplace_tt(d, n, scale=1.0):
    """sum_k I x .. x L_k x .. x I with L = tridiag(-1, 2, -1) (Dirichlet), rank 2."""
    L = scale * (2 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1))
    I = np.eye(n)
    cores = []
    for k in range(d):
        if d == 1:
            c = L.reshape(1, n, n, 1)
        elif k == 0:
            c = np.zeros((1, n, n, 2)); c[0, :, :, 0] = L; c[0, :, :, 1] = I
        elif k == d - 1:
            c = np.zeros((2, n, n, 1)); c[0, :, :, 0] = I; c[1, :, :, 0] = L
        else:
            c = np.zeros((2, n, n, 2))
            c[0, :, :, 0] = I; c[1, :, :, 0] = L; c[1, :, :, 1] = I
        cores.append(c)
    return cores


def tt_matrix_sum(a, b):
    """Cores of the TT-matrix a + b (block-diagonal core stacking)."""
    d = len(a)
    out = []
    for k in range(d):
        x, y = a[k], b[k]
        r1x, n, m, r2x = x.shape
        r1y, _, _, r2y = y.shape
        if d == 1:
            out.append(x + y)
        elif k == 0:
            c = np.zeros((1, n, m, r2x + r2y)); c[:, :, :, :r2x] = x; c[:, :, :, r2x:] = y
            out.append(c)
        elif k == d - 1:
            c = np.zeros((r1x + r1y, n, m, 1)); c[:r1x] = x; c[r1x:] = y
            out.append(c)
        else:
            c = np.zeros((r1x + r1y, n, m, r2x + r2y))
            c[:r1x, :, :, :r2x] = x; c[r1x:, :, :, r2x:] = y
            out.append(c)
    return out


def pack_tt_matrix(cores):
    d = len(cores)
    n = [c.shape[1] for c in cores]
    m = [c.shape[2] for c in cores]
    ra = [cores[0].shape[0]] + [c.shape[3] for c in cores]
    return n, m, ra, np.concatenate([_flat(c) for c in cores])


def ksl_operator(d=16, n=32, rank=4, std=0.01, seed=1):
    """KSL workload operator: -(d-dim Dirichlet Laplacian) + random TT-matrix.

    The perturbation has TT-rank ``rank`` with i.i.d. N(0, std^2) core entries
    drawn from ``numpy.random.default_rng(seed)``; total TT-rank 2 + rank.
    """
    rng = np.random.default_rng(seed)
    lap = laplace_tt(d, n, scale=-1.0)
    pert = []
    for k in range(d):
        r1 = 1 if k == 0 else rank
        r2 = 1 if k == d - 1 else rank
        pert.append(std * rng.standard_normal((r1, n, n, r2)))
    return pack_tt_matrix(tt_matrix_sum(lap, pert))


def amen_operator(d=10, n=64, sigma_frac=0.3):
    """AMEn workload: Laplacian + diag(exp(-|i - c|^2 / sigma^2)), rank 3.

    The grid index is centred at c = (n-1)/2 in every mode, sigma = sigma_frac*n.
    The potential is a rank-1 TT-matrix (a product of diagonal factors).
    """
    lap = laplace_tt(d, n)
    sigma = sigma_frac * n
    g = np.exp(-((np.arange(n) - (n - 1) / 2.0) ** 2) / sigma ** 2)
    pot = [np.diag(g).reshape(1, n, n, 1) for _ in range(d)]
    return pack_tt_matrix(tt_matrix_sum(lap, pot))


def random_tt(d, n, r, last=1, seed=0, dist="normal"):
    """Random TT (block) vector, ranks [1, r, ..., r, last], flat cores.

    Entries N(0,1) (``dist='normal'``) or U[0,1) from default_rng(seed).
    Interior ranks are clipped to what the mode sizes allow.
    """
    rng = np.random.default_rng(seed)
    if np.isscalar(n):
        n = [int(n)] * d
    ry = [1] + [int(r)] * (d - 1) + [int(last)]
    cores = []
    for k in range(d):
        sz = ry[k] * n[k] * ry[k + 1]
        if dist == "normal":
            cores.append(rng.standard_normal(sz))
        else:
            cores.append(rng.random(sz))
    return list(n), ry, np.concatenate(cores)


def random_tt_complex(d, n, r, seed=0):
    rng = np.random.default_rng(seed)
    if np.isscalar(n):
        n = [int(n)] * d
    ry = [1] + [int(r)] * (d - 1) + [1]
    cores = []
    for k in range(d):
        sz = ry[k] * n[k] * ry[k + 1]
        cores.append(rng.standard_normal(sz) + 1j * rng.standard_normal(sz))
    return list(n), ry, np.concatenate(cores)


def tt_dot(d, n, rx, x, ry, y):
    """Inner product sum(conj(x) * y) of two TT vectors given as flat
    Fortran-ordered cores (r_k x n_k x r_{k+1}), contracted left to right."""
    if np.isscalar(n):
        n = [int(n)] * d
    P = np.ones((1, 1), dtype=np.result_type(x, y))
    ox = oy = 0
    for k in range(d):
        sx, sy = rx[k] * n[k] * rx[k + 1], ry[k] * n[k] * ry[k + 1]
        X = np.asarray(x[ox:ox + sx]).reshape(rx[k], n[k], rx[k + 1], order="F")
        Y = np.asarray(y[oy:oy + sy]).reshape(ry[k], n[k], ry[k + 1], order="F")
        ox += sx
        oy += sy
        P = np.einsum("aic,ab,bie->ce", np.conj(X), P, Y, optimize=True)
    return P[0, 0]


def tt_norm(d, n, r, cores):
    """2-norm of a TT vector by a left-to-right QR sweep (no cancellation)."""
    if np.isscalar(n):
        n = [int(n)] * d
    R = np.ones((1, 1), dtype=np.asarray(cores).dtype)
    off = 0
    for k in range(d):
        sz = r[k] * n[k] * r[k + 1]
        C = np.asarray(cores[off:off + sz]).reshape(r[k], n[k] * r[k + 1], order="F")
        off += sz
        C = (R @ C).reshape(-1, r[k + 1], order="F")
        if k == d - 1:
            return float(np.linalg.norm(C))
        _, R = np.linalg.qr(C)
    return float(np.linalg.norm(R))


def tt_sub(d, n, rx, x, ry, y):
    """x - y as one TT vector with ranks rx + ry (block cores)."""
    if np.isscalar(n):
        n = [int(n)] * d
    out, r = [], [1]
    ox = oy = 0
    for k in range(d):
        X = np.asarray(x[ox:ox + rx[k] * n[k] * rx[k + 1]]).reshape(rx[k], n[k], rx[k + 1], order="F")
        Y = np.asarray(y[oy:oy + ry[k] * n[k] * ry[k + 1]]).reshape(ry[k], n[k], ry[k + 1], order="F")
        ox += X.size
        oy += Y.size
        a = 1 if k == 0 else rx[k] + ry[k]
        b = 1 if k == d - 1 else rx[k + 1] + ry[k + 1]
        Z = np.zeros((a, n[k], b), dtype=np.result_type(X, Y))
        if d == 1:
            Z[:] = X - Y
        elif k == 0:
            Z[:, :, :rx[1]] = X
            Z[:, :, rx[1]:] = -Y
        elif k == d - 1:
            Z[:rx[k], :, :] = X
            Z[rx[k]:, :, :] = Y
        else:
            Z[:rx[k], :, :rx[k + 1]] = X
            Z[rx[k]:, :, rx[k + 1]:] = Y
        out.append(Z.ravel(order="F"))
        r.append(b)
    return r, np.concatenate(out)


def tt_rel_diff(d, n, rx, x, ry, y):
    """||x - y|| / ||y|| of two TT vectors, both norms by QR sweeps."""
    rz, z = tt_sub(d, n, rx, x, ry, y)
    return tt_norm(d, n, rz, z) / tt_norm(d, n, ry, y)
