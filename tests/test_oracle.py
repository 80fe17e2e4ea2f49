"""CPU tests: the oracle pinned against golden vectors and dense references."""
import json
import os

import numpy as np
import pytest
import scipy.linalg as sla

from conftest import GOLDEN
from oracle import ops
from oracle.davidson import davidson
from oracle.eigb import tt_eigb, tt_full_block
from ttgpu.operators import xxz_mpo, random_tt, laplace_tt, pack_tt_matrix, amen_operator


def tt_matrix_inner(ra1, c1, ra2, c2, N):
    """Frobenius inner product of two TT-matrices (cores with merged n*m index)."""
    o1 = o2 = 0
    T = np.ones((1, 1))
    for k in range(len(N)):
        a = c1[o1:o1 + ra1[k] * N[k] * ra1[k + 1]].reshape(ra1[k], N[k], ra1[k + 1], order="F")
        b = c2[o2:o2 + ra2[k] * N[k] * ra2[k + 1]].reshape(ra2[k], N[k], ra2[k + 1], order="F")
        o1 += a.size; o2 += b.size
        T = np.einsum("ab,aic,bid->cd", T, a, b)
    return T.item()


def tt_matrix_full(d, n, ra, crA):
    off = 0
    M = np.ones((1, 1, 1))
    for k in range(d):
        c = crA[off:off + ra[k] * n[k] * n[k] * ra[k + 1]].reshape(ra[k], n[k], n[k], ra[k + 1],
                                                                  order="F")
        off += c.size
        # M (I, J, a) x c (a, i, j, b) -> (I i, J j, b), earlier modes fastest
        M = np.einsum("IJa,aijb->IiJjb", M, c)
        s = M.shape
        M = M.reshape(s[0] * s[1], s[2] * s[3], s[4], order="F")
    return M[:, :, 0]


def test_heisenberg_generator_matches_reference_fixture():
    f = np.load(os.path.join(GOLDEN, "heisen20_sdv.npz"))
    N = list(f["n"]); r = list(f["r"]); cores = f["cores"]
    n, m, ra, crA = xxz_mpo(20)
    assert list(ra) == r
    a = tt_matrix_inner(r, cores, r, cores, N)
    b = tt_matrix_inner(ra, crA, ra, crA, N)
    c = tt_matrix_inner(r, cores, ra, crA, N)
    assert abs(a + b - 2 * c) <= 1e-12 * a


def _dense_heis(d):
    n, m, ra, crA = xxz_mpo(d)
    return tt_matrix_full(d, n, ra, crA)


def test_dense_heisenberg_small_is_the_chain():
    # the TT-matrix at d=4 against explicit Kronecker sums
    H = _dense_heis(4)
    sx = np.array([[0, 0.5], [0.5, 0]]); sz = np.diag([0.5, -0.5])
    sy = np.array([[0, -0.5j], [0.5j, 0]])
    I = np.eye(2)

    def op(o, k):
        mats = [I] * 4
        mats[k] = o
        out = mats[3]
        for q in (2, 1, 0):
            out = np.kron(out, mats[q])   # mode 0 fastest
        return out
    ref = sum(op(s, k) @ op(s, k + 1) for k in range(3) for s in (sx, sy, sz))
    assert np.allclose(H, ref.real, atol=1e-14)


def test_bfun3_equals_dense_local_matrix():
    rng = np.random.default_rng(0)
    rx1, m, rx2, ra1, ra2 = 3, 2, 4, 2, 3
    phi1 = rng.standard_normal(rx1 * rx1 * ra1)
    A = rng.standard_normal(ra1 * m * m * ra2)
    phi2 = rng.standard_normal(rx2 * ra2 * rx2)
    x = rng.standard_normal(rx1 * m * rx2)
    y = ops.bfun3(rx1, m, rx2, rx1, m, rx2, ra1, ra2, phi1, A, phi2, x)
    Bm = ops.fullmat(rx1, m, rx2, ra1, ra2, phi1, A, phi2)
    assert np.allclose(y, Bm @ x, rtol=1e-13, atol=1e-13)
    ref = np.einsum("cba,aijd,edf,bje->cif", ops.F(phi1, rx1, rx1, ra1), ops.F(A, ra1, m, m, ra2),
                    ops.F(phi2, rx2, ra2, rx2), ops.F(x, rx1, m, rx2))
    assert np.allclose(y, ops.flat(ref))


def test_phi_updates_are_projections():
    rng = np.random.default_rng(1)
    rx1, m, rx2, ry1, n, ry2, ra1, ra2 = 3, 2, 4, 2, 2, 3, 2, 3
    A = rng.standard_normal(ra1 * n * m * ra2)
    x = rng.standard_normal(rx1 * m * rx2)
    y = rng.standard_normal(ry1 * n * ry2)
    p1 = rng.standard_normal(ry1 * rx1 * ra1)
    p2 = rng.standard_normal(rx2 * ra2 * ry2)
    out = ops.phi_left(rx1, m, rx2, ry1, n, ry2, ra1, ra2, p1, A, x, y)
    ref = np.einsum("cba,cif,aijd,bje->fed", ops.F(p1, ry1, rx1, ra1), ops.F(y, ry1, n, ry2),
                    ops.F(A, ra1, n, m, ra2), ops.F(x, rx1, m, rx2))
    assert np.allclose(out, ops.flat(ref))
    out = ops.phi_right(rx1, m, rx2, ry1, n, ry2, ra1, ra2, p2, A, x, y)
    ref = np.einsum("bje,edf,aijd,cif->bac", ops.F(x, rx1, m, rx2), ops.F(p2, rx2, ra2, ry2),
                    ops.F(A, ra1, n, m, ra2), ops.F(y, ry1, n, ry2))
    assert np.allclose(out, ops.flat(ref))


def test_my_chop3_semantics():
    s = np.array([1.0, 0.5, 1e-3, 1e-6, 1e-9])
    # tail {1e-6, 1e-9} stays below (eps*||s||)^2 = 1.25e-12; the scan stops at
    # 1e-3 (i = 3) and keeps i + 1 = 4 values (one more than needed)
    assert ops.my_chop3(s, 1e-6) == 4
    assert ops.my_chop3(s, 1e-1) == 3
    assert ops.my_chop3(s, 10.0) == 1


def test_davidson_twin_vs_eigh():
    rng = np.random.default_rng(2)
    N, B = 300, 5
    Q = np.linalg.qr(rng.standard_normal((N, N)))[0]
    w = np.sort(rng.standard_normal(N))
    w[1:4] = w[1]                           # a degenerate triplet, like Heisenberg
    A = (Q * w) @ Q.T
    lam, X, rn, nmv, it = davidson(lambda V: A @ V, rng.standard_normal((N, B)), B, 1e-11,
                                   max_matvecs=5000)
    assert np.allclose(lam, np.sort(w)[:B], rtol=1e-10, atol=1e-10)
    R = A @ X - X * lam
    assert np.linalg.norm(R, axis=0).max() <= 1e-9


def test_oracle_eigb_exact_small_chain():
    d, B = 8, 4
    n, m, ra, crA = xxz_mpo(d)
    nn, ry, cr = random_tt(d, 2, 4, last=B, seed=0)
    out = tt_eigb(d, n, m, ra, crA, cr, ry, 1e-12, 64, B, nswp=10, max_full_size=40)
    H = _dense_heis(d)
    w = np.linalg.eigvalsh(H)[:B]
    assert np.allclose(out["lambda"], w, rtol=1e-10, atol=1e-10)
    X = tt_full_block(d, n, out["ry"], out["cores"])
    assert np.linalg.norm(H @ X - X @ (X.T @ H @ X)) < 1e-7


def test_oracle_eigb_heisen20_against_exact_diagonalisation():
    ed = json.load(open(os.path.join(GOLDEN, "heisen20_ed.json")))["eigenvalues"]
    f = np.load(os.path.join(GOLDEN, "heisen20_sdv.npz"))
    d, B = 20, 5
    r = [int(v) for v in f["r"]]
    n = [2] * d
    nn, ry, cr = random_tt(d, 2, 16, last=B, seed=0)
    out = tt_eigb(d, n, n, r, f["cores"], cr, ry, 1e-8, 64, B, nswp=3, max_full_size=200)
    # ranks capped at 64 limit the accuracy to the truncation error (~1e-7)
    assert np.allclose(out["lambda"], ed[:B], rtol=0, atol=5e-7)
    assert max(out["ry"][:d]) <= 64


def test_laplace_and_amen_operators():
    d, n = 3, 4
    lap = laplace_tt(d, n)
    nn, mm, ra, crA = pack_tt_matrix(lap)
    L1 = 2 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)
    I = np.eye(n)
    ref = np.kron(np.kron(I, I), L1) + np.kron(np.kron(I, L1), I) + np.kron(np.kron(L1, I), I)
    assert np.allclose(tt_matrix_full(d, nn, ra, crA), ref)
    nn, mm, ra, crA = amen_operator(d=3, n=4)
    assert ra == [1, 3, 3, 1]
    full = tt_matrix_full(3, nn, ra, crA)
    g = np.exp(-((np.arange(4) - 1.5) ** 2) / (0.3 * 4) ** 2)
    pot = np.kron(np.kron(np.diag(g), np.diag(g)), np.diag(g))
    assert np.allclose(full, ref + pot)


@pytest.mark.parametrize("shape", [(3, 2, 5, 3, 2, 5, 4, 5), (7, 3, 11, 5, 2, 9, 2, 3)])
def test_zbfun3_transp_is_the_adjoint(shape):
    """zbfun3_transp (ttals.f90:85-108), the norm estimate's second product,
    is the conjugate transpose of zbfun3: <B x, y> = <x, B^H y>, also for
    rectangular local problems (ry != rx, n != m)."""
    rx1, m, rx2, ry1, n, ry2, ra1, ra2 = shape
    rng = np.random.default_rng(sum(shape))
    c = lambda k: rng.standard_normal(k) + 1j * rng.standard_normal(k)  # noqa: E731
    phi1, A, phi2 = c(ry1 * rx1 * ra1), c(ra1 * n * m * ra2), c(rx2 * ra2 * ry2)
    x, y = c(rx1 * m * rx2), c(ry1 * n * ry2)
    bx = ops.bfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, x)
    bhy = ops.zbfun3_transp(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, y)
    assert abs(np.vdot(y, bx) - np.vdot(bhy, x)) <= 1e-12 * np.linalg.norm(bx) * np.linalg.norm(y)
