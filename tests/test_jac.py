"""Oracle of the block-Jacobi preconditioners (djac_gen / djac_apply,
tt_linalg.f90:363-531) against a literal transcription of the reference's
steps (dtransp, strided diagonal copies, dgemm, dperm1324, dgesv per block),
and the preconditioned tt_amen_solve oracle against a dense solve."""
import numpy as np
import pytest

from oracle.jac import jac_gen, jac_apply, jac_size
from oracle.ops import F, flat, dtransp
from oracle.als import tt_amen_solve as oracle_als
from oracle.ksl import tt_full
from test_oracle import tt_matrix_full
from ttgpu.operators import amen_operator, random_tt


def _perm1324(n1, n2, n3, n4, a):
    return flat(F(a, n1, n2, n3, n4).transpose(0, 2, 1, 3))


def _diag_copies(phi, r, ra, first_stride):
    out = np.zeros(r * ra)
    for i in range(ra):
        out[i * r:(i + 1) * r] = phi[i * first_stride:][::r + 1][:r]
    return out


def _literal_gen(p, rx1, n, rx2, ra1, ra2, phi1, A, phi2):
    def inv_blocks(w, k, nb):
        return np.concatenate([flat(np.linalg.solve(F(w[q * k * k:(q + 1) * k * k], k, k),
                                                    np.eye(k))) for q in range(nb)])
    d1 = _diag_copies(phi1, rx1, ra1, rx1 * rx1)
    if p == "c":
        w2 = _diag_copies(dtransp(rx2 * ra2, rx2, phi2), rx2, ra2, rx2 * rx2)
        j = F(d1, rx1, ra1) @ F(A, ra1, n * n * ra2)
        w = F(flat(j), rx1 * n * n, ra2) @ F(w2, rx2, ra2).T
        return inv_blocks(dtransp(rx1, n * n * rx2, flat(w)), n, rx2 * rx1)
    if p == "l":
        w2 = _diag_copies(dtransp(rx2 * ra2, rx2, phi2), rx2, ra2, rx2 * rx2)
        w1 = F(phi1, rx1 * rx1, ra1) @ F(A, ra1, n * n * ra2)
        jj = _perm1324(rx1, rx1, n, n * ra2, flat(w1))
        w = F(jj, rx1 * n * rx1 * n, ra2) @ F(w2, rx2, ra2).T
        return inv_blocks(flat(w), rx1 * n, rx2)
    w2 = dtransp(rx2 * ra2, rx2, phi2)
    j = F(d1, rx1, ra1) @ F(A, ra1, n * n * ra2)
    w = F(flat(j), rx1 * n * n, ra2) @ F(w2, rx2 * rx2, ra2).T
    w1 = dtransp(rx1, n * rx2 * n * rx2, _perm1324(rx1 * n, n, rx2, rx2, flat(w)))
    return inv_blocks(w1, n * rx2, rx1)


def _literal_apply(p, rx1, n, rx2, J, x):
    if p == "c":
        w1 = dtransp(rx1, n * rx2, x)
        y = np.concatenate([F(J[i * n * n:(i + 1) * n * n], n, n) @ w1[i * n:(i + 1) * n]
                            for i in range(rx2 * rx1)])
        return dtransp(n * rx2, rx1, y)
    if p == "l":
        k = rx1 * n
        return np.concatenate([F(J[i * k * k:(i + 1) * k * k], k, k) @ x[i * k:(i + 1) * k]
                               for i in range(rx2)])
    k = n * rx2
    w1 = dtransp(rx1, k, x)
    y = np.concatenate([F(J[i * k * k:(i + 1) * k * k], k, k) @ w1[i * k:(i + 1) * k]
                        for i in range(rx1)])
    return dtransp(k, rx1, y)


@pytest.mark.parametrize("p", ["c", "l", "r"])
@pytest.mark.parametrize("shape", [(3, 4, 2, 2, 3), (2, 3, 5, 3, 1), (4, 2, 3, 1, 2)])
def test_jac_oracle_matches_the_reference_steps(p, shape):
    rx1, n, rx2, ra1, ra2 = shape
    rng = np.random.default_rng(sum(shape))
    phi1 = rng.standard_normal(rx1 * rx1 * ra1)
    phi2 = rng.standard_normal(rx2 * ra2 * rx2)
    A = rng.standard_normal(ra1 * n * n * ra2)
    J = jac_gen(p, rx1, n, rx2, ra1, ra2, phi1, A, phi2)
    assert J.size == jac_size(p, rx1, n, rx2)
    Jl = _literal_gen(p, rx1, n, rx2, ra1, ra2, phi1, A, phi2)
    assert np.abs(J - Jl).max() <= 1e-10 * np.abs(Jl).max()
    x = rng.standard_normal(rx1 * n * rx2)
    y = jac_apply(p, rx1, n, rx2, J, x)
    yl = _literal_apply(p, rx1, n, rx2, Jl, x)
    assert np.linalg.norm(y - yl) <= 1e-10 * np.linalg.norm(yl)


def test_jac_inverts_the_kept_part():
    """With rx1 = rx2 = 1 every preconditioner keeps the whole local operator,
    so P is its inverse."""
    rng = np.random.default_rng(0)
    n, ra1, ra2 = 5, 2, 3
    phi1 = rng.standard_normal(ra1)
    phi2 = rng.standard_normal(ra2)
    A = rng.standard_normal(ra1 * n * n * ra2)
    B = np.einsum("a,aijc,c->ij", phi1, F(A, ra1, n, n, ra2), phi2)
    for p in "clr":
        J = F(jac_gen(p, 1, n, 1, ra1, ra2, phi1, A, phi2), n, n)
        assert np.allclose(J @ B, np.eye(n), atol=1e-10)


@pytest.mark.parametrize("prec", ["c", "l", "r"])
def test_als_oracle_with_preconditioner_matches_dense(prec):
    d, n, eps = 4, 6, 1e-9
    nn, mm, ra, crA = amen_operator(d=d, n=n)
    _, ry, y = random_tt(d, n, 2, seed=3)
    _, rx, x0 = random_tt(d, n, 2, seed=7)
    out = oracle_als(d, nn, mm, ry, ra, crA, y, x0, rx, eps, prec=prec)
    A = tt_matrix_full(d, nn, ra, crA)
    yf = tt_full(d, nn, ry, y)
    x = tt_full(d, nn, out["rx"], out["cores"])
    assert np.linalg.norm(A @ x - yf) <= eps * np.linalg.norm(yf)
