"""GPU parity of tt_amen_solve (tt_adapt_als.f90:513-1132) against the oracle.

Bar: the GPU solution meets the reference's stopping test (residual below
eps against the dense operator), and the GPU and oracle solutions agree to
the accuracy both are asked for (relative 2-norm difference of the full
tensors below 100 eps)."""
import numpy as np
import pytest

from oracle.als import tt_amen_solve as oracle_als
from oracle.ksl import tt_full
from test_oracle import tt_matrix_full
from ttgpu.operators import amen_operator, random_tt

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("d,n,ryr,rxr,eps", [(4, 8, 2, 2, 1e-9), (5, 4, 2, 3, 1e-10),
                                             (5, 6, 3, 2, 1e-8)])
def test_als_matches_dense_and_oracle(ctx, d, n, ryr, rxr, eps):
    import ttgpu
    nn, mm, ra, crA = amen_operator(d=d, n=n)
    _, ry, y = random_tt(d, n, ryr, seed=3)
    _, rx, x0 = random_tt(d, n, rxr, seed=7)
    cores, rx1 = ttgpu.tt_amen_solve(d, nn, mm, ry, ra, crA, y, x0, rx, eps, ctx=ctx)
    st = ctx.stats()
    A = tt_matrix_full(d, nn, ra, crA)
    yf = tt_full(d, nn, ry, y)
    xg = tt_full(d, nn, rx1, cores)
    assert np.linalg.norm(A @ xg - yf) <= eps * np.linalg.norm(yf)
    assert st["res"] < eps
    ref = oracle_als(d, nn, mm, ry, ra, crA, y, x0, rx, eps)
    xo = tt_full(d, nn, ref["rx"], ref["cores"])
    assert np.linalg.norm(xg - xo) <= 100 * eps * np.linalg.norm(xo)


def test_als_without_kick_and_unsupported_prec(ctx):
    import ttgpu
    d, n, eps = 4, 6, 1e-9
    nn, mm, ra, crA = amen_operator(d=d, n=n)
    _, ry, y = random_tt(d, n, 2, seed=5)
    _, rx, x0 = random_tt(d, n, 36, seed=6)       # full ranks: no kick needed
    cores, rx1 = ttgpu.tt_amen_solve(d, nn, mm, ry, ra, crA, y, x0, rx, eps, kickrank=0,
                                     nswp=30, ctx=ctx)
    A = tt_matrix_full(d, nn, ra, crA)
    yf = tt_full(d, nn, ry, y)
    xg = tt_full(d, nn, rx1, cores)
    assert np.linalg.norm(A @ xg - yf) <= 10 * eps * np.linalg.norm(yf)
    with pytest.raises(RuntimeError):
        ttgpu.tt_amen_solve(d, nn, mm, ry, ra, crA, y, x0, rx, eps, prec="x", ctx=ctx)


@pytest.mark.parametrize("prec", ["c", "l", "r"])
def test_als_block_jacobi_preconditioners(ctx, prec):
    """prec 'c' / 'l' / 'r' (djac_gen / djac_apply, right preconditioning):
    the GPU meets the stopping test against the dense operator and agrees with
    the oracle run with the same preconditioner."""
    import ttgpu
    d, n, eps = 5, 6, 1e-9
    nn, mm, ra, crA = amen_operator(d=d, n=n)
    _, ry, y = random_tt(d, n, 2, seed=3)
    _, rx, x0 = random_tt(d, n, 2, seed=7)
    cores, rx1 = ttgpu.tt_amen_solve(d, nn, mm, ry, ra, crA, y, x0, rx, eps, prec=prec, ctx=ctx)
    A = tt_matrix_full(d, nn, ra, crA)
    yf = tt_full(d, nn, ry, y)
    xg = tt_full(d, nn, rx1, cores)
    assert np.linalg.norm(A @ xg - yf) <= eps * np.linalg.norm(yf)
    ref = oracle_als(d, nn, mm, ry, ra, crA, y, x0, rx, eps, prec=prec)
    xo = tt_full(d, nn, ref["rx"], ref["cores"])
    assert np.linalg.norm(xg - xo) <= 100 * eps * np.linalg.norm(xo)
