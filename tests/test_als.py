"""CPU tests of the oracle of tt_amen_solve (tt_adapt_als.f90:513-1132)
against dense solves, and of its incremental Cholesky kick (duchol_fort)."""
import numpy as np
import pytest

from oracle.als import tt_amen_solve, uchol
from oracle.ksl import tt_full
from test_oracle import tt_matrix_full
from ttgpu.operators import amen_operator, random_tt


@pytest.mark.parametrize("d,n,ryr,rxr,eps", [(4, 8, 2, 2, 1e-9), (5, 4, 2, 3, 1e-10)])
def test_als_oracle_matches_dense_solve(d, n, ryr, rxr, eps):
    nn, mm, ra, crA = amen_operator(d=d, n=n)
    _, ry, y = random_tt(d, n, ryr, seed=3)
    _, rx, x0 = random_tt(d, n, rxr, seed=7)
    out = tt_amen_solve(d, nn, mm, ry, ra, crA, y, x0, rx, eps)
    A = tt_matrix_full(d, nn, ra, crA)
    yf = tt_full(d, nn, ry, y)
    xf = tt_full(d, nn, out["rx"], out["cores"])
    assert np.linalg.norm(A @ xf - yf) <= eps * np.linalg.norm(yf)
    assert out["res_max"] < eps


def test_uchol_spans_the_dominant_directions():
    rng = np.random.default_rng(4)
    n, m = 60, 9
    B = rng.standard_normal((n, 3)) @ np.diag([10.0, 5.0, 2.0]) @ rng.standard_normal((3, m))
    B += 1e-3 * rng.standard_normal((n, m))
    for trans, dA in (("T", B.ravel(order="F")), ("N", B.T.ravel(order="F"))):
        du, k = uchol(trans, m, n, dA, 3)
        assert k == 3
        assert np.allclose(du.T @ du, np.eye(3), atol=1e-10)
        U = np.linalg.svd(B)[0][:, :3]
        # the three dominant left singular directions lie in span(du)
        assert np.linalg.norm(U - du @ (du.T @ U)) < 1e-2
