"""CPU tests: the AMEn oracle (dtt_amen_solve restatement) against dense solves."""
import numpy as np

from oracle.amen import tt_amen_solve, gmres_hh
from oracle.ksl import tt_full
from test_oracle import tt_matrix_full
from ttgpu.operators import amen_operator, random_tt


def test_householder_gmres_solves():
    rng = np.random.default_rng(0)
    N = 80
    M = rng.standard_normal((N, N)) + N * np.eye(N)
    b = rng.standard_normal(N)
    x, cnt, res = gmres_hh(lambda v: M @ v, b, 40, 1e-12, 3)
    assert np.linalg.norm(M @ x - b) <= 1e-10 * np.linalg.norm(b)


def test_amen_oracle_matches_dense_solve():
    d, n = 4, 8
    nn, mm, ra, crA = amen_operator(d=d, n=n)
    _, ry, y = random_tt(d, n, 2, seed=3)
    _, rx, x0 = random_tt(d, n, 2, seed=7)
    out = tt_amen_solve(d, nn, ra, crA, ry, y, rx, x0, 1e-9)
    A = tt_matrix_full(d, nn, ra, crA)
    yf = tt_full(d, nn, ry, y)
    xf = tt_full(d, nn, out["rx"], out["cores"])
    assert np.linalg.norm(A @ xf - yf) <= 1e-9 * np.linalg.norm(yf)
    assert out["res_max"] < 1e-9
