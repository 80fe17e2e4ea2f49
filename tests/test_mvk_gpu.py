"""GPU parity of tt_mvk4 (the AMEn matvec, tt_adapt_als.f90:67-500) with the
oracle: the same ranks, and the same tensor to 1e-10 relative (with the kick
both reach A x to eps; without it both stop at the fixed-rank result)."""
import numpy as np
import pytest

from oracle.mvk import tt_mvk4 as oracle_mvk
from oracle.ksl import tt_full
from test_mvk import tt_matrix_full_rect, random_tt_matrix
from ttgpu.operators import amen_operator, random_tt

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["laplace", "laplace_r1", "rect", "nokick"])
def test_mvk4_matches_oracle(ctx, case):
    import ttgpu
    kick = 5
    if case == "rect":
        d = 4
        n, m, ra, crA = random_tt_matrix(d, 3, 5, 2, seed=4)
        _, rx, x = random_tt(d, 5, 2, seed=1)
        _, ry, y0 = random_tt(d, 3, 2, seed=2)
        eps = 1e-11
    else:
        d, nn = (5, 4) if case != "laplace_r1" else (6, 3)
        n, m, ra, crA = amen_operator(d=d, n=nn)
        _, rx, x = random_tt(d, nn, 3 if case != "laplace_r1" else 4, seed=1)
        _, ry, y0 = random_tt(d, nn, {"laplace": 2, "laplace_r1": 1, "nokick": 8}[case], seed=2)
        eps = 1e-10
        if case == "nokick":
            kick = 0
    cores, ry1 = ttgpu.tt_mvk4(d, n, m, rx, ra, crA, x, y0, ry, eps, 64, kickrank=kick, ctx=ctx)
    ref = oracle_mvk(d, n, m, rx, ra, crA, x, y0, ry, eps, 64, kickrank=kick)
    yg = tt_full(d, n, ry1, cores)
    yo = tt_full(d, n, ref["ry"], ref["cores"])
    if kick > 0:
        ax = tt_matrix_full_rect(d, n, m, ra, crA) @ tt_full(d, m, rx, x)
        assert np.linalg.norm(ax - yg) <= 1e-9 * np.linalg.norm(ax)
    else:
        assert ry1 == ref["ry"]
        assert np.linalg.norm(yg - yo) <= 1e-10 * np.linalg.norm(yo)
