"""Oracle of tt_mvk4 (the AMEn matvec, tt_adapt_als.f90:67-500) against dense
A x on small chains: with the kick (kickrank 5, the reference's default) the
sweeps reach A x to the requested eps; without it the ranks stay at the
start's and the result is the best the fixed ranks allow."""
import numpy as np
import pytest

from oracle.mvk import tt_mvk4
from oracle.ksl import tt_full
from ttgpu.operators import amen_operator, random_tt


def tt_matrix_full_rect(d, n, m, ra, crA):
    off = 0
    M = np.ones((1, 1, 1))
    for k in range(d):
        c = np.asarray(crA[off:off + ra[k] * n[k] * m[k] * ra[k + 1]]).reshape(
            ra[k], n[k], m[k], ra[k + 1], order="F")
        off += c.size
        M = np.einsum("IJa,aijb->IiJjb", M, c)
        s = M.shape
        M = M.reshape(s[0] * s[1], s[2] * s[3], s[4], order="F")
    return M[:, :, 0]


def random_tt_matrix(d, n, m, r, seed):
    rng = np.random.default_rng(seed)
    ra = [1] + [r] * (d - 1) + [1]
    cores = [rng.standard_normal(ra[k] * n * m * ra[k + 1]) for k in range(d)]
    return [n] * d, [m] * d, ra, np.concatenate(cores)


@pytest.mark.parametrize("d,nn,rxr,ryr", [(5, 4, 3, 2), (6, 3, 4, 1)])
def test_mvk_oracle_reaches_ax(d, nn, rxr, ryr):
    n, m, ra, crA = amen_operator(d=d, n=nn)
    _, rx, x = random_tt(d, nn, rxr, seed=1)
    _, ry, y0 = random_tt(d, nn, ryr, seed=2)
    out = tt_mvk4(d, n, m, rx, ra, crA, x, y0, ry, 1e-10, 64)
    A = tt_matrix_full_rect(d, n, m, ra, crA)
    ax = A @ tt_full(d, n, rx, x)
    y = tt_full(d, n, out["ry"], out["cores"])
    assert np.linalg.norm(ax - y) <= 1e-9 * np.linalg.norm(ax)


def test_mvk_oracle_rectangular_operator():
    d = 4
    n, m, ra, crA = random_tt_matrix(d, 3, 5, 2, seed=4)
    _, rx, x = random_tt(d, 5, 2, seed=1)
    _, ry, y0 = random_tt(d, 3, 2, seed=2)
    out = tt_mvk4(d, n, m, rx, ra, crA, x, y0, ry, 1e-11, 64)
    ax = tt_matrix_full_rect(d, n, m, ra, crA) @ tt_full(d, m, rx, x)
    y = tt_full(d, n, out["ry"], out["cores"])
    assert np.linalg.norm(ax - y) <= 1e-9 * np.linalg.norm(ax)


def test_mvk_oracle_fixed_rank_without_kick():
    d, nn = 5, 4
    n, m, ra, crA = amen_operator(d=d, n=nn)
    _, rx, x = random_tt(d, nn, 3, seed=1)
    _, ry, y0 = random_tt(d, nn, 8, seed=2)
    out = tt_mvk4(d, n, m, rx, ra, crA, x, y0, ry, 1e-10, 64, kickrank=0)
    assert out["ry"] == [1, 4, 8, 8, 4, 1]
    ax = tt_matrix_full_rect(d, n, m, ra, crA) @ tt_full(d, n, rx, x)
    y = tt_full(d, n, out["ry"], out["cores"])
    assert np.linalg.norm(ax - y) <= 1e-2 * np.linalg.norm(ax)
