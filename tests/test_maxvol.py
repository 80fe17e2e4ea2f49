"""maxvol oracle (maxvol.f90:27-119) against its contract: every entry of
Z = A inv(A[p, :]) is at most 1 + tol in modulus, Z[p, :] = I, and the
selected rows have a volume no smaller than the LU start's."""
import numpy as np
import pytest

from oracle.maxvol import maxvol, maxvol_contract


@pytest.mark.parametrize("m,n,seed", [(50, 5, 0), (200, 20, 1), (512, 64, 2), (8, 8, 3),
                                      (1000, 1, 4), (33, 32, 5)])
def test_maxvol_contract(m, n, seed):
    a = np.random.default_rng(seed).standard_normal((m, n))
    p, z, it = maxvol(a)
    assert len(set(p.tolist())) == n and p.min() >= 0 and p.max() < m
    assert maxvol_contract(a, p, z)
    assert 1 <= it <= 1024


def test_maxvol_square_selects_every_row():
    a = np.random.default_rng(7).standard_normal((12, 12))
    p, z, _ = maxvol(a)
    assert sorted(p.tolist()) == list(range(12))
    assert np.allclose(z[p], np.eye(12))


def test_maxvol_finds_the_planted_rows():
    # rows of a scaled identity dominate: maxvol must select them
    rng = np.random.default_rng(8)
    a = 0.1 * rng.standard_normal((300, 6))
    rows = [17, 250, 3, 99, 180, 42]
    for j, r in enumerate(rows):
        a[r, :] = 0.0
        a[r, j] = 10.0
    p, z, _ = maxvol(a)
    assert sorted(p.tolist()) == sorted(rows)


def test_maxvol_tolerance_bounds_the_coefficients():
    a = np.random.default_rng(9).standard_normal((400, 10))
    for tol in (1e-2, 0.5):
        p, z, _ = maxvol(a, tol=tol)
        assert np.max(np.abs(z)) <= 1 + tol + 1e-12
