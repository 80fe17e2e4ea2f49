"""GPU parity of the AMEn solve (ttamen algorithm) against the oracle.

Bar: the residual of the GPU solution below the requested tolerance (the
reference's stopping test), and the GPU and oracle solutions equal to the
accuracy both are asked for."""
import numpy as np
import pytest

from oracle.amen import tt_amen_solve as oracle_amen
from oracle.ksl import tt_full
from test_oracle import tt_matrix_full
from ttgpu.operators import amen_operator, random_tt

pytestmark = pytest.mark.gpu


def tt_dot(n, r1, c1, r2, c2):
    o1 = o2 = 0
    T = np.ones((1, 1))
    for k in range(len(n)):
        a = c1[o1:o1 + r1[k] * n[k] * r1[k + 1]].reshape(r1[k], n[k], r1[k + 1], order="F")
        b = c2[o2:o2 + r2[k] * n[k] * r2[k + 1]].reshape(r2[k], n[k], r2[k + 1], order="F")
        o1 += a.size; o2 += b.size
        T = np.einsum("ab,aic,bid->cd", T, a, b)
    return T.item()


def tt_rel_diff(n, r1, c1, r2, c2):
    aa, bb, ab = tt_dot(n, r1, c1, r1, c1), tt_dot(n, r2, c2, r2, c2), tt_dot(n, r1, c1, r2, c2)
    return np.sqrt(max(aa + bb - 2 * ab, 0.0) / bb)


@pytest.mark.parametrize("d,n,ryr,rxr", [(4, 8, 2, 2), (5, 6, 3, 2)])
def test_amen_dense_check(ctx, d, n, ryr, rxr):
    import ttgpu
    tol = 1e-9
    nn, mm, ra, crA = amen_operator(d=d, n=n)
    _, ry, y = random_tt(d, n, ryr, seed=3)
    _, rx, x0 = random_tt(d, n, rxr, seed=7)
    cores, rx1 = ttgpu.dtt_amen_solve(d, nn, mm, ry, ra, crA, y, x0, rx, tol, ctx=ctx)
    A = tt_matrix_full(d, nn, ra, crA)
    yf = tt_full(d, nn, ry, y)
    xf = tt_full(d, nn, rx1, cores)
    assert np.linalg.norm(A @ xf - yf) <= tol * np.linalg.norm(yf)
    ref = oracle_amen(d, nn, ra, crA, ry, y, rx, x0, tol)
    xo = tt_full(d, nn, ref["rx"], ref["cores"])
    assert np.linalg.norm(xf - xo) <= 1e-8 * np.linalg.norm(xo)


@pytest.mark.parametrize("d,n,ryr,rxr", [(4, 8, 2, 2), (5, 6, 3, 2), (3, 16, 2, 3)])
def test_amen_chosen_dense_check(ctx, d, n, ryr, rxr):
    """Chosen form (split-precision GMRES inside FP64 iterative refinement):
    the FP64 residual against the dense operator meets the same tolerance,
    and the solution equals the oracle's to 1e-8."""
    import ttgpu
    tol = 1e-9
    nn, mm, ra, crA = amen_operator(d=d, n=n)
    _, ry, y = random_tt(d, n, ryr, seed=3)
    _, rx, x0 = random_tt(d, n, rxr, seed=7)
    cores, rx1 = ttgpu.dtt_amen_solve(d, nn, mm, ry, ra, crA, y, x0, rx, tol, method="split",
                                      ctx=ctx)
    A = tt_matrix_full(d, nn, ra, crA)
    yf = tt_full(d, nn, ry, y)
    xf = tt_full(d, nn, rx1, cores)
    assert np.linalg.norm(A @ xf - yf) <= tol * np.linalg.norm(yf)
    ref = oracle_amen(d, nn, ra, crA, ry, y, rx, x0, tol)
    xo = tt_full(d, nn, ref["rx"], ref["cores"])
    assert np.linalg.norm(xf - xo) <= 1e-8 * np.linalg.norm(xo)


def test_amen_workload_family(ctx):
    """Laplacian + Gaussian potential (rank 3), rhs rank 4, d=6, n=16: the
    reference's algorithm needs many sweeps here (GMRES(40) x 2 without a
    preconditioner), so both solvers run six sweeps and the states must
    agree: same ranks, same iterate, same largest local residual."""
    import ttgpu
    d, n, tol, nswp = 6, 16, 1e-8, 6
    nn, mm, ra, crA = amen_operator(d=d, n=n)
    _, ry, y = random_tt(d, n, 4, seed=3)
    _, rx, x0 = random_tt(d, n, 2, seed=5)
    cores, rx1 = ttgpu.dtt_amen_solve(d, nn, mm, ry, ra, crA, y, x0, rx, tol, nswp=nswp, ctx=ctx)
    st = ctx.stats()
    ref = oracle_amen(d, nn, ra, crA, ry, y, rx, x0, tol, nswp=nswp)
    assert rx1 == ref["rx"]
    assert st["sweeps"] == ref["sweeps"]
    assert abs(st["res"] - ref["res_max"]) <= 1e-3 * ref["res_max"]
    assert tt_rel_diff(nn, rx1, cores, ref["rx"], ref["cores"]) < 1e-6


def test_amen_config_size_six_sweeps(ctx):
    """The AMEn workload at its configured size: d=10, n=64, Laplacian +
    exp(-|i-c|^2/sigma^2) (rank 3), rhs rank 4, tol 1e-9, ranks up to 128.
    The oracle needs minutes to converge at these ranks, so both run six
    sweeps from the same start (ranks reach 26) and the states must agree:
    same ranks, same sweep count, same largest local residual, same iterate."""
    import ttgpu
    from ttgpu.operators import tt_rel_diff as qr_rel_diff
    d, n, tol, nswp = 10, 64, 1e-9, 6
    nn, mm, ra, crA = amen_operator(d=d, n=n)
    _, ry, y = random_tt(d, n, 4, seed=3)
    _, rx, x0 = random_tt(d, n, 2, seed=7)
    cores, rx1 = ttgpu.dtt_amen_solve(d, nn, mm, ry, ra, crA, y, x0, rx, tol, rmax=128,
                                      nswp=nswp, ctx=ctx)
    st = ctx.stats()
    ref = oracle_amen(d, nn, ra, crA, ry, y, rx, x0, tol, nswp=nswp)
    assert rx1 == ref["rx"]
    assert st["sweeps"] == ref["sweeps"]
    assert abs(st["res"] - ref["res_max"]) <= 1e-3 * ref["res_max"]
    assert qr_rel_diff(d, nn, rx1, cores, ref["rx"], ref["cores"]) < 1e-6
