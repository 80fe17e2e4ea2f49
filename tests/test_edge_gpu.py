"""Edge cases of the drivers on the GPU against dense references and the
oracle: ragged mode sizes, a single eigenpair, the two-site chain, the
non-symmetric KSL scheme (typ = 1), and argument errors reported as error
codes (raised as RuntimeError by the binding)."""
import numpy as np
import pytest

from oracle.eigb import tt_eigb as oracle_eigb
from oracle.ksl import ztt_ksl as oracle_ksl, tt_full
from oracle.amen import tt_amen_solve as oracle_amen
from oracle.als import tt_amen_solve as oracle_als
from test_mvk import tt_matrix_full_rect
from ttgpu.operators import xxz_mpo, random_tt

pytestmark = pytest.mark.gpu

RAGGED = [2, 3, 4, 3, 2]


def _pack(cores):
    return np.concatenate([c.ravel(order="F") for c in cores])


def sum_operator(n, mats, shift=0.0):
    """A = sum_k I x .. x M_k x .. x I + shift I as TT-matrix cores of rank 2
    (modes of sizes n, M_k of size n_k x n_k)."""
    d = len(n)
    cores = []
    for k in range(d):
        I = np.eye(n[k])
        Mk = mats[k] + (shift * I if k == 0 else 0)
        if d == 1:
            c = Mk.reshape(1, n[k], n[k], 1)
        elif k == 0:
            c = np.zeros((1, n[k], n[k], 2)); c[0, :, :, 0] = Mk; c[0, :, :, 1] = I
        elif k == d - 1:
            c = np.zeros((2, n[k], n[k], 1)); c[0, :, :, 0] = I; c[1, :, :, 0] = Mk
        else:
            c = np.zeros((2, n[k], n[k], 2))
            c[0, :, :, 0] = I; c[1, :, :, 0] = Mk; c[1, :, :, 1] = I
        cores.append(c)
    ra = [1] + [2] * (d - 1) + [1]
    return ra, _pack(cores)


def random_start(n, r, last, seed):
    rng = np.random.default_rng(seed)
    d = len(n)
    ry = [1] + [r] * (d - 1) + [last]
    return ry, _pack([rng.standard_normal((ry[k], n[k], ry[k + 1])) for k in range(d)])


def test_eigb_ragged_mode_sizes(ctx):
    import ttgpu
    n = RAGGED
    d = len(n)
    rng = np.random.default_rng(1)
    mats = []
    for k in range(d):
        S = rng.standard_normal((n[k], n[k]))
        mats.append(S + S.T)
    ra, crA = sum_operator(n, mats)
    B = 2
    ry, cr = random_start(n, 4, B, seed=2)
    lam, cores, ry_out = ttgpu.tt_eigb(d, n, n, ra, crA, cr, ry, 1e-12, 64, B, nswp=12,
                                       max_full_size=20, ctx=ctx)
    w = np.linalg.eigvalsh(tt_matrix_full_rect(d, n, n, ra, crA))[:B]
    assert np.allclose(lam, w, rtol=1e-10, atol=1e-10)
    ref = oracle_eigb(d, n, n, ra, crA, cr, ry, 1e-12, 64, B, nswp=12, max_full_size=20)
    assert np.allclose(lam, ref["lambda"], rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("d,B", [(2, 1), (8, 1), (2, 2)])
def test_eigb_small_chains_and_single_pair(ctx, d, B):
    import ttgpu
    # with B = 1 the sweep cannot raise ranks (tt_eigb grows them through the
    # block index), so the start has the chain's full ranks
    n, m, ra, crA = xxz_mpo(d, delta=0.8)
    _, ry, cr = random_tt(d, 2, 16, last=B, seed=d + B)
    lam, _, _ = ttgpu.tt_eigb(d, n, m, ra, crA, cr, ry, 1e-12, 64, B, nswp=10, max_full_size=8,
                              ctx=ctx)
    w = np.linalg.eigvalsh(tt_matrix_full_rect(d, n, m, ra, crA))[:B]
    assert np.allclose(lam, w, rtol=1e-10, atol=1e-12)


def test_eigb_argument_errors(ctx):
    import ttgpu
    d, B = 6, 2
    n, m, ra, crA = xxz_mpo(d)
    _, ry, cr = random_tt(d, 2, 4, last=B, seed=0)
    with pytest.raises(RuntimeError):        # last rank must be B
        ttgpu.tt_eigb(d, n, m, ra, crA, cr, ry, 1e-8, 16, B + 1, ctx=ctx)
    bad = list(ra)
    bad[0] = 2
    with pytest.raises(RuntimeError):        # boundary ranks must be 1
        ttgpu.tt_eigb(d, n, m, bad, crA, cr, ry, 1e-8, 16, B, ctx=ctx)
    # the context stays usable after the errors
    lam, _, _ = ttgpu.tt_eigb(d, n, m, ra, crA, cr, ry, 1e-10, 16, B, ctx=ctx)
    assert np.all(np.isfinite(lam))


def _complex_ragged_operator(n, seed):
    rng = np.random.default_rng(seed)
    mats = [1j * (lambda S: S + S.T)(rng.standard_normal((k, k))) for k in n]
    d = len(n)
    cores = []
    for k in range(d):
        I = np.eye(n[k])
        if k == 0:
            c = np.zeros((1, n[k], n[k], 2), complex); c[0, :, :, 0] = mats[k]; c[0, :, :, 1] = I
        elif k == d - 1:
            c = np.zeros((2, n[k], n[k], 1), complex); c[0, :, :, 0] = I; c[1, :, :, 0] = mats[k]
        else:
            c = np.zeros((2, n[k], n[k], 2), complex)
            c[0, :, :, 0] = I; c[1, :, :, 0] = mats[k]; c[1, :, :, 1] = I
        cores.append(c)
    return [1] + [2] * (d - 1) + [1], _pack(cores)


@pytest.mark.parametrize("typ", [1, 2])
def test_ksl_ragged_modes_and_scheme(ctx, typ):
    """typ 1 (plain KSL) and 2 (symmetric) on ragged modes against the oracle."""
    import ttgpu
    n = RAGGED
    d = len(n)
    ra, crA = _complex_ragged_operator(n, 4)
    rng = np.random.default_rng(5)
    ry = [1, 2, 3, 3, 2, 1]
    y = _pack([rng.standard_normal((ry[k], n[k], ry[k + 1])) +
               1j * rng.standard_normal((ry[k], n[k], ry[k + 1])) for k in range(d)])
    tau = 0.02
    cores, ry1 = ttgpu.ztt_ksl(d, n, n, ra, crA, y, ry, tau, 10, typ=typ, nsteps=2, ctx=ctx)
    c, r = y, list(ry)
    for _ in range(2):
        out = oracle_ksl(d, n, n, ra, crA, c, r, tau, 10, typ=typ)
        c, r = out["cores"], out["ry"]
    assert ry1 == r
    a, b = tt_full(d, n, ry1, cores), tt_full(d, n, r, c)
    assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(b)


def _spd_ragged(n, seed):
    rng = np.random.default_rng(seed)
    mats = []
    for k in n:
        L = 2 * np.eye(k) - np.eye(k, k=1) - np.eye(k, k=-1)
        mats.append(L + 0.1 * np.diag(rng.random(k)))
    return sum_operator(n, mats, shift=0.5)


def test_amen_solvers_ragged_modes(ctx):
    """dtt_amen_solve and tt_amen_solve on ragged modes: the residual against
    the dense operator meets the tolerance and both agree with the oracles."""
    import ttgpu
    n = RAGGED
    d = len(n)
    ra, crA = _spd_ragged(n, 6)
    ry, y = random_start(n, 2, 1, seed=7)
    rx, x0 = random_start(n, 2, 1, seed=8)
    A = tt_matrix_full_rect(d, n, n, ra, crA)
    yf = tt_full(d, n, ry, y)
    tol = 1e-10
    c1, r1 = ttgpu.dtt_amen_solve(d, n, n, ry, ra, crA, y, x0, rx, tol, ctx=ctx)
    x1 = tt_full(d, n, r1, c1)
    assert np.linalg.norm(A @ x1 - yf) <= tol * np.linalg.norm(yf)
    ref = oracle_amen(d, n, ra, crA, ry, y, rx, x0, tol)
    assert np.linalg.norm(x1 - tt_full(d, n, ref["rx"], ref["cores"])) <= 1e-8 * np.linalg.norm(x1)
    c2, r2 = ttgpu.tt_amen_solve(d, n, n, ry, ra, crA, y, x0, rx, tol, ctx=ctx)
    x2 = tt_full(d, n, r2, c2)
    assert np.linalg.norm(A @ x2 - yf) <= tol * np.linalg.norm(yf)
    ref2 = oracle_als(d, n, n, ry, ra, crA, y, x0, rx, tol)
    assert np.linalg.norm(x2 - tt_full(d, n, ref2["rx"], ref2["cores"])) <= 1e-8 * np.linalg.norm(x2)
