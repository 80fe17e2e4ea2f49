"""CPU tests: the KSL oracle (ztt_ksl, Expokit, normest) pinned against the
reference's closed-form fixture and dense references."""
import os

import numpy as np
import scipy.linalg as sla

from conftest import GOLDEN
from oracle.expokit import zgpadm, zexp_mv
from oracle.ksl import ztt_ksl, tt_full
from oracle.normest import znormest, Seed, unit_randoms


def load_dat(name):
    D = dict(np.load(os.path.join(GOLDEN, name)))
    return (int(D["d"]), [int(v) for v in D["n"]], [int(v) for v in D["m"]],
            [int(v) for v in D["ra"]], [int(v) for v in D["ry"]], D["crA"], D["crY"],
            float(D["tau"]))


def test_eye_fixture_is_exp_i_tau():
    """test_eye_ksl.dat: A = i*I, one step must return exp(i tau) y0."""
    d, n, m, ra, ry, crA, crY, tau = load_dat("test_eye_ksl_dat.npz")
    out = ztt_ksl(d, n, m, ra, crA, crY, ry, tau, 150)
    x0 = tt_full(d, n, ry, crY)
    x1 = tt_full(d, n, out["ry"], out["cores"])
    assert np.linalg.norm(x1 - np.exp(1j * tau) * x0) <= 1e-12 * np.linalg.norm(x0)


def separable(d, nn, seed):
    rng = np.random.default_rng(seed)
    a = [rng.standard_normal((nn, nn)) + 1j * rng.standard_normal((nn, nn)) for _ in range(d)]
    I = np.eye(nn)
    cores = []
    for k in range(d):
        if k == 0:
            c = np.zeros((1, nn, nn, 2), complex); c[0, :, :, 0] = a[k]; c[0, :, :, 1] = I
        elif k == d - 1:
            c = np.zeros((2, nn, nn, 1), complex); c[0, :, :, 0] = I; c[1, :, :, 0] = a[k]
        else:
            c = np.zeros((2, nn, nn, 2), complex)
            c[0, :, :, 0] = I; c[1, :, :, 0] = a[k]; c[1, :, :, 1] = I
        cores.append(c)
    crA = np.concatenate([c.ravel(order="F") for c in cores])
    ra = [1] + [2] * (d - 1) + [1]
    full = np.zeros((nn ** d, nn ** d), complex)
    for k in range(d):
        mats = [I] * d
        mats[k] = a[k]
        M = mats[d - 1]
        for q in range(d - 2, -1, -1):
            M = np.kron(M, mats[q])
        full += M
    y = np.concatenate([rng.standard_normal(nn) + 1j * rng.standard_normal(nn) for _ in range(d)])
    return crA, ra, full, y


def test_separable_rank1_is_exact():
    """For A = sum_k a_k (Kronecker sum) and a rank-1 start the exact solution
    stays rank 1, so the projector-splitting step is exact up to Expokit."""
    d, nn, tau = 5, 3, 0.05
    crA, ra, full, y = separable(d, nn, 0)
    out = ztt_ksl(d, [nn] * d, [nn] * d, ra, crA, y, [1] * (d + 1), tau, 10)
    x0 = tt_full(d, [nn] * d, [1] * (d + 1), y)
    x1 = tt_full(d, [nn] * d, out["ry"], out["cores"])
    ref = sla.expm(tau * full) @ x0
    assert np.linalg.norm(x1 - ref) <= 1e-10 * np.linalg.norm(ref)


def test_zgpadm_and_zexp_mv_against_expm():
    rng = np.random.default_rng(4)
    for mdim in (3, 7, 10):
        H = rng.standard_normal((mdim, mdim)) + 1j * rng.standard_normal((mdim, mdim))
        for t in (0.01, -0.3, 2.0):
            assert np.allclose(zgpadm(6, mdim, t, H), sla.expm(t * H), rtol=1e-12, atol=1e-12)
    N = 60
    A = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) / np.sqrt(N)
    v = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    w, st = zexp_mv(N, 8, 0.7, v, 1e-10, np.abs(A).sum(axis=0).max(), lambda x: A @ x)
    ref = sla.expm(0.7 * A) @ v
    assert np.linalg.norm(w - ref) <= 1e-8 * np.linalg.norm(ref)
    assert st["nstep"] >= 1


def test_normest_is_a_lower_bound_close_to_the_1norm():
    rng = np.random.default_rng(5)
    for N in (1, 3, 17, 120):
        A = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
        est = znormest(N, 4, lambda X: A @ X, lambda X: A.conj().T @ X, Seed())
        true = np.abs(A).sum(axis=0).max()
        assert est <= true * (1 + 1e-12)
        assert est >= 0.3 * true


def test_unit_randoms_stream():
    z = unit_randoms(0, 5)
    assert np.allclose(np.abs(z), 1.0)
    assert np.allclose(unit_randoms(2, 3), z[2:5])


def diag_sum_operator(d, nn, seed, complex_=True):
    """A = sum_k I x .. x diag(a_k) x .. x I as diagonal cores A(a1, i, a2)
    of rank 2, and a rank-1 start: ztt_diag_ksl is exact on it."""
    rng = np.random.default_rng(seed)
    a = [rng.standard_normal(nn) + (1j * rng.standard_normal(nn) if complex_ else 0)
         for _ in range(d)]
    ra = [1] + [2] * (d - 1) + [1]
    cores = []
    for k in range(d):
        c = np.zeros((ra[k], nn, ra[k + 1]), complex if complex_ else float)
        if k == 0:
            c[0, :, 0] = a[k]; c[0, :, 1] = 1
        elif k == d - 1:
            c[0, :, 0] = 1; c[1, :, 0] = a[k]
        else:
            c[0, :, 0] = 1; c[1, :, 0] = a[k]; c[1, :, 1] = 1
        cores.append(c.ravel(order="F"))
    y0 = [rng.standard_normal(nn) + (1j * rng.standard_normal(nn) if complex_ else 0)
          for _ in range(d)]
    return ra, np.concatenate(cores), a, y0


def test_diag_ksl_oracle_is_exact_on_separable_diagonal_operators():
    from oracle.ksl import ztt_diag_ksl
    d, nn, tau = 5, 4, 0.1
    ra, crA, a, y0 = diag_sum_operator(d, nn, 0)
    out = ztt_diag_ksl(d, [nn] * d, ra, crA, np.concatenate(y0), [1] * (d + 1), tau, 10)
    ex = y0[0] * np.exp(tau * a[0])
    for k in range(1, d):
        ex = np.kron(y0[k] * np.exp(tau * a[k]), ex)
    x1 = tt_full(d, [nn] * d, out["ry"], out["cores"])
    assert np.linalg.norm(x1 - ex) <= 1e-12 * np.linalg.norm(ex)


def scaled_identity(d, nn, c):
    """c * I as a rank-1 TT-matrix (real)."""
    cores = []
    for k in range(d):
        core = np.eye(nn).reshape(1, nn, nn, 1) * (c if k == 0 else 1.0)
        cores.append(core.ravel(order="F"))
    return [1] * (d + 1), np.concatenate(cores)


def test_tt_ksl_real_scaled_identity_is_exact():
    """The real tt_ksl scheme on A = c I: every K-step multiplies by
    exp(c tau/2) and every S-step by exp(-c tau/2); d + d K-steps against
    (d-1) + (d-1) S-steps leave exp(c tau) y0 for any start of any rank."""
    from oracle.ksl import tt_ksl_real
    d, nn, c, tau = 5, 3, 0.7, 0.3
    ra, crA = scaled_identity(d, nn, c)
    ry = [1, 3, 4, 4, 3, 1]
    rng = np.random.default_rng(1)
    y = np.concatenate([rng.standard_normal(ry[k] * nn * ry[k + 1]) for k in range(d)])
    out = tt_ksl_real(d, [nn] * d, [nn] * d, ra, crA, y, ry, tau, 10)
    x0 = tt_full(d, [nn] * d, ry, y)
    x1 = tt_full(d, [nn] * d, out["ry"], out["cores"])
    assert out["ry"] == ry
    assert np.linalg.norm(x1 - np.exp(c * tau) * x0) <= 1e-12 * np.linalg.norm(x0)


def test_tt_ksl_real_is_second_order_on_separable_operators():
    """The real scheme's forward half sweep does the S-step of each bond
    before the K-step of the core on its left, so unlike ztt_ksl it is not
    exact on a Kronecker sum with a rank-1 start.  Its one-step error is
    O(tau^3): halving tau divides it by about 8."""
    from oracle.ksl import tt_ksl_real
    d, nn = 5, 3
    crA, ra, full, y = separable(d, nn, 0)
    crA, full, y = crA.real.copy(), full.real.copy(), y.real.copy()
    x0 = tt_full(d, [nn] * d, [1] * (d + 1), y)
    errs = []
    for tau in (0.05, 0.025):
        out = tt_ksl_real(d, [nn] * d, [nn] * d, ra, crA, y, [1] * (d + 1), tau, 10)
        x1 = tt_full(d, [nn] * d, out["ry"], out["cores"])
        ref = sla.expm(tau * full) @ x0
        errs.append(np.linalg.norm(x1 - ref) / np.linalg.norm(ref))
    assert errs[0] < 1e-3
    assert 6.0 < errs[0] / errs[1] < 10.0


def test_tt_ksl_real_single_core_is_a_half_step():
    """d = 1: the backward K-step is never stored, so one call returns
    exp(tau/2 A) y0."""
    from oracle.ksl import tt_ksl_real
    rng = np.random.default_rng(2)
    nn, tau = 6, 0.2
    a = rng.standard_normal((nn, nn))
    y = rng.standard_normal(nn)
    out = tt_ksl_real(1, [nn], [nn], [1, 1], a.ravel(order="F"), y, [1, 1], tau, 10)
    ref = sla.expm(tau / 2 * a) @ y
    assert np.linalg.norm(out["cores"] - ref) <= 1e-10 * np.linalg.norm(ref)


def test_tt_ksl_real_rejects_ranks_the_qr_would_cut():
    from oracle.ksl import tt_ksl_real
    import pytest
    d, nn = 3, 2
    ra, crA = scaled_identity(d, nn, 1.0)
    ry = [1, 2, 4, 1]            # r_2 = 4 > n_3 r_3 = 2
    y = np.ones(sum(ry[k] * nn * ry[k + 1] for k in range(d)))
    with pytest.raises(ValueError):
        tt_ksl_real(d, [nn] * d, [nn] * d, ra, crA, y, ry, 0.1, 10)


def test_tt_ksl_real_ragged_modes_scaled_identity():
    """c I on ragged modes, with a start rank the first QR cuts: still
    exp(c tau) times the start."""
    from oracle.ksl import tt_ksl_real
    n, c, tau = [2, 3, 4, 2], -0.4, 0.25
    cores = [np.eye(nk).reshape(1, nk, nk, 1) * (c if k == 0 else 1.0) for k, nk in enumerate(n)]
    crA = np.concatenate([x.ravel(order="F") for x in cores])
    ry = [1, 4, 3, 2, 1]
    rng = np.random.default_rng(12)
    y = np.concatenate([rng.standard_normal(ry[k] * n[k] * ry[k + 1]) for k in range(4)])
    out = tt_ksl_real(4, n, n, [1] * 5, crA, y, ry, tau, 10)
    assert out["ry"] == [1, 2, 3, 2, 1]
    x0 = tt_full(4, n, ry, y)
    x1 = tt_full(4, n, out["ry"], out["cores"])
    assert np.linalg.norm(x1 - np.exp(c * tau) * x0) <= 1e-12 * np.linalg.norm(x0)
