"""GPU parity of ztt_ksl (KSL time stepping) against the oracle restatement.

Bar: KSL states to 1e-8 relative in the 2-norm (the Expokit tolerance of the
reference); the closed-form fixture to 1e-12."""
import numpy as np
import pytest

from oracle.ksl import ztt_ksl as oracle_ksl, tt_full
from test_ksl import load_dat, separable
from ttgpu.operators import ksl_operator, random_tt_complex

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_ksl_eye_fixture(ctx):
    import ttgpu
    d, n, m, ra, ry, crA, crY, tau = load_dat("test_eye_ksl_dat.npz")
    cores, ry1 = ttgpu.ztt_ksl(d, n, m, ra, crA, crY, ry, tau, 150, ctx=ctx)
    x0 = tt_full(d, n, ry, crY)
    assert _rel(tt_full(d, n, ry1, cores), np.exp(1j * tau) * x0) < 1e-12


def test_ksl_reference_fixture_ten_steps(ctx):
    """test_ksl.f90 calls ztt_ksl ten times on test_ksl.dat."""
    import ttgpu
    d, n, m, ra, ry, crA, crY, tau = load_dat("test_ksl_dat.npz")
    cores, ry1 = ttgpu.ztt_ksl(d, n, m, ra, crA, crY, ry, tau, 150, nsteps=10, ctx=ctx)
    c, r = crY, list(ry)
    for _ in range(10):
        out = oracle_ksl(d, n, m, ra, crA, c, r, tau, 150)
        c, r = out["cores"], out["ry"]
    assert ry1 == r
    assert _rel(tt_full(d, n, ry1, cores), tt_full(d, n, r, c)) < 1e-8


def test_ksl_separable_exact(ctx):
    import ttgpu
    import scipy.linalg as sla
    d, nn, tau = 5, 3, 0.05
    crA, ra, full, y = separable(d, nn, 0)
    cores, ry1 = ttgpu.ztt_ksl(d, [nn] * d, [nn] * d, ra, crA, y, [1] * (d + 1), tau, 10, ctx=ctx)
    x0 = tt_full(d, [nn] * d, [1] * (d + 1), y)
    ref = sla.expm(tau * full) @ x0
    assert _rel(tt_full(d, [nn] * d, ry1, cores), ref) < 1e-10


def test_ksl_laplace_perturbed_small(ctx):
    """The KSL workload's operator family at a size the oracle finishes fast:
    -(Laplacian) + random rank-4 TT-matrix, rank-4 start, 3 steps."""
    import ttgpu
    d, n, r, tau = 6, 8, 4, 1e-3
    nn, mm, ra, crA = ksl_operator(d=d, n=n, rank=4, std=0.1, seed=1)
    _, ry, y = random_tt_complex(d, n, r, seed=2)
    cores, ry1 = ttgpu.ztt_ksl(d, nn, mm, ra, crA, y, ry, tau, 64, nsteps=3, ctx=ctx)
    c, rr = y, list(ry)
    for _ in range(3):
        out = oracle_ksl(d, nn, mm, ra, crA, c, rr, tau, 64)
        c, rr = out["cores"], out["ry"]
    assert ry1 == rr
    assert _rel(tt_full(d, nn, ry1, cores), tt_full(d, nn, rr, c)) < 1e-8


@pytest.mark.parametrize("d,n,r,steps", [(6, 8, 4, 3), (5, 16, 8, 4)])
def test_ksl_split_against_fp64(ctx, d, n, r, steps):
    """Chosen form: the K-step products on the BF16x3 tensor-core operator
    (complex operator realified with doubled ranks); S-steps, QR and the
    norm estimate's transposed products stay FP64.  Bar: 1e-5 relative to
    the FP64 state (the split products carry ~1e-6 relative error)."""
    import ttgpu
    tau = 1e-3
    nn, mm, ra, crA = ksl_operator(d=d, n=n, rank=4, std=0.1, seed=3)
    _, ry, y = random_tt_complex(d, n, r, seed=4)
    c64, r64 = ttgpu.ztt_ksl(d, nn, mm, ra, crA, y, ry, tau, 64, nsteps=steps, ctx=ctx)
    csp, rsp = ttgpu.ztt_ksl(d, nn, mm, ra, crA, y, ry, tau, 64, nsteps=steps, method="split",
                             ctx=ctx)
    assert rsp == r64
    err = _rel(tt_full(d, nn, rsp, csp), tt_full(d, nn, r64, c64))
    assert err < 1e-5, err


def test_ksl_split_eye_fixture(ctx):
    import ttgpu
    d, n, m, ra, ry, crA, crY, tau = load_dat("test_eye_ksl_dat.npz")
    cores, ry1 = ttgpu.ztt_ksl(d, n, m, ra, crA, crY, ry, tau, 150, method="split", ctx=ctx)
    x0 = tt_full(d, n, ry, crY)
    assert _rel(tt_full(d, n, ry1, cores), np.exp(1j * tau) * x0) < 1e-6


def _diag_random(d, n, ra_r, ry_r, seed, complex_):
    rng = np.random.default_rng(seed)
    ra = [1] + [ra_r] * (d - 1) + [1]
    ry = [1] + [ry_r] * (d - 1) + [1]
    def draw(sz):
        v = rng.standard_normal(sz)
        return v + 1j * rng.standard_normal(sz) if complex_ else v
    crA = np.concatenate([0.5 * draw(ra[k] * n * ra[k + 1]) for k in range(d)])
    y = np.concatenate([draw(ry[k] * n * ry[k + 1]) for k in range(d)])
    return ra, ry, crA, y


@pytest.mark.parametrize("complex_", [True, False])
def test_diag_ksl_matches_oracle(ctx, complex_):
    """ztt_diag_ksl / dtt_diag_ksl (tt_diag_ksl.f90:315,560) against the
    oracle over 3 steps: per-slice Krylov exponentials, anorm = 1."""
    import ttgpu
    from oracle.ksl import ztt_diag_ksl
    d, n, tau = 4, 3, 0.05
    ra, ry, crA, y = _diag_random(d, n, 2, 3, 11, complex_)
    cores, ry1 = ttgpu.tt_diag_ksl(d, [n] * d, ra, crA, y, ry, tau, 10, nsteps=3, ctx=ctx)
    assert np.iscomplexobj(cores) == complex_
    c, r = y, list(ry)
    for _ in range(3):
        out = ztt_diag_ksl(d, [n] * d, ra, crA, c, r, tau, 10)
        c, r = out["cores"], out["ry"]
    assert ry1 == r
    assert _rel(tt_full(d, [n] * d, ry1, cores), tt_full(d, [n] * d, r, c)) < 1e-8


def test_diag_ksl_exact_on_separable(ctx):
    import ttgpu
    from test_ksl import diag_sum_operator
    d, nn, tau = 5, 4, 0.1
    ra, crA, a, y0 = diag_sum_operator(d, nn, 0)
    cores, ry1 = ttgpu.tt_diag_ksl(d, [nn] * d, ra, crA, np.concatenate(y0), [1] * (d + 1), tau,
                                   10, ctx=ctx)
    ex = y0[0] * np.exp(tau * a[0])
    for k in range(1, d):
        ex = np.kron(y0[k] * np.exp(tau * a[k]), ex)
    assert _rel(tt_full(d, [nn] * d, ry1, cores), ex) < 1e-12


def _cme():
    import os
    from conftest import GOLDEN
    f = np.load(os.path.join(GOLDEN, "cme20_ksl.npz"))
    n = [int(v) for v in f["n"]]
    return (len(n), n, [int(v) for v in f["ra"]], f["crA"].astype(np.complex128),
            [int(v) for v in f["ry"]], f["crY"].astype(np.complex128), float(f["tau"]))


def test_ksl_cme_fixture_two_steps(ctx):
    """The reference's own KSL application (test_ksl_cme.f90: the chemical
    master equation of cme20_A.sdv / cme20_u0.sdv, d = 121, tau = T/Nt = 0.01):
    two steps on the GPU against two oracle steps, and the chosen (split)
    method against the plain one.  Each step runs 2d - 1 = 241 local Krylov
    exponentials, each accurate to Expokit's tolerance 1e-8, so two correct
    implementations (different summation orders, which move the step-size
    choices) differ by a few 1e-8 per step (measured 1.9e-8 after one step,
    4e-8 after two); the bar here is 1e-7 after two steps."""
    import ttgpu
    d, n, ra, crA, ry, crY, tau = _cme()
    cores, ry1 = ttgpu.ztt_ksl(d, n, n, ra, crA, crY, ry, tau, 500, nsteps=2, ctx=ctx)
    c, r = crY, list(ry)
    for _ in range(2):
        out = oracle_ksl(d, n, n, ra, crA, c, r, tau, 500)
        c, r = out["cores"], out["ry"]
    assert ry1 == r
    from ttgpu.operators import tt_rel_diff
    assert tt_rel_diff(d, n, ry1, cores, r, c) < 1e-7
    cs, rs = ttgpu.ztt_ksl(d, n, n, ra, crA, crY, ry, tau, 500, nsteps=2, method="split", ctx=ctx)
    assert rs == ry1
    assert tt_rel_diff(d, n, rs, cs, ry1, cores) < 1e-4


def test_tt_ksl_real_scaled_identity(ctx):
    """Real tt_ksl scheme, A = c I: exp(c tau) y0 for a start of any rank."""
    import ttgpu
    from test_ksl import scaled_identity
    d, nn, c, tau = 5, 3, 0.7, 0.3
    ra, crA = scaled_identity(d, nn, c)
    ry = [1, 3, 4, 4, 3, 1]
    rng = np.random.default_rng(1)
    y = np.concatenate([rng.standard_normal(ry[k] * nn * ry[k + 1]) for k in range(d)])
    cores, ry1 = ttgpu.tt_ksl(d, [nn] * d, [nn] * d, ra, crA, y, ry, tau, 10, ctx=ctx)
    assert cores.dtype == np.float64 and ry1 == ry
    x0 = tt_full(d, [nn] * d, ry, y)
    assert _rel(tt_full(d, [nn] * d, ry1, cores), np.exp(c * tau) * x0) < 1e-12


@pytest.mark.parametrize("d,n,r,steps", [(6, 8, 4, 3), (4, 4, 2, 2)])
def test_tt_ksl_real_matches_oracle(ctx, d, n, r, steps):
    """Real tt_ksl (tt_ksl.f90:191-428) on the KSL operator family with a real
    start, nsteps on the device against the oracle called step by step."""
    import ttgpu
    from oracle.ksl import tt_ksl_real
    from ttgpu.operators import random_tt
    tau = 1e-3
    nn, mm, ra, crA = ksl_operator(d=d, n=n, rank=4, std=0.1, seed=5)
    _, ry, y = random_tt(d, n, r, seed=6)
    cores, ry1 = ttgpu.tt_ksl(d, nn, mm, ra, crA, y, ry, tau, 64, nsteps=steps, ctx=ctx)
    c, rr = y, list(ry)
    for _ in range(steps):
        out = tt_ksl_real(d, nn, mm, ra, crA, c, rr, tau, 64)
        c, rr = out["cores"], out["ry"]
    assert ry1 == rr
    assert _rel(tt_full(d, nn, ry1, cores), tt_full(d, nn, rr, c)) < 1e-8


def test_tt_ksl_real_split_against_fp64(ctx):
    """Chosen form for the real scheme: K-step products on the BF16x3
    tensor-core operator; bar 1e-5 relative to the FP64 state."""
    import ttgpu
    from ttgpu.operators import random_tt
    d, n, r, steps, tau = 5, 16, 8, 3, 1e-3
    nn, mm, ra, crA = ksl_operator(d=d, n=n, rank=4, std=0.1, seed=7)
    _, ry, y = random_tt(d, n, r, seed=8)
    c64, r64 = ttgpu.tt_ksl(d, nn, mm, ra, crA, y, ry, tau, 64, nsteps=steps, ctx=ctx)
    csp, rsp = ttgpu.tt_ksl(d, nn, mm, ra, crA, y, ry, tau, 64, nsteps=steps, method="split",
                            ctx=ctx)
    assert rsp == r64
    assert _rel(tt_full(d, nn, rsp, csp), tt_full(d, nn, r64, c64)) < 1e-5


def test_tt_ksl_real_single_core_half_step(ctx):
    import ttgpu
    import scipy.linalg as sla
    rng = np.random.default_rng(2)
    nn, tau = 6, 0.2
    a = rng.standard_normal((nn, nn))
    y = rng.standard_normal(nn)
    cores, _ = ttgpu.tt_ksl(1, [nn], [nn], [1, 1], a.ravel(order="F"), y, [1, 1], tau, 10,
                            ctx=ctx)
    ref = sla.expm(tau / 2 * a) @ y
    assert _rel(cores, ref) < 1e-10


def test_tt_ksl_real_rejects_ranks_the_qr_would_cut(ctx):
    import ttgpu
    from test_ksl import scaled_identity
    d, nn = 3, 2
    ra, crA = scaled_identity(d, nn, 1.0)
    ry = [1, 2, 4, 1]
    y = np.ones(sum(ry[k] * nn * ry[k + 1] for k in range(d)))
    with pytest.raises(RuntimeError):
        ttgpu.tt_ksl(d, [nn] * d, [nn] * d, ra, crA, y, ry, 0.1, 10, ctx=ctx)
    # the context stays usable
    ry_ok = [1, 1, 2, 1]
    y_ok = np.ones(sum(ry_ok[k] * nn * ry_ok[k + 1] for k in range(d)))
    cores, ry1 = ttgpu.tt_ksl(d, [nn] * d, [nn] * d, ra, crA, y_ok, ry_ok, 0.1, 10, ctx=ctx)
    x0 = tt_full(d, [nn] * d, ry_ok, y_ok)
    assert _rel(tt_full(d, [nn] * d, ry1, cores), np.exp(0.1) * x0) < 1e-12


def _ragged_operator(seed):
    """Real TT-matrix with ragged mode sizes n = [2, 3, 4, 2] and ranks
    [1, 2, 3, 2, 1], N(0, 0.3^2) entries."""
    rng = np.random.default_rng(seed)
    n, ra = [2, 3, 4, 2], [1, 2, 3, 2, 1]
    crA = np.concatenate([0.3 * rng.standard_normal(ra[k] * n[k] * n[k] * ra[k + 1])
                          for k in range(4)])
    return n, ra, crA


def test_tt_ksl_real_ragged_modes_and_rank_cut(ctx):
    """Ragged modes, and a start whose first rank (4) is above what core 1
    allows (2): the left-to-right QR cuts it, on the GPU as in the oracle."""
    import ttgpu
    from oracle.ksl import tt_ksl_real
    n, ra, crA = _ragged_operator(11)
    ry = [1, 4, 3, 2, 1]
    rng = np.random.default_rng(12)
    y = np.concatenate([rng.standard_normal(ry[k] * n[k] * ry[k + 1]) for k in range(4)])
    cores, ry1 = ttgpu.tt_ksl(4, n, n, ra, crA, y, ry, 0.05, 10, nsteps=2, ctx=ctx)
    c, rr = y, list(ry)
    for _ in range(2):
        out = tt_ksl_real(4, n, n, ra, crA, c, rr, 0.05, 10)
        c, rr = out["cores"], out["ry"]
    assert ry1 == rr == [1, 2, 3, 2, 1]
    assert _rel(tt_full(4, n, ry1, cores), tt_full(4, n, rr, c)) < 1e-8


def test_ksl_config_size_plain_vs_oracle(ctx):
    """The KSL workload at its configured size: d=16, n=32, A = -(Dirichlet
    Laplacian) + random rank-4 TT-matrix with N(0, 0.01^2) entries (operator
    rank 6), x0 a random rank-8 TT vector of norm 1, tau = 1e-3; 10 steps of
    the PLAIN (FP64) method against 10 oracle steps.  The 2-norm of the
    difference tensor is taken by QR sweeps (resolves far below 1e-8).  Bar:
    1e-8 relative, the KSL state tolerance of the reference's Expokit."""
    import ttgpu
    from ttgpu.operators import tt_dot, tt_rel_diff
    d, nn, r, tau, steps = 16, 32, 8, 1e-3, 10
    n_, m_, ra, crA = ksl_operator(d=d, n=nn, rank=4, std=0.01, seed=1)
    _, ry, y = random_tt_complex(d, nn, r, seed=2)
    y = y.copy()
    y[:ry[1] * nn] /= np.sqrt(tt_dot(d, n_, ry, y, ry, y).real)
    cores, ry1 = ttgpu.ztt_ksl(d, n_, m_, ra, crA, y, ry, tau, 64, nsteps=steps, ctx=ctx)
    c, rr = y, list(ry)
    for _ in range(steps):
        out = oracle_ksl(d, n_, m_, ra, crA, c, rr, tau, 64)
        c, rr = out["cores"], out["ry"]
    assert ry1 == rr
    assert tt_rel_diff(d, n_, ry1, cores, rr, c) < 1e-8
