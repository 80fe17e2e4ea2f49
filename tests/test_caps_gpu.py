"""Iteration caps of the local solvers (error paths) through the C-ABI.

The reference tolerates a local solve that stops at its cap: PRIMME returns
-3 (maxMatvecs reached) and tt_eigb goes on (tt_eigb.f90:285-288), Expokit sets
iflag = 1 and zexp_mv prints it (explib.f90:108-111), and the local GMRES
returns after nrestart x niters.  The library does the same by default and
counts such solves (ttg_capped); with strict limits the first one ends the
driver call with TTG_ERR_NOCONV.  Every case here forces a cap with tiny
limits and checks that the call returns (no hang) with the right status."""
import numpy as np
import pytest

from ttgpu.operators import xxz_mpo, random_tt, ksl_operator, random_tt_complex, amen_operator

pytestmark = pytest.mark.gpu


@pytest.fixture()
def cctx():
    import ttgpu
    c = ttgpu.Context(0)
    yield c
    c.close()


def _eigb(ttgpu, ctx, method="plain"):
    d, B = 10, 3
    n, m, ra, crA = xxz_mpo(d)
    _, ry, cr = random_tt(d, 2, 8, last=B, seed=4)
    # max_full_size 1 keeps every local problem on the iterative eigensolver;
    # eps 1e-8 (local tolerance eps/sqrt(d)/10) is reachable within the
    # reference's 500 matvecs, so only the lowered cap stops a local solve
    return ttgpu.tt_eigb(d, n, m, ra, crA, cr, ry, 1e-8, 32, B, nswp=2, max_full_size=1,
                         method=method, ctx=ctx)


@pytest.mark.parametrize("method", ["plain", "split"])
def test_eigb_matvec_cap(cctx, method):
    import ttgpu
    lam, _, _ = _eigb(ttgpu, cctx, method)          # default caps: nothing capped
    assert cctx.capped() == 0
    cctx.set_limits(max_matvecs=6)
    lam_c, _, _ = _eigb(ttgpu, cctx, method)        # tolerated, counted, finite
    assert cctx.capped() > 0
    assert np.all(np.isfinite(lam_c))
    cctx.set_limits(max_matvecs=6, strict=True)
    with pytest.raises(ttgpu.TTGError) as e:
        _eigb(ttgpu, cctx, method)
    assert e.value.code == ttgpu.TTG_ERR_NOCONV
    assert "matvec cap" in str(e.value)
    cctx.set_limits()                               # back to the reference's caps
    lam2, _, _ = _eigb(ttgpu, cctx, method)
    assert cctx.capped() == 0
    assert np.allclose(lam2, lam, rtol=1e-10, atol=0)


def _ksl(ttgpu, ctx, tau):
    d, n = 4, 8
    nn, mm, ra, crA = ksl_operator(d=d, n=n, rank=2, std=0.1, seed=1)
    _, ry, y = random_tt_complex(d, n, 3, seed=2)
    return ttgpu.ztt_ksl(d, nn, mm, ra, crA, y, ry, tau, 16, ctx=ctx)


def test_ksl_expokit_step_cap(cctx):
    import ttgpu
    tau = 4.0   # ||A|| tau ~ 60: each Krylov exponential needs several steps
    _ksl(ttgpu, cctx, tau)
    assert cctx.capped() == 0
    cctx.set_limits(max_expokit_steps=1)
    cores, _ = _ksl(ttgpu, cctx, tau)
    assert cctx.capped() > 0
    assert np.all(np.isfinite(cores))
    cctx.set_limits(max_expokit_steps=1, strict=True)
    with pytest.raises(ttgpu.TTGError) as e:
        _ksl(ttgpu, cctx, tau)
    assert e.value.code == ttgpu.TTG_ERR_NOCONV
    assert "step cap" in str(e.value)


def test_amen_gmres_restart_cap(cctx):
    """tt_amen_solve with GMRES(2) x 1 on the Laplacian family cannot meet
    the local tolerance: counted by default, NOCONV when strict."""
    import ttgpu
    d, n = 4, 16
    nn, mm, ra, crA = amen_operator(d=d, n=n)
    _, ry, y = random_tt(d, n, 2, seed=3)
    _, rx, x0 = random_tt(d, n, 2, seed=7)

    def run():
        return ttgpu.tt_amen_solve(d, nn, mm, ry, ra, crA, y, x0, rx, 1e-10, nswp=2,
                                   nrestart=2, niters=1, ctx=cctx)
    cores, _ = run()
    assert cctx.capped() > 0
    assert np.all(np.isfinite(cores))
    cctx.set_limits(strict=True)
    with pytest.raises(ttgpu.TTGError) as e:
        run()
    assert e.value.code == ttgpu.TTG_ERR_NOCONV


def test_set_limits_rejects_negative(cctx):
    import ttgpu
    with pytest.raises(ValueError):
        cctx.set_limits(max_matvecs=-1)
    rc = ttgpu.lib().ttg_set_limits(cctx.handle, ttgpu._i64(-1), ttgpu._i64(0), 0)
    assert rc == ttgpu.TTG_ERR_ARG
