"""GPU tests of the reference-named, by-reference entry points (dbfun3,
djac_gen, djac_apply, dqr of tt_linalg.f90:30,127,363,497).

They are called here exactly as gmres_3d.c calls them (gmres_3d.c:3-4,60-64):
through ctypes with `long*` sizes and HOST arrays, the matvec once in place
(x and y the same array), inside the oracle's restatement of the reference's
right-preconditioned Householder GMRES.  The same GMRES on the oracle's own
products must give the same solution."""
import ctypes as C

import numpy as np
import pytest

from oracle.amen import gmres_hh
from oracle.jac import jac_gen, jac_apply
from oracle.ops import bfun3, dqr as oracle_dqr

pytestmark = pytest.mark.gpu
_L = C.POINTER(C.c_long)


def _lib():
    import ttgpu
    L = ttgpu.lib()
    L.dbfun3.argtypes = [_L] * 8 + [C.c_void_p] * 7
    L.dbfun3.restype = None
    L.djac_gen.argtypes = [C.c_char_p] + [_L] * 5 + [C.c_void_p] * 4
    L.djac_gen.restype = None
    L.djac_apply.argtypes = [C.c_char_p] + [_L] * 3 + [C.c_void_p] * 4
    L.djac_apply.restype = None
    L.dqr.argtypes = [_L, _L, C.c_void_p, C.c_void_p, C.c_void_p, _L, C.c_void_p]
    L.dqr.restype = None
    return L


def _l(v):
    return C.byref(C.c_long(int(v)))


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _local_system(rx1, n, rx2, ra1, ra2, seed):
    """A well-conditioned local operator: the (a1, a2) = (0, 0) slice is
    identity x (shifted 1D Laplacian) x identity, the rest small noise."""
    rng = np.random.default_rng(seed)
    phi1 = 0.05 * rng.standard_normal((rx1, rx1, ra1))
    phi2 = 0.05 * rng.standard_normal((rx2, ra2, rx2))
    phi1[:, :, 0] += np.eye(rx1)
    phi2[:, 0, :] += np.eye(rx2)
    A = 0.05 * rng.standard_normal((ra1, n, n, ra2))
    A[0, :, :, 0] += 3.0 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)
    fl = lambda a: np.asfortranarray(a).ravel(order="F").copy()
    return fl(phi1), fl(A), fl(phi2)


@pytest.mark.parametrize("ptype", ["c", "l", "r"])
def test_gmres_on_by_reference_shims(ctx, ptype):
    L = _lib()
    rx1, n, rx2, ra1, ra2 = 5, 7, 6, 3, 2
    N = rx1 * n * rx2
    phi1, A, phi2 = _local_system(rx1, n, rx2, ra1, ra2, seed=1)
    # block-Jacobi blocks through the shim against the oracle's
    jsz = int(__import__("ttgpu").djac_size(ptype, rx1, n, rx2))
    jacs = np.zeros(jsz)
    L.djac_gen(ptype.encode(), _l(rx1), _l(n), _l(rx2), _l(ra1), _l(ra2), _p(phi1), _p(A),
               _p(phi2), _p(jacs))
    jref = jac_gen(ptype, rx1, n, rx2, ra1, ra2, phi1, A, phi2)
    assert np.linalg.norm(jacs - jref) <= 1e-10 * np.linalg.norm(jref)
    res1 = np.zeros(rx1 * n * ra2 * rx2 + rx1 * ra1 * n * rx2)
    res2 = np.zeros_like(res1)
    work = np.zeros(N)

    def mv_shim(v):
        # gmres_3d.c:60-61: w = P sol, then dbfun3(w, w) in place
        w = np.array(v, dtype=np.float64)
        L.djac_apply(ptype.encode(), _l(rx1), _l(n), _l(rx2), _p(jacs), _p(w), _p(w), _p(work))
        L.dbfun3(_l(rx1), _l(n), _l(rx2), _l(rx1), _l(n), _l(rx2), _l(ra1), _l(ra2), _p(phi1),
                 _p(A), _p(phi2), _p(w), _p(w), _p(res1), _p(res2))
        return w

    def mv_ref(v):
        return bfun3(rx1, n, rx2, rx1, n, rx2, ra1, ra2, phi1, A, phi2,
                     jac_apply(ptype, rx1, n, rx2, jref, v))

    rhs = np.random.default_rng(2).standard_normal(N)
    z1, k1, _ = gmres_hh(mv_shim, rhs, 40, 1e-12, 3)
    z2, k2, _ = gmres_hh(mv_ref, rhs, 40, 1e-12, 3)
    import ttgpu
    assert L.ttg_fshim_status() == ttgpu.TTG_OK
    assert np.linalg.norm(z1 - z2) <= 1e-10 * np.linalg.norm(z2)
    # the solve itself: B P z = rhs
    assert np.linalg.norm(mv_ref(z1) - rhs) <= 1e-10 * np.linalg.norm(rhs)


def test_dbfun3_shim_rectangular_and_dqr(ctx):
    L = _lib()
    rng = np.random.default_rng(3)
    rx1, m, rx2, ry1, n, ry2, ra1, ra2 = 4, 3, 5, 6, 2, 7, 2, 3
    phi1 = rng.standard_normal(ry1 * rx1 * ra1)
    A = rng.standard_normal(ra1 * n * m * ra2)
    phi2 = rng.standard_normal(rx2 * ra2 * ry2)
    x = rng.standard_normal(rx1 * m * rx2)
    y = np.zeros(ry1 * n * ry2)
    scratch = np.zeros(1)
    L.dbfun3(_l(rx1), _l(m), _l(rx2), _l(ry1), _l(n), _l(ry2), _l(ra1), _l(ra2), _p(phi1), _p(A),
             _p(phi2), _p(x), _p(y), _p(scratch), _p(scratch))
    ref = bfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, x)
    assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref)
    # dqr: Q overwrites A (LAPACK's reflector convention), R is min x m
    nr, mc = 40, 9
    M = rng.standard_normal(nr * mc)
    Q = M.copy()
    R = np.zeros(mc * mc)
    L.dqr(_l(nr), _l(mc), _p(Q), _p(R), _p(scratch), _l(1), _p(scratch))
    Qo, Ro = oracle_dqr(nr, mc, M)
    assert np.allclose(Q, np.asarray(Qo).ravel(order="F")[:nr * mc], atol=1e-12)
    assert np.allclose(R, np.asarray(Ro).ravel(order="F"), atol=1e-12)
    import ttgpu
    assert L.ttg_fshim_status() == ttgpu.TTG_OK


def test_shim_failure_is_reported_not_fatal(ctx):
    """A shim cannot return a status (the Fortran interface returns
    nothing): a failing call prints, fills its output with NaN and sets the
    status that ttg_fshim_status reports once."""
    import ttgpu
    L = _lib()
    y = np.zeros(4)
    z = np.zeros(1)
    # a zero size is rejected by the kernel-level entry point
    L.dbfun3(_l(0), _l(1), _l(1), _l(1), _l(2), _l(2), _l(1), _l(1), _p(z), _p(z), _p(z), _p(z),
             _p(y), _p(z), _p(z))
    assert np.all(np.isnan(y))
    assert L.ttg_fshim_status() == ttgpu.TTG_ERR_ARG
    assert L.ttg_fshim_status() == ttgpu.TTG_OK
