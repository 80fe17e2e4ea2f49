"""CPU tests of the C-ABI library: it loads, exports every declared symbol, and
its host-side logic (no GPU needed) matches the oracle."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from oracle import ops


def _declared():
    txt = open(os.path.join(ROOT, "include", "ttgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    # ttg_* entry points and the reference-named by-reference kernels
    pat = r"\b(ttg_[a-z0-9_]+|dbfun3|djac_gen|djac_apply|dqr)\s*\("
    return sorted(set(re.findall(pat, txt)))


@pytest.fixture(scope="module")
def lib():
    import ttgpu
    return ttgpu.lib()


def test_library_exports_every_declared_symbol(lib):
    import ttgpu
    names = _declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(ttgpu.EXPORTED)


def test_my_chop3_c_abi_matches_oracle(lib):
    import ttgpu
    rng = np.random.default_rng(0)
    for _ in range(200):
        k = int(rng.integers(1, 40))
        s = np.sort(np.abs(rng.standard_normal(k)) * 10.0 ** rng.uniform(-12, 0, k))[::-1]
        eps = 10.0 ** rng.uniform(-12, 0)
        assert ttgpu.my_chop3(s, eps) == ops.my_chop3(s, eps)


def test_version_and_null_context(lib):
    import ctypes as C
    assert lib.ttg_version() >= 10000
    # every entry point rejects a null context with TTG_ERR_ARG, never crashes
    assert lib.ttg_synchronize(C.c_void_p()) == -1
    assert lib.ttg_free_result(C.c_void_p()) == -1


def test_real_entry_points_refuse_complex_arrays(lib):
    """A real entry point given complex data raises instead of dropping the
    imaginary parts (the array check runs before any device work)."""
    import ttgpu
    assert ttgpu._darr([1, 2.5]).dtype == np.float64
    assert ttgpu._darr(np.arange(3, dtype=np.float32)).flags["C_CONTIGUOUS"]
    with pytest.raises(TypeError):
        ttgpu._darr(np.array([1.0 + 0.5j]))
    with pytest.raises(TypeError):
        ttgpu._darr(np.zeros(2, dtype=np.complex128))


def test_driver_wrappers_check_array_sizes_before_any_device_work(lib):
    """The C drivers take bare pointers; the Python mirror rejects arrays
    shorter than their sizes say (TTG_ERR_ARG), before a context exists."""
    import ttgpu
    from ttgpu.operators import xxz_mpo, random_tt
    d, B = 6, 2
    n, m, ra, crA = xxz_mpo(d)
    _, ry, cr = random_tt(d, 2, 4, last=B, seed=1)
    cases = [
        lambda: ttgpu.tt_eigb(d, n, m, ra, crA[:-1], cr, ry, 1e-8, 16, B),
        lambda: ttgpu.tt_eigb(d, n, m, ra, crA, cr[:-3], ry, 1e-8, 16, B),
        lambda: ttgpu.tt_eigb(d, n[:-1], m, ra, crA, cr, ry, 1e-8, 16, B),
        lambda: ttgpu.tt_eigb(0, n, m, ra, crA, cr, ry, 1e-8, 16, B),
        lambda: ttgpu.ztt_ksl(d, n, m, ra, crA, cr[:5].astype(complex), [1] + [4] * (d - 1) + [1],
                              1e-3, 16),
        lambda: ttgpu.tt_ksl(d, n, m, ra[:-1], crA, cr, ry, 1e-3, 16),
        lambda: ttgpu.tt_mvk4(d, n, m, ry, ra, crA, cr[:10], cr, ry, 1e-8, 16),
        lambda: ttgpu.dtt_amen_solve(d, n, m, ry, ra, crA, cr, cr[:7], ry, 1e-8),
        lambda: ttgpu.tt_amen_solve(d, n, m, ry, ra, crA, cr[:7], cr, ry, 1e-8),
        lambda: ttgpu.tt_diag_ksl(d, n, [1] * (d + 1), np.ones(2 * d - 1), np.ones(2 * d),
                                  [1] * (d + 1), 1e-3, 16),
    ]
    for k, call in enumerate(cases):
        with pytest.raises(ttgpu.TTGError) as e:
            call()
        assert e.value.code == ttgpu.TTG_ERR_ARG, k


class _FakeDev:
    """Stands in for a contiguous torch CUDA tensor: only what the pointer
    checks read."""
    is_cuda = True

    def __init__(self, n, dtype="float64"):
        self.n, self.dtype = int(n), "torch." + dtype

    def is_contiguous(self):
        return True

    def numel(self):
        return self.n

    def data_ptr(self):
        return 0


class _StubCtx:
    handle = None

    def bind_torch_stream(self):
        pass

    def check(self, rc):
        assert rc == 0


def test_kernel_wrappers_check_tensor_sizes_and_types(monkeypatch):
    """Every kernel-level wrapper accepts tensors of exactly the sizes its
    GPU tests allocate, and rejects one element fewer (TTG_ERR_ARG) or the
    wrong element type (TypeError) before the library is called."""
    import ttgpu

    real = ttgpu.lib()

    class _Lib:
        def __getattr__(self, name):
            if name == "ttg_djac_size":            # host-side, no device work
                return real.ttg_djac_size
            return lambda *a: 0

    monkeypatch.setattr(ttgpu, "lib", lambda: _Lib())
    ctx = _StubCtx()
    F = _FakeDev
    rx1, m, rx2, ry1, n, ry2, ra1, ra2, nv = 7, 3, 11, 5, 2, 9, 2, 3, 2
    sizes = dict(phi1=ry1 * rx1 * ra1, A=ra1 * n * m * ra2, phi2=rx2 * ra2 * ry2,
                 x=rx1 * m * rx2 * nv, y=ry1 * n * ry2 * nv)
    dims = (rx1, m, rx2, ry1, n, ry2, ra1, ra2)

    def calls(sz, dt="float64", ct="complex128"):
        f = lambda k: F(sz[k], dt)  # noqa: E731
        z = lambda k: F(sz[k], ct)  # noqa: E731
        return [
            lambda: ttgpu.dbfun3(*dims, f("phi1"), f("A"), f("phi2"), f("x"), f("y"), nvec=nv,
                                 ctx=ctx),
            lambda: ttgpu.zbfun3(*dims, z("phi1"), z("A"), z("phi2"), z("x"), z("y"), nvec=nv,
                                 ctx=ctx),
            lambda: ttgpu.zbfun3(*dims, z("phi1"), z("A"), z("phi2"), z("y"), z("x"), nvec=nv,
                                 transp=True, ctx=ctx),
        ]

    for call in calls(sizes):
        call()
    for key in sizes:
        short = dict(sizes)
        short[key] -= 1
        for call in calls(short):
            with pytest.raises(ttgpu.TTGError):
                call()
    with pytest.raises(TypeError):
        calls(sizes, dt="float32")[0]()
    with pytest.raises(TypeError):
        calls(sizes, ct="float64")[1]()

    # interface updates, dense algebra, maxvol, block-Jacobi, prepared operator
    px, py = rx1 * m * rx2, ry1 * n * ry2
    ok = [
        lambda s: ttgpu.phi_left(*dims, F(ry1 * rx1 * ra1 - s), F(sizes["A"]), F(px), F(py),
                                 F(ry2 * rx2 * ra2), ctx=ctx),
        lambda s: ttgpu.phi_right(*dims, F(rx2 * ra2 * ry2), F(sizes["A"]), F(px), F(py),
                                  F(rx1 * ra1 * ry1 - s), ctx=ctx),
        lambda s: ttgpu.phi_left(*dims, F(ry1 * rx1 * ra1, "complex128"),
                                 F(sizes["A"], "complex128"), F(px - s, "complex128"),
                                 F(py, "complex128"), F(ry2 * rx2 * ra2, "complex128"),
                                 complex_=True, ctx=ctx),
        lambda s: ttgpu.phi2_left(6, 5, 4, 3, 7, F(4 * 6), F(6 * 3 * 5), F(4 * 3 * 7),
                                  F(7 * 5 - s), ctx=ctx),
        lambda s: ttgpu.phi2_right(6, 5, 4, 3, 7, F(5 * 7), F(6 * 3 * 5 - s), F(4 * 3 * 7),
                                   F(6 * 4), ctx=ctx),
        lambda s: ttgpu.fullmat(4, 2, 5, 3, 4, F(4 * 4 * 3), F(3 * 2 * 2 * 4), F(5 * 4 * 5),
                                F(40 * 40 - s), ctx=ctx),
        lambda s: ttgpu.dqr(300, 7, F(2100), F(7 * 7 - s), ctx=ctx),
        lambda s: ttgpu.dqr(64, 128, F(64 * 128 - s), F(64 * 128), ctx=ctx),
        lambda s: ttgpu.dqr(40, 9, F(360, "complex128"), F(81 - s, "complex128"),
                            complex_=True, ctx=ctx),
        lambda s: ttgpu.dsyev(17, F(289 - s), F(17), ctx=ctx),
        lambda s: ttgpu.dgesvd(7, 3, F(21), F(21), F(3), F(9 - s), ctx=ctx),
        lambda s: ttgpu.dgesvd(3, 7, F(21), F(9 - s), F(3), F(21), ctx=ctx),
        lambda s: ttgpu.dmaxvol(50, 5, F(250), F(5 - s, "int64"), F(250), ctx=ctx),
        lambda s: ttgpu.dmaxvol(3, 4, F(12 - s), F(4, "int64"), ctx=ctx),
        lambda s: ttgpu.djac_gen("l", 3, 4, 2, 2, 3, F(18), F(96), F(12),
                                 F(ttgpu.djac_size("l", 3, 4, 2) - s), ctx=ctx),
        lambda s: ttgpu.djac_apply("r", 3, 4, 2, F(ttgpu.djac_size("r", 3, 4, 2)), F(24),
                                   F(24 - s), ctx=ctx),
    ]
    for k, call in enumerate(ok):
        call(0)
        with pytest.raises(ttgpu.TTGError):
            call(1)
    op = ttgpu.LocalOp(24, 2, 40, 24, 2, 40, 5, 4, F(24 * 24 * 5), F(5 * 2 * 2 * 4),
                       F(40 * 4 * 40), nvec_max=4, ctx=ctx)
    op.apply(F(24 * 2 * 40 * 3), F(24 * 2 * 40 * 3), 3)
    with pytest.raises(ttgpu.TTGError):
        op.apply(F(24 * 2 * 40 * 3), F(24 * 2 * 40 * 3 - 1), 3)
    op._h = None
    with pytest.raises(TypeError):
        ttgpu.dmaxvol(50, 5, F(250), F(5, "int32"), ctx=ctx)
