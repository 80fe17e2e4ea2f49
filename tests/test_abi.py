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
    return sorted(set(re.findall(r"\b(ttg_[a-z0-9_]+)\s*\(", txt)))


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
