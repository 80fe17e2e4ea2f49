"""GPU test of ttg_dbfun3_noalloc, the allocation-free local operator.

It serves callers that cannot allocate device memory during a call (hosts
whose device memory belongs to another allocator, solver callbacks that cannot
absorb cudaMalloc's synchronisation).  Its output must equal ttg_dbfun3's on
the same inputs (same GEMM sequence, same tolerance as the other FP64 kernel
tests), on two calls in a row that share the fixed scratch array, and it must
reject sizes beyond the fixed maximum.  Collected last so that a failure here
does not hide the other tests in a run that stops at the first failure.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _call(fn, ctx, dims, ptrs, nvec):
    return fn(ctx.handle, *[C.c_int64(v) for v in dims], *[C.c_void_p(p.data_ptr()) for p in ptrs],
              C.c_int64(nvec))


def test_noalloc_matches_dbfun3_twice(torch_cuda):
    import ttgpu
    torch = torch_cuda
    ctx = ttgpu.Context(0)
    ctx.bind_torch_stream()
    lib = ttgpu.lib()
    shapes = [(64, 2, 64, 64, 2, 64, 5, 5, 5), (7, 3, 11, 5, 2, 9, 2, 3, 2)]
    for call, (rx1, m, rx2, ry1, n, ry2, ra1, ra2, nvec) in enumerate(shapes):
        rng = np.random.default_rng(100 + call)
        t = lambda k: torch.from_numpy(rng.standard_normal(k)).cuda()
        phi1, A, phi2 = t(ry1 * rx1 * ra1), t(ra1 * n * m * ra2), t(rx2 * ra2 * ry2)
        X = t(rx1 * m * rx2 * nvec)
        ysz = ry1 * n * ry2 * nvec
        y_ref = torch.zeros(ysz, dtype=torch.float64, device="cuda")
        y_new = torch.full((ysz,), float("nan"), dtype=torch.float64, device="cuda")
        dims = (rx1, m, rx2, ry1, n, ry2, ra1, ra2)
        ctx.check(_call(lib.ttg_dbfun3, ctx, dims, (phi1, A, phi2, X, y_ref), nvec))
        ctx.check(_call(lib.ttg_dbfun3_noalloc, ctx, dims, (phi1, A, phi2, X, y_new), nvec))
        ctx.synchronize()
        a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
        assert np.all(np.isfinite(a))
        assert np.linalg.norm(a - b) <= TOL * np.linalg.norm(b)
    ctx.close()


def test_noalloc_leaves_device_memory_unchanged(torch_cuda):
    """The point of the entry point: after the first call's set-up, further
    calls at the largest shape the fixed array allows take no device memory
    (free memory as the driver reports it does not move)."""
    import ttgpu
    torch = torch_cuda
    ctx = ttgpu.Context(0)
    ctx.bind_torch_stream()
    lib = ttgpu.lib()
    # (rx1*m*ra2*ry2 + rx1*ra1*n*ry2) * nvec = 2 * 128*2*5*128 * 6 = 1,966,080 <= 2^21
    rx1 = rx2 = ry1 = ry2 = 128
    m = n = 2
    ra1 = ra2 = 5
    nvec = 6
    rng = np.random.default_rng(7)
    t = lambda k: torch.from_numpy(rng.standard_normal(k)).cuda()
    phi1, A, phi2 = t(ry1 * rx1 * ra1), t(ra1 * n * m * ra2), t(rx2 * ra2 * ry2)
    X = t(rx1 * m * rx2 * nvec)
    y = torch.zeros(ry1 * n * ry2 * nvec, dtype=torch.float64, device="cuda")
    dims = (rx1, m, rx2, ry1, n, ry2, ra1, ra2)
    ctx.check(_call(lib.ttg_dbfun3_noalloc, ctx, dims, (phi1, A, phi2, X, y), nvec))
    ctx.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(4):
        ctx.check(_call(lib.ttg_dbfun3_noalloc, ctx, dims, (phi1, A, phi2, X, y), nvec))
    ctx.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert torch.isfinite(y).all().item()
    ctx.close()


def test_noalloc_rejects_oversized_problem(torch_cuda):
    import ttgpu
    torch = torch_cuda
    ctx = ttgpu.Context(0)
    lib = ttgpu.lib()
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    # (rx1*m*ra2*ry2 + rx1*ra1*n*ry2) * nvec = 2 * 256*2*5*256 * 4 > 2^21
    rc = _call(lib.ttg_dbfun3_noalloc, ctx, (256, 2, 256, 256, 2, 256, 5, 5),
               (dummy, dummy, dummy, dummy, dummy), 4)
    assert rc == -1
    assert "fixed maximum" in lib.ttg_last_error(ctx.handle).decode()
    # sizes whose scratch product overflows 64 bits are rejected the same way
    big = 1 << 40
    rc = _call(lib.ttg_dbfun3_noalloc, ctx, (1, 1, 1, 1, 1, 1, big, big),
               (dummy, dummy, dummy, dummy, dummy), big)
    assert rc == -1
    assert "fixed maximum" in lib.ttg_last_error(ctx.handle).decode()
    ctx.close()
