"""GPU parity of the kernel-level C-ABI entry points against the oracle.

FP64 kernels: relative error <= 1e-12 (GEMM summation order differs from the
oracle's BLAS, nothing else)."""
import numpy as np
import pytest

from oracle import ops

pytestmark = pytest.mark.gpu
TOL = 1e-12

SHAPES = [
    # rx1, m, rx2, ry1, n, ry2, ra1, ra2
    (1, 2, 2, 1, 2, 2, 1, 4),
    (3, 2, 5, 3, 2, 5, 4, 5),
    (16, 2, 16, 16, 2, 16, 5, 5),
    (64, 2, 64, 64, 2, 64, 5, 5),
    (7, 3, 11, 5, 2, 9, 2, 3),       # ragged, rectangular (ry != rx, n != m)
    (8, 32, 8, 8, 32, 8, 6, 6),      # KSL-like, large middle contraction
    (33, 64, 17, 33, 64, 17, 3, 3),  # AMEn-like n = 64
]


def _t(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("shape", SHAPES)
def test_dbfun3_block(torch_cuda, ctx, shape):
    import ttgpu
    torch = torch_cuda
    rx1, m, rx2, ry1, n, ry2, ra1, ra2 = shape
    rng = np.random.default_rng(sum(shape))
    nvec = 3
    phi1 = rng.standard_normal(ry1 * rx1 * ra1)
    A = rng.standard_normal(ra1 * n * m * ra2)
    phi2 = rng.standard_normal(rx2 * ra2 * ry2)
    X = rng.standard_normal(rx1 * m * rx2 * nvec)
    ref = ops.bfun3_block(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, X, nvec)
    Y = torch.zeros(ry1 * n * ry2 * nvec, dtype=torch.float64, device="cuda")
    ttgpu.dbfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, _t(torch, phi1), _t(torch, A),
                 _t(torch, phi2), _t(torch, X), Y, nvec=nvec)
    ctx.synchronize()
    assert _rel(Y.cpu().numpy(), ref) < TOL


@pytest.mark.parametrize("shape", SHAPES)
def test_dphi_left_right(torch_cuda, ctx, shape):
    import ttgpu
    torch = torch_cuda
    rx1, m, rx2, ry1, n, ry2, ra1, ra2 = shape
    rng = np.random.default_rng(7 + sum(shape))
    A = rng.standard_normal(ra1 * n * m * ra2)
    x = rng.standard_normal(rx1 * m * rx2)
    y = rng.standard_normal(ry1 * n * ry2)
    p1 = rng.standard_normal(ry1 * rx1 * ra1)
    p2 = rng.standard_normal(rx2 * ra2 * ry2)
    refL = ops.phi_left(rx1, m, rx2, ry1, n, ry2, ra1, ra2, p1, A, x, y)
    refR = ops.phi_right(rx1, m, rx2, ry1, n, ry2, ra1, ra2, p2, A, x, y)
    outL = torch.zeros(ry2 * rx2 * ra2, dtype=torch.float64, device="cuda")
    outR = torch.zeros(rx1 * ra1 * ry1, dtype=torch.float64, device="cuda")
    ttgpu.phi_left(rx1, m, rx2, ry1, n, ry2, ra1, ra2, _t(torch, p1), _t(torch, A),
                   _t(torch, x), _t(torch, y), outL)
    ttgpu.phi_right(rx1, m, rx2, ry1, n, ry2, ra1, ra2, _t(torch, p2), _t(torch, A),
                    _t(torch, x), _t(torch, y), outR)
    ctx.synchronize()
    assert _rel(outL.cpu().numpy(), refL) < TOL
    assert _rel(outR.cpu().numpy(), refR) < TOL


@pytest.mark.parametrize("shape", SHAPES[:6])
def test_complex_kernels(torch_cuda, ctx, shape):
    import ttgpu
    torch = torch_cuda
    rx1, m, rx2, ry1, n, ry2, ra1, ra2 = shape
    rng = np.random.default_rng(11 + sum(shape))
    c = lambda k: rng.standard_normal(k) + 1j * rng.standard_normal(k)
    phi1, A, phi2 = c(ry1 * rx1 * ra1), c(ra1 * n * m * ra2), c(rx2 * ra2 * ry2)
    x, y = c(rx1 * m * rx2), c(ry1 * n * ry2)
    ref = ops.bfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, x)
    out = torch.zeros(ry1 * n * ry2, dtype=torch.complex128, device="cuda")
    ttgpu.zbfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, _t(torch, phi1), _t(torch, A),
                 _t(torch, phi2), _t(torch, x), out)
    ctx.synchronize()
    assert _rel(out.cpu().numpy(), ref) < TOL
    # adjoint: <B x, y> = <x, B^H y>
    refT = ops.zbfun3_transp(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, y)
    outT = torch.zeros(rx1 * m * rx2, dtype=torch.complex128, device="cuda")
    ttgpu.zbfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, _t(torch, phi1), _t(torch, A),
                 _t(torch, phi2), _t(torch, y), outT, transp=True)
    ctx.synchronize()
    assert _rel(outT.cpu().numpy(), refT) < TOL
    assert abs(np.vdot(y, ref) - np.vdot(refT, x)) < 1e-10 * abs(np.vdot(y, ref))
    for left in (True, False):
        if left:
            p = c(ry1 * rx1 * ra1)
            refp = ops.phi_left(rx1, m, rx2, ry1, n, ry2, ra1, ra2, p, A, x, y, conj=True)
            outp = torch.zeros(ry2 * rx2 * ra2, dtype=torch.complex128, device="cuda")
            ttgpu.phi_left(rx1, m, rx2, ry1, n, ry2, ra1, ra2, _t(torch, p), _t(torch, A),
                           _t(torch, x), _t(torch, y), outp, complex_=True)
        else:
            p = c(rx2 * ra2 * ry2)
            refp = ops.phi_right(rx1, m, rx2, ry1, n, ry2, ra1, ra2, p, A, x, y, conj=True)
            outp = torch.zeros(rx1 * ra1 * ry1, dtype=torch.complex128, device="cuda")
            ttgpu.phi_right(rx1, m, rx2, ry1, n, ry2, ra1, ra2, _t(torch, p), _t(torch, A),
                            _t(torch, x), _t(torch, y), outp, complex_=True)
        ctx.synchronize()
        assert _rel(outp.cpu().numpy(), refp) < TOL


def test_phi2_and_fullmat(torch_cuda, ctx):
    import ttgpu
    torch = torch_cuda
    rng = np.random.default_rng(5)
    rx1, rx2, ry1, n, ry2 = 6, 5, 4, 3, 7
    p1 = rng.standard_normal(ry1 * rx1)
    p2 = rng.standard_normal(rx2 * ry2)
    x = rng.standard_normal(rx1 * n * rx2)
    y = rng.standard_normal(ry1 * n * ry2)
    o = torch.zeros(ry2 * rx2, dtype=torch.float64, device="cuda")
    ttgpu.phi2_left(rx1, rx2, ry1, n, ry2, _t(torch, p1), _t(torch, x), _t(torch, y), o)
    ctx.synchronize()
    assert _rel(o.cpu().numpy(), ops.phi2_left(rx1, rx2, ry1, n, ry2, p1, x, y)) < TOL
    o = torch.zeros(rx1 * ry1, dtype=torch.float64, device="cuda")
    ttgpu.phi2_right(rx1, rx2, ry1, n, ry2, _t(torch, p2), _t(torch, x), _t(torch, y), o)
    ctx.synchronize()
    assert _rel(o.cpu().numpy(), ops.phi2_right(rx1, rx2, ry1, n, ry2, p2, x, y)) < TOL
    rx1, m, rx2, ra1, ra2 = 4, 2, 5, 3, 4
    phi1 = rng.standard_normal(rx1 * rx1 * ra1)
    A = rng.standard_normal(ra1 * m * m * ra2)
    phi2 = rng.standard_normal(rx2 * ra2 * rx2)
    N = rx1 * m * rx2
    o = torch.zeros(N * N, dtype=torch.float64, device="cuda")
    ttgpu.fullmat(rx1, m, rx2, ra1, ra2, _t(torch, phi1), _t(torch, A), _t(torch, phi2), o)
    ctx.synchronize()
    ref = ops.fullmat(rx1, m, rx2, ra1, ra2, phi1, A, phi2)
    assert _rel(o.cpu().numpy(), ops.flat(ref)) < TOL


@pytest.mark.parametrize("nm", [(8, 8), (128, 64), (64, 128), (512, 256), (1, 5), (300, 7)])
def test_dqr_lapack_convention(torch_cuda, ctx, nm):
    import ttgpu
    torch = torch_cuda
    nr, nc = nm
    rng = np.random.default_rng(nr + nc)
    A = rng.standard_normal(nr * nc)
    q, r = ops.dqr(nr, nc, A)
    At = _t(torch, A.copy())
    R = torch.zeros(min(nr, nc) * nc, dtype=torch.float64, device="cuda")
    ttgpu.dqr(nr, nc, At, R)
    ctx.synchronize()
    k = min(nr, nc)
    assert _rel(At.cpu().numpy()[:nr * k], q) < 1e-11
    assert _rel(R.cpu().numpy(), r) < 1e-11


def test_zqr(torch_cuda, ctx):
    import ttgpu
    import scipy.linalg as sla
    torch = torch_cuda
    rng = np.random.default_rng(3)
    nr, nc = 40, 9
    A = rng.standard_normal((nr, nc)) + 1j * rng.standard_normal((nr, nc))
    q, r = sla.qr(A, mode="economic")
    At = _t(torch, ops.flat(A))
    R = torch.zeros(nc * nc, dtype=torch.complex128, device="cuda")
    ttgpu.dqr(nr, nc, At, R, complex_=True)
    ctx.synchronize()
    assert _rel(At.cpu().numpy(), ops.flat(q)) < 1e-11
    assert _rel(R.cpu().numpy(), ops.flat(r)) < 1e-11


@pytest.mark.parametrize("k", [1, 2, 5, 17, 64, 100, 200])
def test_dsyev_jacobi(torch_cuda, ctx, k):
    import ttgpu
    torch = torch_cuda
    rng = np.random.default_rng(k)
    M = rng.standard_normal((k, k))
    M = M + M.T
    w_ref = np.linalg.eigvalsh(M)
    At = _t(torch, ops.flat(M))
    w = torch.zeros(k, dtype=torch.float64, device="cuda")
    ttgpu.dsyev(k, At, w)
    ctx.synchronize()
    wv = w.cpu().numpy()
    V = ops.F(At.cpu().numpy(), k, k)
    scale = np.abs(w_ref).max()
    assert np.abs(wv - w_ref).max() < 1e-12 * scale * max(1, k / 10)
    assert np.linalg.norm(M @ V - V * wv) < 1e-11 * scale * k
    assert np.linalg.norm(V.T @ V - np.eye(k)) < 1e-12 * k


@pytest.mark.parametrize("pq", [(320, 128), (128, 320), (40, 40), (7, 3), (3, 7), (640, 256),
                                (2048, 512), (300, 900), (3000, 12), (2000, 5), (301, 41)])
def test_dgesvd_jacobi(torch_cuda, ctx, pq):
    import ttgpu
    torch = torch_cuda
    p, q = pq
    rng = np.random.default_rng(p * q)
    # graded singular values down to 1e-13 (what my_chop3 sums)
    r = min(p, q)
    U0 = np.linalg.qr(rng.standard_normal((p, r)))[0]
    V0 = np.linalg.qr(rng.standard_normal((q, r)))[0]
    s0 = np.logspace(0, -13, r)
    M = (U0 * s0) @ V0.T
    U = torch.zeros(p * r, dtype=torch.float64, device="cuda")
    s = torch.zeros(r, dtype=torch.float64, device="cuda")
    Vt = torch.zeros(r * q, dtype=torch.float64, device="cuda")
    ttgpu.dgesvd(p, q, _t(torch, ops.flat(M)), U, s, Vt)
    ctx.synchronize()
    sv = s.cpu().numpy()
    s_ref = np.linalg.svd(M, compute_uv=False)
    assert np.all(np.diff(sv) <= 0)
    assert np.abs(sv - s_ref).max() < 1e-14 * max(p, q)
    Uh = ops.F(U.cpu().numpy(), p, r)
    Vh = ops.F(Vt.cpu().numpy(), r, q)
    assert np.linalg.norm((Uh * sv) @ Vh - M) < 1e-13 * max(p, q)
    # well-separated leading singular vectors agree with LAPACK up to sign
    # (LAPACK's own vector error is ~eps*s_max/gap, so only large gaps)
    Ur, _, Vr = np.linalg.svd(M, full_matrices=False)
    for j in range(min(5, r)):
        gap = min([abs(s_ref[j] - s_ref[k]) for k in range(r) if k != j] or [1.0])
        if gap > 1e-3 * s_ref[0]:
            assert abs(abs(Uh[:, j] @ Ur[:, j]) - 1) < 1e-10

