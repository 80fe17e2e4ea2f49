"""GPU parity of the block-Jacobi preconditioner kernels (djac_gen /
djac_apply, tt_linalg.f90:363-531) against the oracle, through the C ABI.

Bar: the inverted blocks to 1e-9 relative (LU of the same blocks, different
summation order), the applied vector to 1e-9.  Shapes cover the
shared-memory inverse (block <= 112), the global-memory inverse (128), the
in-place apply (x == y) and unequal ranks."""
import numpy as np
import pytest

from oracle.jac import jac_gen, jac_apply

pytestmark = pytest.mark.gpu

SHAPES = [
    # rx1, n, rx2, ra1, ra2
    (3, 4, 2, 2, 3),
    (8, 16, 8, 3, 3),      # 'l' and 'r' blocks of 128 (global-memory LU)
    (16, 64, 12, 3, 3),    # 'c': 192 blocks of 64
    (5, 7, 9, 4, 1),
]


@pytest.mark.parametrize("p", ["c", "l", "r"])
@pytest.mark.parametrize("shape", SHAPES)
def test_djac_gen_apply(torch_cuda, ctx, p, shape):
    import ttgpu
    torch = torch_cuda
    rx1, n, rx2, ra1, ra2 = shape
    rng = np.random.default_rng(3 + sum(shape))
    # diagonally dominant local operators, as near-converged sweeps give
    phi1 = rng.standard_normal((rx1, rx1, ra1)) + 4 * np.eye(rx1)[:, :, None]
    phi2 = rng.standard_normal((rx2, ra2, rx2)) + 4 * np.eye(rx2)[:, None, :]
    A = rng.standard_normal((ra1, n, n, ra2)) + 4 * np.eye(n)[None, :, :, None]
    phi1, phi2, A = (a.ravel(order="F") for a in (phi1, phi2, A))
    ref = jac_gen(p, rx1, n, rx2, ra1, ra2, phi1, A, phi2)
    size = ttgpu.djac_size(p, rx1, n, rx2)
    assert size == ref.size
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    J = torch.zeros(size, dtype=torch.float64, device="cuda")
    ttgpu.djac_gen(p, rx1, n, rx2, ra1, ra2, dev(phi1), dev(A), dev(phi2), J, ctx=ctx)
    ctx.synchronize()
    Jg = J.cpu().numpy()
    assert np.linalg.norm(Jg - ref) <= 1e-9 * np.linalg.norm(ref)
    x = rng.standard_normal(rx1 * n * rx2)
    yref = jac_apply(p, rx1, n, rx2, ref, x)
    X = dev(x)
    Y = torch.zeros_like(X)
    ttgpu.djac_apply(p, rx1, n, rx2, J, X, Y, ctx=ctx)
    ttgpu.djac_apply(p, rx1, n, rx2, J, X, X, ctx=ctx)     # in place, as the reference allows
    ctx.synchronize()
    for out in (Y, X):
        assert np.linalg.norm(out.cpu().numpy() - yref) <= 1e-9 * np.linalg.norm(yref)
