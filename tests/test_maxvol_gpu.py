"""GPU maxvol (ttg_dmaxvol) against the oracle restatement of maxvol0_d
(maxvol.f90:27-119): the same rows in the same order (index work: exact), Z
to 1e-10 relative, and the maxvol contract."""
import numpy as np
import pytest

from oracle.maxvol import maxvol, maxvol_contract

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,seed,tol", [(50, 5, 0, 1e-2), (200, 20, 1, 1e-2),
                                          (512, 64, 2, 1e-2), (8, 8, 3, 1e-2),
                                          (1000, 1, 4, 1e-2), (3000, 100, 5, 1e-2),
                                          (100000, 16, 6, 1e-2), (400, 10, 9, 0.5)])
def test_dmaxvol_matches_oracle(torch_cuda, ctx, m, n, seed, tol):
    import ttgpu
    torch = torch_cuda
    a = np.random.default_rng(seed).standard_normal((m, n))
    p_ref, z_ref, _ = maxvol(a, tol=tol)
    A = torch.from_numpy(np.asfortranarray(a).ravel(order="F")).cuda()
    p = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    Z = torch.full((m * n,), float("nan"), dtype=torch.float64, device="cuda")
    ttgpu.dmaxvol(m, n, A, p, Z, tol=tol)
    ctx.synchronize()
    p_gpu = p.cpu().numpy()
    z_gpu = Z.cpu().numpy().reshape((m, n), order="F")
    assert p_gpu.tolist() == p_ref.tolist()
    assert np.linalg.norm(z_gpu - z_ref) <= 1e-10 * np.linalg.norm(z_ref)
    assert maxvol_contract(a, p_gpu, z_gpu, tol=tol)


def test_dmaxvol_rejects_wide(torch_cuda, ctx):
    import ttgpu
    torch = torch_cuda
    A = torch.zeros(12, dtype=torch.float64, device="cuda")
    p = torch.zeros(4, dtype=torch.int64, device="cuda")
    with pytest.raises(RuntimeError):
        ttgpu.dmaxvol(3, 4, A, p)


def test_dmaxvol_singular_is_an_error(torch_cuda, ctx):
    import ttgpu
    torch = torch_cuda
    A = torch.zeros(20, dtype=torch.float64, device="cuda")
    p = torch.zeros(2, dtype=torch.int64, device="cuda")
    with pytest.raises(RuntimeError):
        ttgpu.dmaxvol(10, 2, A, p)
