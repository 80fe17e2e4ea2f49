"""GPU learned preconditioner (no reference counterpart): forward pass and
parameter gradients of the hand-written kernels against the oracle, and the
gain of the trained network on a held-out chain.

Tolerances: with FP32 layer products the forward output to 1e-5 relative and
the flat gradient to 1e-4 relative (atomic accumulation in the bias
gradients reorders FP32 sums).  With the BF16 tensor-core products (the
default) the oracle rounds the same operands to bf16 before every product;
what remains is FP32 summation order, which now and then moves an
activation across a bf16 rounding boundary before the next layer (a 2^-8
change of that element): forward 5e-4, loss 1e-4, gradient 2e-3.  The eigenvalues of the preconditioned solve
to 1e-10 relative of the plain solve: both meet the same FP64 residual test
with exact ranks."""
import numpy as np
import pytest

from oracle import mlp as M
from ttgpu.operators import xxz_mpo, random_tt

pytestmark = pytest.mark.gpu


def _problem(N, B, seed):
    rng = np.random.default_rng(seed)
    D = rng.standard_normal(N) * 2.0
    theta = np.sort(rng.standard_normal(B))
    X, _ = np.linalg.qr(rng.standard_normal((N, B)))
    R = rng.standard_normal((N, B))
    R -= X @ (X.T @ R)
    V = rng.standard_normal((N, B))
    V -= X @ (X.T @ V)
    return D, theta, X, R, V


def _params(width, depth, seed):
    flat = M.init_params(width, depth, seed)
    rng = np.random.default_rng(seed + 100)
    dims = M.widths(width, depth)
    off = sum(dims[l] * dims[l + 1] + dims[l + 1] for l in range(len(dims) - 2))
    flat[off:] = (0.05 * rng.standard_normal(len(flat) - off)).astype(np.float32)
    return flat, dims


TOL = {False: (1e-5, 1e-5, 1e-4), True: (5e-4, 1e-4, 2e-3)}   # forward, loss, gradient


@pytest.mark.parametrize("bf16", [True, False])
@pytest.mark.parametrize("width", [64, 512])
def test_mlp_forward_matches_oracle(torch_cuda, ctx, bf16, width):
    import ttgpu
    torch = torch_cuda
    net = ttgpu.LearnedPrec(width=width, depth=3, seed=2, ctx=ctx)
    net.set_precision(bf16)
    assert np.array_equal(net.get_params(), M.init_params(width, 3, 2))
    flat, dims = _params(width, 3, 2)
    net.set_params(flat)
    P = 5000
    F = np.random.default_rng(3).standard_normal((P, M.NFEAT)).astype(np.float32)
    h = torch.empty(P, dtype=torch.float32, device="cuda")
    net.forward(P, torch.from_numpy(F).cuda(), h)
    ctx.synchronize()
    net.check()
    ref, _ = M.forward(M.unflatten(flat, dims), F, bf16=bf16)
    got = h.cpu().numpy()
    assert np.linalg.norm(got - ref) <= TOL[bf16][0] * np.linalg.norm(ref)
    net.close()


@pytest.mark.parametrize("bf16", [True, False])
@pytest.mark.parametrize("N,B,width", [(500, 4, 64), (2048, 5, 64), (4096, 8, 512)])
def test_mlp_gradient_matches_oracle(torch_cuda, ctx, N, B, width, bf16):
    import ttgpu
    torch = torch_cuda
    net = ttgpu.LearnedPrec(width=width, depth=3, seed=4, ctx=ctx)
    net.set_precision(bf16)
    flat, dims = _params(width, 3, 4)
    net.set_params(flat)
    D, theta, X, R, V = _problem(N, B, seed=N)
    t = lambda a: torch.from_numpy(np.asfortranarray(a).ravel(order="F")).cuda()
    loss = net.loss_grad(N, B, t(D), t(theta), t(X), t(R), t(V))
    net.check()
    g = net.get_grads()
    loss_ref, g_ref = M.loss_grad(flat, dims, D, theta, X, R, V, bf16=bf16)
    assert abs(loss - loss_ref) <= TOL[bf16][1] * max(1e-12, abs(loss_ref))
    assert np.linalg.norm(g - g_ref) <= TOL[bf16][2] * np.linalg.norm(g_ref)
    net.close()


def test_learned_preconditioner_gains_on_a_held_out_chain(ctx):
    """Record the plain method's local problems on two XXZ chains
    (delta 0.8 and 1.2), train the network on them on the GPU, then solve a
    held-out chain (delta 1.0) with and without it."""
    import ttgpu
    d, B, r, rmax, eps = 14, 4, 8, 64, 1e-10
    rec = ttgpu.Context(0)
    ttgpu.set_learned(None, 2, ctx=rec)
    for delta, seed in ((0.8, 21), (1.2, 22)):
        n, m, ra, crA = xxz_mpo(d, delta=delta)
        _, ry, cr = random_tt(d, 2, r, last=B, seed=seed)
        ttgpu.tt_eigb(d, n, m, ra, crA, cr, ry, eps, rmax, B, nswp=10, max_full_size=100, ctx=rec)
    nprob, npts = ttgpu.record_count(ctx=rec)
    assert nprob > 10 and npts > 1000
    net = ttgpu.LearnedPrec(width=512, depth=3, seed=0, ctx=ctx)
    l0, l1 = net.train_recorded(rec, steps=300, lr=1e-4, seed=1)
    assert np.isfinite(l0) and np.isfinite(l1) and 0.0 <= l0 <= 1.0
    n, m, ra, crA = xxz_mpo(d, delta=1.0)
    _, ry, cr = random_tt(d, 2, r, last=B, seed=23)
    ttgpu.set_learned(None, 0, ctx=ctx)
    lam0, _, _ = ttgpu.tt_eigb(d, n, m, ra, crA, cr, ry, eps, rmax, B, nswp=10,
                               max_full_size=100, ctx=ctx)
    mv0 = ctx.stats()["matvecs"]
    ttgpu.set_learned(net, 1, ctx=ctx)
    lam1, _, _ = ttgpu.tt_eigb(d, n, m, ra, crA, cr, ry, eps, rmax, B, nswp=10,
                               max_full_size=100, ctx=ctx)
    mv1 = ctx.stats()["matvecs"]
    ttgpu.set_learned(None, 0, ctx=ctx)
    print(f"learned preconditioner: loss {l0:.4f} -> {l1:.4f}; matvecs {mv0} -> {mv1}")
    assert np.allclose(lam1, lam0, rtol=1e-10, atol=0)
    assert mv1 < 0.9 * mv0
    net.close()
    rec.close()
