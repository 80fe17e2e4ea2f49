"""Oracle of the learned preconditioner (no reference counterpart): the
analytic gradient against central differences in float64, the untrained
network equals the classical diagonal preconditioner, and the recorded
training problem is built as the sweeps build it."""
import numpy as np

from oracle import mlp as M


def synthetic_problem(N=40, B=3, seed=0):
    rng = np.random.default_rng(seed)
    D = rng.standard_normal(N) * 2.0
    theta = np.sort(rng.standard_normal(B))
    X, _ = np.linalg.qr(rng.standard_normal((N, B)))
    R = rng.standard_normal((N, B))
    R -= X @ (X.T @ R)
    V = rng.standard_normal((N, B))
    V -= X @ (X.T @ V)
    return D, theta, X, R, V


def test_gradient_matches_central_differences():
    dims = M.widths(6, 2)
    flat = M.init_params(6, 2, seed=3).astype(np.float64)
    rng = np.random.default_rng(1)
    flat += 0.3 * rng.standard_normal(flat.shape)    # non-trivial output layer
    D, theta, X, R, V = synthetic_problem()
    loss, g = M.loss_grad(flat, dims, D, theta, X, R, V)
    assert 0.0 <= loss <= 1.0
    for k in rng.choice(len(flat), size=25, replace=False):
        e = np.zeros_like(flat)
        e[k] = 1e-6
        lp, _ = M.loss_grad(flat + e, dims, D, theta, X, R, V)
        lm, _ = M.loss_grad(flat - e, dims, D, theta, X, R, V)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def test_untrained_network_is_the_classical_preconditioner():
    dims = M.widths(16, 3)
    flat = M.init_params(16, 3, seed=0)
    D, theta, X, R, _ = synthetic_problem(N=50, B=2, seed=2)
    T = M.apply_prec(flat, dims, D, theta, R)
    s = np.max(np.abs(D[:, None] - theta[None, :]), axis=0)
    q = np.clip(s[None, :] / (D[:, None] - theta[None, :]), -M.QCLIP, M.QCLIP)
    assert np.allclose(T, q * R / s[None, :], rtol=1e-12, atol=0)


def test_training_problem_targets_the_converged_block():
    rng = np.random.default_rng(5)
    N, B = 30, 3
    Hm = rng.standard_normal((N, N))
    Hm = Hm + Hm.T
    w, U = np.linalg.eigh(Hm)
    Xs = U[:, :B]
    X0 = Xs + 0.05 * rng.standard_normal((N, B))
    theta, X, R, V = M.training_problem(np.diag(Hm), X0, lambda Y: Hm @ Y, Xs)
    assert np.allclose(X.T @ X, np.eye(B), atol=1e-12)
    assert np.allclose(X.T @ R, 0.0, atol=1e-10)
    assert np.allclose(X.T @ V, 0.0, atol=1e-12)
    # the correction V lies in span(Xs) + span(X)
    P = np.hstack([Xs, X])
    res = V - P @ np.linalg.lstsq(P, V, rcond=None)[0]
    assert np.linalg.norm(res) < 1e-10
