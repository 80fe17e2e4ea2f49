"""Learned preconditioner of the local eigensolver (oracle).

Test infrastructure only (see ``oracle/__init__.py``).  There is no
counterpart in the reference: PRIMME's ``applyPreconditioner`` hook exists
but tt_eigb leaves it unset (primme/primme.h:144-145, tt_eigb.f90:252-283),
so the reference expands the Davidson basis with plain residuals.  The
library corrects the classical diagonal (Davidson) preconditioner with a ReLU
multilayer perceptron evaluated per entry of the local problem:

  D       diagonal of the local operator, theta_j Ritz value of column j
  s_j     = max_i |D_i - theta_j|
  q_ij    = clip(s_j / (D_i - theta_j), -100, 100)
  feats   = [(D_i - theta_j)/s_j, r_ij sqrt(N)/||r_j||, q_ij/100]
  t_ij    = q_ij (1 + h_ij) r_ij / s_j       (r_ij where not finite)

with h = MLP(feats); the output layer starts at zero, so the untrained
network is the classical preconditioner.  Training pairs are recorded from
plain sweeps: the start Ritz block X (N x B) of a local problem with values
theta and residuals R, and V = X* Q - X projected off span(X), X* the
converged block and Q the orthogonal Procrustes rotation onto X.  The loss
of one problem is mean_j (1 - cos^2(P t_j, V_j)), P = I - X X^T.

Network: widths [3, w, ..., w, 1], parameters flat layer by layer (W_l in x
out row-major, then b_l), He-normal weights from the splitmix64/Box-Muller
stream, Adam (0.9, 0.999, 1e-8).
"""
import numpy as np

NFEAT = 3
QCLIP = 100.0


def widths(width, depth):
    return [NFEAT] + [width] * depth + [1]


def init_params(width, depth, seed):
    """Flat float32 parameters as ``ttg_mlp_create`` builds them."""
    from .amen import sm_normals
    dims = widths(width, depth)
    nw = sum(dims[l] * dims[l + 1] for l in range(len(dims) - 1))
    z = sm_normals(seed, nw)
    out = []
    zi = 0
    for l in range(len(dims) - 1):
        k, n = dims[l], dims[l + 1]
        W = z[zi:zi + k * n] * np.sqrt(2.0 / k)
        zi += k * n
        if l == len(dims) - 2:
            W = np.zeros_like(W)
        out.append(W.astype(np.float32))
        out.append(np.zeros(n, dtype=np.float32))
    return np.concatenate(out)


def unflatten(flat, dims):
    params = []
    off = 0
    for l in range(len(dims) - 1):
        k, n = dims[l], dims[l + 1]
        W = flat[off:off + k * n].reshape(k, n)
        off += k * n
        b = flat[off:off + n]
        off += n
        params.append((W, b))
    return params


def flatten(grads):
    return np.concatenate([np.concatenate([gW.ravel(), gb.ravel()]) for gW, gb in grads])


def to_bf16(x):
    """float32 values rounded to the nearest bfloat16 (ties to even), as
    float32 -- the rounding of __float2bfloat16_rn on finite values."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def _mm(a, b, bf16):
    """a @ b in float64 on operands rounded to bf16 (bf16=True, the library's
    tensor-core products: exact bf16 products summed in FP32), or as given."""
    if not bf16:
        return a @ b
    return (to_bf16(a).astype(np.float64) @ to_bf16(b).astype(np.float64)).astype(np.float32)


def forward(params, Fx, bf16=False):
    """Network output (P,) and the layer inputs/outputs, in the parameters'
    precision (float32 as on the device; float64 for derivative checks).
    bf16=True rounds both operands of every layer product to bf16, as the
    tensor-core path does."""
    dt = params[0][0].dtype
    acts = [np.asarray(Fx, dtype=dt)]
    h = acts[0]
    L = len(params)
    for l, (W, b) in enumerate(params):
        z = _mm(h, W, bf16) + b
        h = (np.maximum(z, 0.0) if l < L - 1 else z).astype(dt)
        acts.append(h)
    return acts[-1][:, 0], acts


def local_diag(rx1, n, rx2, ra1, ra2, phi1, A, phi2):
    """D(b1, j, b2) = sum_{a1,a2} Phi1(b1,b1,a1) A(a1,j,j,a2) Phi2(b2,a2,b2)."""
    p1 = np.asarray(phi1).reshape(rx1, rx1, ra1, order="F")
    A4 = np.asarray(A).reshape(ra1, n, n, ra2, order="F")
    p2 = np.asarray(phi2).reshape(rx2, ra2, rx2, order="F")
    a = np.einsum("bba->ba", p1)
    c = np.einsum("cac->ac", p2)
    Ad = np.einsum("ijja->ija", A4)
    return np.einsum("ba,aja,ac->bjc", a, Ad, c).reshape(-1, order="F")


def features(D, theta, R):
    """Features (N*t x 3, point p = i + N j) and the classical term base."""
    N, t = R.shape
    dd = D[:, None] - theta[None, :]
    s = np.max(np.abs(dd), axis=0)
    s = np.where(s > 0, s, 1.0)
    rn = np.linalg.norm(R, axis=0)
    rn = np.where(rn > 0, rn, 1.0)
    with np.errstate(divide="ignore"):
        q = np.where(dd != 0, s[None, :] / np.where(dd != 0, dd, 1.0), QCLIP)
    q = np.clip(q, -QCLIP, QCLIP)
    F = np.stack([dd / s[None, :], R * np.sqrt(N) / rn[None, :], q / QCLIP], axis=2)
    F = F.transpose(1, 0, 2).reshape(N * t, NFEAT).astype(np.float32)
    base = (q * R / s[None, :]).T.reshape(-1)
    return F, base


def apply_prec(flat, dims, D, theta, R):
    """The preconditioned expansion block T (N x t)."""
    N, t = R.shape
    F, base = features(D, theta, R)
    h, _ = forward(unflatten(flat, dims), F)
    T = (base * (1.0 + h.astype(np.float64))).reshape(t, N).T
    return np.where(np.isfinite(T), T, R)


def loss_grad(flat, dims, D, theta, X, R, V, bf16=False):
    """Loss of one recorded problem and the flat parameter gradient (bf16:
    every layer product of the forward and backward passes on bf16-rounded
    operands, as the tensor-core path computes them)."""
    params = unflatten(flat, dims)
    N, B = X.shape
    F, base = features(D, theta, R)
    h, acts = forward(params, F, bf16)
    u = (base * (1.0 + h.astype(np.float64))).reshape(B, N).T
    u = u - X @ (X.T @ u)
    uu = np.sum(u * u, axis=0)
    vv = np.sum(V * V, axis=0)
    uv = np.sum(u * V, axis=0)
    ok = (uu > 0) & (vv > 0)
    loss = float(np.mean(np.where(ok, 1.0 - uv * uv / np.where(ok, uu * vv, 1.0), 0.0)))
    coef = np.where(ok, -2.0 * uv / np.where(ok, uu * vv, 1.0) / B, 0.0)
    g = coef[None, :] * (V - (uv / np.where(uu > 0, uu, 1.0))[None, :] * u)
    g = g - X @ (X.T @ g)
    dh = (g.T.reshape(-1) * base).astype(params[0][0].dtype)
    gz = dh[:, None]
    grads = [None] * len(params)
    for l in range(len(params) - 1, -1, -1):
        W, b = params[l]
        a = acts[l]
        grads[l] = (_mm(a.T, gz, bf16), gz.sum(axis=0))
        if l > 0:
            gz = _mm(gz, W.T, bf16) * (acts[l] > 0)
    return loss, flatten(grads)


def training_problem(D, X0, mv, Xs):
    """(theta, X, R, V) of one local problem as the sweeps record it."""
    V0, _ = np.linalg.qr(X0)
    W = mv(V0)
    H = V0.T @ W
    theta, S = np.linalg.eigh(0.5 * (H + H.T))
    X = V0 @ S
    R = W @ S - X * theta
    U, _, Vt = np.linalg.svd(Xs.T @ X)
    Y = Xs @ (U @ Vt) - X
    Y = Y - X @ (X.T @ Y)
    return theta, X, R, Y
