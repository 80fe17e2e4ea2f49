"""Models, on the CPU, of the two choices the device truncation SVD makes
(ttg_linalg.cu): (1) the factor assembly of the twice-preconditioned one-sided
Jacobi, with the kernels' permutation and transpose conventions; (2) the
rotation angle taken in FP32 with c = 1/sqrt(1 + t^2), s = c t formed in
FP64: the rotations stay orthogonal to FP64 precision, and the sweeps and the
singular values come out as with FP64 angles."""
import numpy as np
import pytest


def _jacobi(M, fp32_angle):
    """One-sided Jacobi with the device's round-robin order and thresholds."""
    M = M.copy()
    p, q = M.shape
    K = q + (q & 1)
    tol, tolc = np.sqrt(p) * 2.2e-16, p * 2.2e-16
    for sweep in range(60):
        counted = 0
        for r in range(K - 1):
            for i in range(K // 2):
                a, b = (r, K - 1) if i == 0 else ((r + i) % (K - 1), (r - i + K - 1) % (K - 1))
                if a >= q or b >= q:
                    continue
                x, y = M[:, a].copy(), M[:, b].copy()
                A, Bv, G = x @ x, y @ y, x @ y
                if G == 0 or G * G <= tol * tol * A * Bv:
                    continue
                zeta = (Bv - A) / (2 * G)
                if fp32_angle and abs(zeta) < 1e18:
                    z = np.float32(zeta)
                    t = float(np.copysign(np.float32(1) / (np.float32(abs(z)) +
                                                           np.sqrt(np.float32(1) + z * z)), z))
                elif fp32_angle:
                    t = 0.5 / zeta
                else:
                    t = np.sign(zeta or 1.0) / (abs(zeta) + np.sqrt(1 + zeta * zeta))
                c = 1 / np.sqrt(1 + t * t)
                s = c * t
                if G * G > tolc * tolc * A * Bv:
                    counted += 1
                M[:, a], M[:, b] = c * x - s * y, s * x + c * y
        if counted == 0:
            return np.sort(np.linalg.norm(M, axis=0))[::-1], sweep + 1
    return np.sort(np.linalg.norm(M, axis=0))[::-1], 60


@pytest.mark.parametrize("q,lo", [(24, -13), (20, -3)])
def test_fp32_angle_sweeps_and_values_match_fp64_angle(q, lo):
    rng = np.random.default_rng(q)
    p = 2 * q
    U = np.linalg.qr(rng.standard_normal((p, q)))[0]
    W = np.linalg.qr(rng.standard_normal((q, q)))[0]
    M = (U * np.logspace(0, lo, q)) @ W.T
    R = np.linalg.qr(M[:, np.argsort(-np.linalg.norm(M, axis=0))], mode="r").T
    ref = np.linalg.svd(R, compute_uv=False)
    s64, n64 = _jacobi(R, False)
    s32, n32 = _jacobi(R, True)
    assert abs(n32 - n64) <= 1
    big = ref > 1e-10 * ref[0]
    assert np.max(np.abs(s32 - ref)[big] / ref[big]) < 1e-13
    assert np.max(np.abs(s64 - ref)[big] / ref[big]) < 1e-13


def test_two_qr_factor_assembly():
    """M P = Q1 R1 (columns sorted by norm: A[:, rank[j]] = M[:, j]),
    R1^T = Q2 R2, R2^T = U2 S V2^T: U = Q1 [U2; 0] and
    Vt[k, j] = (Q2 V2)[rank[j], k] (the qr_vt_kernel map)."""
    rng = np.random.default_rng(1)
    p, q = 40, 17
    M = rng.standard_normal((p, q)) * np.logspace(0, -6, q)
    nrm = np.linalg.norm(M, axis=0)
    rank = np.array([sum((nrm[t] > nrm[j]) or (nrm[t] == nrm[j] and t < j) for t in range(q))
                     for j in range(q)])
    A = np.zeros_like(M)
    A[:, rank] = M
    Q1, R1 = np.linalg.qr(A)
    Q2, R2 = np.linalg.qr(R1.T)
    U2, S, V2t = np.linalg.svd(R2.T)
    U = Q1 @ U2
    W = Q2 @ V2t.T
    Vt = np.array([[W[rank[j], k] for j in range(q)] for k in range(q)])
    assert np.linalg.norm(U * S @ Vt - M) <= 1e-14 * np.linalg.norm(M)
    assert np.linalg.norm(U.T @ U - np.eye(q)) < 1e-13
    assert np.linalg.norm(Vt @ Vt.T - np.eye(q)) < 1e-13
