"""The core-contracted form of the split local operator, as index algebra on
the CPU: the operand orders its kernels use (build_q_kernel's Q rows and K,
the X tile rows, the epilogue's map of a product element into the last
product's operand T2) reproduce dbfun3 (ttals.f90:9-32) in FP64.  The GPU
kernels implement exactly these maps; test_split_gpu.py checks them on the
device against the same oracle."""
import numpy as np
import pytest

from oracle import ops


def _core_contracted(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, X, nvec):
    MQ, KQ, NX = n * ry2 * ra1, m * rx2, rx1 * nvec
    # Q[mq, kq] = sum_a2 A(a1,i,j,a2) Phi2(b2,a2,c2), mq = (i + n c2) + n ry2 a1, kq = j + m b2
    Q = np.zeros((MQ, KQ))
    for r in range(MQ):
        ic2, a1 = r % (n * ry2), r // (n * ry2)
        i, c2 = ic2 % n, ic2 // n
        for kq in range(KQ):
            j, b2 = kq % m, kq // m
            Q[r, kq] = sum(A[a1 + ra1 * (i + n * j) + ra1 * n * m * a2] *
                           phi2[b2 + rx2 * ra2 * c2 + rx2 * a2] for a2 in range(ra2))
    # X rows (b1, v), K (j, b2): element x_v[b1 + rx1 * kq]
    xs = rx1 * m * rx2
    Xm = np.array([[X[(row // rx1) * xs + row % rx1 + k * rx1] for k in range(KQ)]
                   for row in range(NX)])
    Z = Q @ Xm.T
    # epilogue: product (mq, nx) -> T2 row (i + n c2) + n ry2 v, K b1 + rx1 a1
    N3, K3 = n * ry2 * nvec, rx1 * ra1
    T2 = np.zeros((N3, K3))
    for row in range(MQ):
        ic2, kb = row % (n * ry2), rx1 * (row // (n * ry2))
        for nx in range(NX):
            T2[ic2 + n * ry2 * (nx // rx1), nx % rx1 + kb] = Z[row, nx]
    P1 = np.array([[phi1[c1 + ry1 * k] for k in range(K3)] for c1 in range(ry1)])
    return (P1 @ T2.T).ravel(order="F")      # y[c1 + ry1 * (i, c2, v)]


@pytest.mark.parametrize("shape", [(16, 2, 12, 9, 2, 10, 3, 4, 3), (8, 1, 5, 7, 2, 6, 1, 5, 2),
                                   (24, 2, 8, 16, 2, 8, 5, 1, 2), (8, 2, 7, 8, 2, 9, 2, 2, 1)])
def test_core_contracted_form_reproduces_dbfun3(shape):
    rx1, m, rx2, ry1, n, ry2, ra1, ra2, nvec = shape
    rng = np.random.default_rng(sum(shape))
    phi1 = rng.standard_normal(ry1 * rx1 * ra1)
    A = rng.standard_normal(ra1 * n * m * ra2)
    phi2 = rng.standard_normal(rx2 * ra2 * ry2)
    X = rng.standard_normal(rx1 * m * rx2 * nvec)
    ref = ops.bfun3_block(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, X, nvec)
    got = _core_contracted(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, X, nvec)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
