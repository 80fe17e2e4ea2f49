"""Block 1-norm estimator used by the KSL integrator (oracle).

Test infrastructure only (see ``oracle/__init__.py``).  Restates
``znormest_higham`` (expm/normest.f90:52-94) driving ``ZLACN1``
(expm/zlacn1.f, Higham & Tisseur's block estimator, t = 4 columns,
ITMAX = 5) step by step, including two behaviours of the reference:

* the S-step adjoint product writes into its input (``zsfun_matvec_transp``,
  tt_ksl.f90:154-164), so the reference's estimator sees the sign matrix
  itself where Z = A^H X is expected; ``transp=None`` reproduces that;
* the history of visited unit vectors is stored only at positions beyond n
  (zlacn1.f label 140, as written there), so an index counts as visited only
  once the history scan runs past n.

Two choices are made where the reference depends on third-party code that is
not part of it: the random start columns come from ``unit_randoms`` below (a
splitmix64 stream mapped to the unit circle) instead of LAPACK's ZLARNV, and
the descending sort (DLAPST) breaks ties by the lower index.  Both the oracle
and the CUDA library use these same definitions, so their step sizes agree.
"""
import numpy as np

GOLD = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)


def unit_randoms(counter0, count):
    """exp(2 pi i u_k), u_k from splitmix64(counter0 + k + 1), k < count."""
    k = np.arange(count, dtype=np.uint64) + np.uint64(counter0 + 1)
    with np.errstate(over="ignore"):
        z = k * GOLD
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    ang = 2.0 * np.pi * u
    return np.cos(ang) + 1j * np.sin(ang)


class Seed:
    """Stateful stream position (the reference's module variable iseed)."""

    def __init__(self):
        self.counter = 0


def znormest(n, t0, matvec, transp, seed, itmax=5):
    """Estimate ||A||_1.  matvec/transp map an (n, t) block column by column;
    transp=None reproduces the S-step estimator (Z = X)."""
    t = min(n, t0)
    X = np.zeros((n, t), dtype=np.complex128)
    X[:, 0] = 1.0
    for j in range(1, t):
        X[:, j] = unit_randoms(seed.counter, n)
        seed.counter += n
    X *= 1.0 / n
    ind = np.arange(n)
    indh = np.full(n, -1)
    estold = 0.0
    ibest = 0
    it = 1
    X = matvec(X)
    while True:
        # zlacn1.f label 30
        if it == 1 and n == 1:
            return abs(X[0, 0])
        colsum = np.abs(X).sum(axis=0)
        itemp = int(np.argmax(colsum))          # first maximum, as the > scan
        est = float(colsum[itemp])
        if est > estold or it == 2:
            ibest = int(ind[itemp])
        if est <= estold and it >= 2:
            return estold
        estold = est
        if it > itmax:
            return est
        ax = np.abs(X)
        S = np.where(ax > np.finfo(float).tiny, X / np.where(ax > 0, ax, 1.0), 1.0 + 0j)
        X = S.copy() if transp is None else transp(S)
        # label 70
        h = np.abs(X).max(axis=1)
        ind = np.arange(n)
        if it >= 2 and h[int(np.argmax(h))] == h[ibest]:
            return est
        order = np.argsort(-h, kind="stable")
        h = h[order]
        ind = ind[order]
        # zlacn1.f labels 90-140.  The history INDH(1..N) is never written
        # (entries are stored only at positions beyond N) and an index counts
        # as visited exactly when the scan passes position N, i.e. when
        # (iter-1)*t > n; so either every index is new or all are visited.
        if it >= 2 and t > 1 and (it - 1) * t > n:
            return est
        X = np.zeros((n, t), dtype=np.complex128)
        for j in range(t):
            X[ind[j], j] = 1.0
        it += 1
        X = matvec(X)
