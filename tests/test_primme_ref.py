"""The oracle pinned to the reference's own eigensolver (CPU, no GPU).

tt_eigb's local eigensolver is the vendored PRIMME (tt_eigb.f90:252-283).
oracle/build_ref.py compiles those C sources unchanged (from the tt-fort
source tree) into oracle/_ref/; these tests run it and check the oracle's
Davidson restatement against it, and check the committed PRIMME golden
fixtures.  Without the tt-fort source tree (a machine with only this
repository) the tests that run PRIMME skip; the fixture checks still run."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import primme
from oracle.davidson import davidson
from oracle.eigb import tt_eigb
from oracle.ops import bfun3_block, flat, F
from ttgpu.operators import xxz_mpo, random_tt

needs_primme = pytest.mark.skipif(not primme.available(),
                                  reason="tt-fort source tree absent: PRIMME not built")


@needs_primme
@pytest.mark.parametrize("method", ["GD_plusK", "DYNAMIC"])
def test_primme_dense_known_spectrum(method):
    rng = np.random.default_rng(0)
    N, B = 300, 5
    Q = np.linalg.qr(rng.standard_normal((N, N)))[0]
    w = np.sort(rng.uniform(-3, 3, N))
    H = Q @ np.diag(w) @ Q.T
    lam, V, rn, nmv, ierr = primme.dprimme(lambda X: H @ X, N, B, rng.standard_normal((N, B)),
                                           1e-10, method=method)
    assert ierr == 0
    assert np.max(np.abs(lam - w[:B])) < 1e-12
    assert np.linalg.norm(H @ V - V * lam) < 1e-8


def _local_mv(p):
    r1, nn, r2, ra1, ra2 = (int(v) for v in p["dims"])
    N = r1 * nn * r2

    def mv(X):
        X = np.asarray(X).reshape(N, -1, order="F")
        k = X.shape[1]
        return F(bfun3_block(r1, nn, r2, r1, nn, r2, ra1, ra2, p["phi1"], p["A"], p["phi2"],
                             flat(X), k), N, k)
    return mv, N


@needs_primme
def test_oracle_davidson_matches_primme_on_sweep_problems():
    """Local problems recorded from a truncated XXZ sweep: the oracle's
    block Davidson and PRIMME (GD+k, tt_eigb's settings) reach the same
    eigenvalues to 1e-10 relative, each below its residual tolerance."""
    d, B = 12, 4
    n, m, ra, crA = xxz_mpo(d, delta=0.8)
    _, ry, cr = random_tt(d, 2, 8, last=B, seed=5)
    rec = []
    tt_eigb(d, n, m, ra, crA, cr, ry, 1e-9, 24, B, nswp=1, max_full_size=100, record=rec)
    assert len(rec) >= 4
    for p in rec[::max(1, len(rec) // 4)]:
        mv, N = _local_mv(p)
        lp, Vp, rp, _, ierr = primme.dprimme(mv, N, B, p["X0"], p["tol"])
        assert ierr == 0
        ld, Vd, rd, _, _ = davidson(mv, np.array(p["X0"]), B, p["tol"], max_matvecs=500)
        assert np.max(np.abs(ld - lp) / np.abs(lp)) < 1e-10
        scale = np.max(np.abs(lp))
        assert np.all(rp <= p["tol"] * scale * 1.01)


@needs_primme
def test_oracle_sweep_on_primme_matches_davidson_sweep():
    """A whole tt_eigb sweep with PRIMME as the local solver (the reference's
    configuration, GD+k pinned) and the same sweep on the oracle's Davidson:
    same sweeps, same ranks, eigenvalues to 1e-10 relative."""
    d, B = 12, 4
    n, m, ra, crA = xxz_mpo(d, delta=1.0)
    _, ry, cr = random_tt(d, 2, 8, last=B, seed=6)
    a = tt_eigb(d, n, m, ra, crA, cr, ry, 1e-9, 24, B, nswp=6, max_full_size=100,
                local_solver=primme.local_solver("GD_plusK"))
    b = tt_eigb(d, n, m, ra, crA, cr, ry, 1e-9, 24, B, nswp=6, max_full_size=100)
    assert a["sweeps"] == b["sweeps"] and a["ry"] == b["ry"]
    assert np.max(np.abs(a["lambda"] - b["lambda"]) / np.abs(a["lambda"])) < 1e-10


def test_primme_golden_agrees_with_oracle_and_ed():
    """The committed PRIMME sweep of the d=20 Heisenberg workload
    (make_primme_golden.py) against the oracle's own sweep and exact
    diagonalisation: GD+k and DYNAMIC land on the same eigenvalues."""
    g = json.load(open(os.path.join(GOLDEN, "eigb_heisen20_primme.json")))
    o = json.load(open(os.path.join(GOLDEN, "eigb_heisen20_oracle.json")))
    ed = json.load(open(os.path.join(GOLDEN, "heisen20_ed.json")))["eigenvalues"]
    for meth in ("GD_plusK", "DYNAMIC"):
        lam = np.array(g[meth]["lambda"])
        assert g[meth]["ierr"] == [0]
        assert np.max(np.abs(lam - o["lambda"]) / np.abs(lam)) < 1e-10
        assert np.max(np.abs(lam - ed[:5])) < 5e-7


def test_primme_local_fixture_matches_oracle_davidson():
    """The committed local problems (the largest of the sweep, N = 8192, and
    one of N = 4096): PRIMME's eigenvalues from the stored start, with
    residuals below the tolerance it was given, equal the oracle Davidson's
    from the same start to 1e-10 relative."""
    z = np.load(os.path.join(GOLDEN, "primme_local_heisen20.npz"))
    for q in range(2):
        p = {k: z[f"p{q}_{k}"] for k in ("dims", "phi1", "A", "phi2")}
        mv, N = _local_mv(p)
        lam, tol = z[f"p{q}_lambda"], float(z[f"p{q}_tol"])
        B = lam.size
        assert np.all(z[f"p{q}_rnorms"] <= tol * np.max(np.abs(lam)) * 1.01)
        X0 = F(z[f"p{q}_X0"], N, B)
        ld, _, _, _, _ = davidson(mv, X0.copy(), B, tol, max_matvecs=500)
        assert np.max(np.abs(ld - lam) / np.abs(lam)) < 1e-10
