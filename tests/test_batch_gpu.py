"""Batched eigen sweeps (many independent chains on worker threads with one
stream each) give each chain the result of its own tt_eigb call.

Bar: eigenvalues to 1e-10 relative (exact ranks: rmax covers every bond of
these chains, so the sweeps have one fixed point) and the same ranks."""
import numpy as np
import pytest

from ttgpu.operators import xxz_mpo, random_tt

pytestmark = pytest.mark.gpu


def _chains(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for c in range(count):
        d = int(rng.integers(6, 11))
        delta = float(rng.uniform(0.5, 1.5))
        B = int(rng.choice([2, 4]))
        method = "split" if c % 3 == 2 else "plain"
        n, m, ra, crA = xxz_mpo(d, delta=delta)
        _, ry, cr = random_tt(d, 2, 8, last=B, seed=100 + c)
        out.append((d, n, m, ra, crA, cr, ry, B, method))
    return out


def test_batch_matches_single_chain_calls(ctx):
    import ttgpu
    chains = _chains(10, seed=4)
    batch = ttgpu.EigbBatch(nworkers=4, ctx=ctx)
    for (d, n, m, ra, crA, cr, ry, B, method) in chains:
        batch.add(d, n, m, ra, crA, cr, ry, 1e-10, 32, B, nswp=10, max_full_size=100, method=method)
    batch.run()
    for i, (d, n, m, ra, crA, cr, ry, B, method) in enumerate(chains):
        lam_b, _, ry_b, st = batch.result(i)
        lam_s, _, ry_s = ttgpu.tt_eigb(d, n, m, ra, crA, cr, ry, 1e-10, 32, B, nswp=10,
                                       max_full_size=100, method=method, ctx=ctx)
        assert np.allclose(lam_b, lam_s, rtol=1e-10, atol=0), (i, lam_b, lam_s)
        assert ry_b == ry_s
        assert st["matvecs"] > 0
    batch.close()


def test_batch_reports_a_failing_chain(ctx):
    """A chain whose local problem is smaller than its block fails on its own;
    the others still run and the batch returns the failing chain's status."""
    import ttgpu
    d, n, m, ra, crA, cr, ry, B, _ = _chains(1, seed=5)[0]
    batch = ttgpu.EigbBatch(nworkers=2, ctx=ctx)
    batch.add(d, n, m, ra, crA, cr, ry, 1e-8, 32, B, nswp=4, max_full_size=100)
    n2, m2, ra2, crA2 = xxz_mpo(2)
    _, ry2, cr2 = random_tt(2, 2, 1, last=4, seed=9)       # ranks [1, 1, 4]: N = 2 < B = 4
    batch.add(2, n2, m2, ra2, crA2, cr2, ry2, 1e-8, 32, 4, nswp=4, max_full_size=100)
    with pytest.raises(RuntimeError):
        batch.run()
    lam, _, _, _ = batch.result(0)
    assert np.all(np.isfinite(lam))
    with pytest.raises(RuntimeError):
        batch.result(1)
    batch.close()
