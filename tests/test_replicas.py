"""CPU tests of the multi-rank host path: chains partitioned over ranks, the
result gather, the max-over-ranks timing and failure reporting, run as two
``gloo`` ranks.  The per-chain solver here is a dense eigensolver of small
chains (no GPU); the library's GPU solvers plug into the same hooks."""
import datetime
import os
import socket

import numpy as np
import pytest

from ttgpu.replicas import chain_cost, partition, run_partitioned, max_over_ranks


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _jobs(count, seed):
    """Small symmetric 'chains': (id, dense matrix); cost grows with size."""
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(count):
        k = int(rng.integers(4, 24))
        a = rng.standard_normal((k, k))
        jobs.append((i, a + a.T))
    return jobs


def _solve(job):
    i, a = job
    if i == 5 and os.environ.get("TTG_TEST_FAIL_JOB") == "5":
        raise ValueError("planted failure")
    return float(np.linalg.eigvalsh(a)[0])


def test_partition_covers_every_chain_once_and_balances():
    rng = np.random.default_rng(0)
    costs = rng.uniform(1, 100, size=57)
    for world in (1, 2, 3, 8):
        parts = partition(costs, world)
        assert len(parts) == world
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        # LPT: no rank exceeds the lightest by more than the largest chain
        assert max(loads) - min(loads) <= max(costs) + 1e-9
    assert partition([], 4) == [[], [], [], []]
    with pytest.raises(ValueError):
        partition([1.0], 0)


def test_chain_cost_grows_with_rank():
    n, ra = [2] * 6, [1, 5, 5, 5, 5, 5, 1]
    c8 = chain_cost(n, ra, [1, 2, 4, 8, 4, 2, 1])
    c16 = chain_cost(n, ra, [1, 2, 4, 16, 4, 2, 1])
    assert c16 > c8 > 0


def test_single_rank_without_process_group():
    jobs = _jobs(7, 1)
    out = run_partitioned(jobs, solve=_solve)
    assert out == [_solve(j) for j in jobs]
    assert max_over_ranks([1.5, 2.0]) == [1.5, 2.0]
    with pytest.raises(ValueError):
        run_partitioned(jobs)


def _worker(rank, world, port, mode, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    if mode == "fail":
        os.environ["TTG_TEST_FAIL_JOB"] = "5"
    # a short process-group timeout: a rank that never arrives fails the
    # collective (and the test) instead of hanging it
    dist.init_process_group("gloo", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=60))
    try:
        jobs = _jobs(11, 2)
        costs = [float(j[1].shape[0]) ** 3 for j in jobs]
        if mode == "ok":
            out = run_partitioned(jobs, solve=_solve, costs=costs)
            many = run_partitioned(jobs, solve_many=lambda js: [_solve(j) for j in js],
                                   costs=costs)
            t = max_over_ranks([0.1 * (rank + 1), 3.0 - rank])
            np.save(os.path.join(outdir, "r%d.npy" % rank), np.array(out + many + t))
        else:
            try:
                run_partitioned(jobs, solve=_solve, costs=costs)
                msg = "no error"
            except RuntimeError as e:
                msg = str(e)
            with open(os.path.join(outdir, "r%d.txt" % rank), "w") as f:
                f.write(msg)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("mode", ["ok", "fail"])
def test_two_gloo_ranks(tmp_path, mode):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(2, _free_port(), mode, str(tmp_path)), nprocs=2, join=True)
    jobs = _jobs(11, 2)
    if mode == "ok":
        ref = [_solve(j) for j in jobs]
        for rank in range(2):
            got = np.load(str(tmp_path / ("r%d.npy" % rank)))
            assert np.array_equal(got[:11], ref)          # every rank holds every result
            assert np.array_equal(got[11:22], ref)
            assert np.allclose(got[22:], [0.2, 3.0])       # max over ranks
    else:
        for rank in range(2):
            msg = (tmp_path / ("r%d.txt" % rank)).read_text()
            assert msg.startswith("chain 5 failed on rank"), msg
            assert "planted failure" in msg
