"""Independent chains over several ranks (one process per GPU), host side.

A single sweep does not shard: every local step needs the interfaces that the
step before produced (tt_eigb.f90:353,392; ttamen.f90:217-218).  Many
independent chains do: they are partitioned over the ranks by estimated cost,
each rank solves its share on its own GPU (one chain after another, or all of
them through ``EigbBatch``), and the results are gathered on the host.  No
collective touches the data path; the only collectives are the result gather
and the max-over-ranks timing.

Every function works without ``torch.distributed`` initialised (one rank).
"""
import heapq


def _world(group=None):
    try:
        import torch.distributed as dist
    except ImportError:                                   # pragma: no cover
        return 0, 1, None
    if not dist.is_available() or not dist.is_initialized():
        return 0, 1, None
    return dist.get_rank(group), dist.get_world_size(group), dist


def chain_cost(n, ra, r):
    """Estimated work of one sweep of a chain with mode sizes n (d), operator
    ranks ra (d+1) and TT ranks r (d+1): the local matvec of core k costs
    about r_k r_{k+1} n_k (r_k ra_k + r_{k+1} ra_{k+1}) multiply-adds, the
    r^3 n ra scaling of the sweep."""
    d = len(n)
    return float(sum(r[k] * r[k + 1] * n[k] * (r[k] * ra[k] + r[k + 1] * ra[k + 1])
                     for k in range(d)))


def partition(costs, world):
    """Longest-processing-time assignment: chains in decreasing cost, each to
    the rank with the least load so far (ties to the lower rank).  Returns one
    ascending index list per rank; every index appears exactly once."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, q) for q in range(world)]
    parts = [[] for _ in range(world)]
    for i in order:
        load, q = heapq.heappop(heap)
        parts[q].append(i)
        heapq.heappush(heap, (load + float(costs[i]), q))
    return [sorted(p) for p in parts]


def run_partitioned(jobs, solve=None, solve_many=None, costs=None, group=None):
    """Solve ``jobs`` spread over the ranks and return every result, in job
    order, on every rank.

    ``solve(job)`` solves one job; ``solve_many(list_of_jobs)`` solves a
    rank's whole share at once (e.g. through ``EigbBatch``) and returns the
    results in the same order.  ``costs`` (default: equal) feed
    :func:`partition`.  A rank whose solver raises still takes part in the
    gather, so no rank waits on it; afterwards every rank raises
    ``RuntimeError`` naming the first failing job."""
    if (solve is None) == (solve_many is None):
        raise ValueError("give exactly one of solve and solve_many")
    rank, world, dist = _world(group)
    parts = partition(costs if costs is not None else [1.0] * len(jobs), world)
    mine = parts[rank]
    local = {"ok": {}, "err": None}
    try:
        if solve_many is not None:
            res = solve_many([jobs[i] for i in mine])
            if len(res) != len(mine):
                raise RuntimeError("solve_many returned %d results for %d jobs"
                                   % (len(res), len(mine)))
            local["ok"] = dict(zip(mine, res))
        else:
            for i in mine:
                try:
                    local["ok"][i] = solve(jobs[i])
                except Exception as e:            # noqa: BLE001  (reported to every rank)
                    local["err"] = (i, rank, repr(e))
                    break
    except Exception as e:                        # noqa: BLE001
        local["err"] = (mine[0] if mine else -1, rank, repr(e))
    if world > 1:
        gathered = [None] * world
        dist.all_gather_object(gathered, local, group=group)
    else:
        gathered = [local]
    errs = [g["err"] for g in gathered if g["err"] is not None]
    if errs:
        i, q, msg = min(errs)
        raise RuntimeError("chain %d failed on rank %d: %s" % (i, q, msg))
    merged = {}
    for g in gathered:
        merged.update(g["ok"])
    return [merged[i] for i in range(len(jobs))]


def max_over_ranks(values, group=None):
    """Element-wise maximum of a list of floats over the ranks (the timing
    rule: a step takes as long as its slowest rank).  NCCL groups reduce on
    the current CUDA device, others on the host."""
    rank, world, dist = _world(group)
    vals = [float(v) for v in values]
    if world == 1:
        return vals
    import torch
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor(vals, dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return [float(v) for v in t.cpu().tolist()]
