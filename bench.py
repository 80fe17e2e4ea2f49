"""Benchmark of the tt_eigb sweep hot path on one GB300.

Workload (one "step"): the block eigensolver tt_eigb on the d=20 open-boundary
spin-1/2 Heisenberg chain (TT-matrix n=2, rank 5 -- the operator of the
reference fixture Heisen_20.sdv), B=5 lowest eigenpairs, random N(0,1) start
block with ranks 16 (seed 0), ranks capped at 64, eps=1e-8, max_full_size=200,
swept to convergence.  Metric: wall time of one full solve (lower is better).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--method plain|split]
                  [--workload heisenberg20|xxz100|amen10|ksl16|batch256|matvec|svd]

The default workload (heisenberg20) is the metric's.  Two larger workloads
are measured the same way, one timed run per method after a warm-up solve:
xxz100 = tt_eigb on the XXZ chain d=100, delta=1, B=8, ranks up to 256 (local
problems r^2 n = 131k), two sweeps; amen10 = the ttamen AMEn solve of
(Laplacian + exp(-|i-c|^2/sigma^2)) x = y, d=10, n=64, operator rank 3, rhs
rank 4, tol 1e-9, ranks up to 128, 20 sweeps; ksl16 = ztt_ksl, 200 steps of
tau=1e-3 of dx/dt = A x, A = -(Dirichlet Laplacian, d=16, n=32) + a random
rank-4 TT-matrix with N(0, 0.01^2) entries, x0 a random rank-8 TT vector of
norm 1, with the split state's relative error against the FP64 state;
batch256 = the batched chains (see batch_chains); matvec = the split and plain
local matvecs alone at r=64 (block 5) and r=256 (block 8); svd = the
truncation SVD alone at the two workloads' block shapes.

GPU arm: times K solves through the C-ABI with CUDA events on the library's
stream (value), the same solves end to end from pinned host buffers (e2e),
the dominant kernel's roofline from a local-matvec microbenchmark timed with
CUDA events, SM clocks sampled by nvidia-smi during the timed region, and the
CPU oracle timed on the host cores (cpu_baseline).  Reference arm: the CPU
restatement of tt_eigb (oracle/eigb.py, numpy + OpenBLAS on all host cores).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "tt-fort_gb300")]

import numpy as np  # noqa: E402

D, B, R0, RMAX, EPS, MFS = 20, 5, 16, 64, 1e-8, 200


def workload():
    from ttgpu.operators import xxz_mpo, random_tt
    n, m, ra, crA = xxz_mpo(D)
    _, ry, cr = random_tt(D, 2, R0, last=B, seed=0)
    return n, m, ra, crA, ry, cr


def config():
    return {"workload": f"tt_eigb heisenberg d={D} n=2 ra=5 B={B} start_rank={R0} rmax={RMAX} "
                        f"eps={EPS:g} max_full_size={MFS}",
            "d": D, "B": B, "rmax": RMAX, "eps": EPS, "n": 2, "ra": 5,
            "l2": "inputs < L2: 256 MiB buffer written between timed steps"}


def bfun3_flops(rx1, m, rx2, ry1, n, ry2, ra1, ra2):
    return 2 * rx1 * m * rx2 * ra2 * ry2 + 2 * ra1 * n * m * ra2 * ry2 * rx1 + 2 * ry1 * n * ry2 * rx1 * ra1


class ClockSampler:
    def __init__(self):
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 3 + k and r[3 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return json.load(open(p)), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def fp64_peak_tflops(torch):
    """cuBLAS DGEMM 4096^3 (torch.matmul float64), best of 5: the FP64 roof."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = 1e9
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2 * 4096 ** 3 / best / 1e12


# DRAM bytes (read + write) of one split block matvec at r=64, n=2, ra=5, 5
# vectors: the sum over its three launches (split X, the core-contracted first
# product, the last product) in one ncu capture
# (profiles/split_matvec_r64_b5_traffic.md), cold L2 per launch
SPLIT_MV_TRAFFIC = 337920 + 517632 + 1012992
SPLIT_MV_TRAFFIC_NOTE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum summed over the three "
                         "launches of one apply, cold L2 (profiles/split_matvec_r64_b5_traffic.md)")


def matvec_roofline(torch, ctx, split=False, r=RMAX, nvec=B):
    """Local matvec through a prepared operator (the form the solver calls)
    at the workload's largest local problem (r=64, n=2, ra=5, block of B
    vectors).  The applies are captured into a CUDA graph and the graph is
    replayed, so the figure is device time per apply (CUDA events on the
    capturing stream), not the host cost of launching from Python; the
    solver itself launches from C++ or from captured graphs."""
    import ttgpu
    n, ra = 2, 5
    rng = np.random.default_rng(0)
    phi1 = torch.from_numpy(rng.standard_normal(r * r * ra)).cuda()
    A = torch.from_numpy(rng.standard_normal(ra * n * n * ra)).cuda()
    phi2 = torch.from_numpy(rng.standard_normal(r * ra * r)).cuda()
    X = torch.from_numpy(rng.standard_normal(r * n * r * nvec)).cuda()
    Y = torch.zeros(r * n * r * nvec, dtype=torch.float64, device="cuda")
    prev = torch.cuda.current_stream()
    cap = torch.cuda.Stream()
    reps, replays = 50, 10
    with torch.cuda.stream(cap):
        ctx.bind_torch_stream()
        op = ttgpu.LocalOp(r, n, r, r, n, r, ra, ra, phi1, A, phi2, nvec_max=nvec,
                           method="split" if split else "plain", ctx=ctx)
        for _ in range(5):
            op.apply(X, Y, nvec)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=cap):
            for _ in range(reps):
                op.apply(X, Y, nvec)
        g.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(cap)
        for _ in range(replays):
            g.replay()
        e1.record(cap)
        torch.cuda.synchronize()
        op.close()
    torch.cuda.set_stream(prev)
    ctx.bind_torch_stream()
    dt = e0.elapsed_time(e1) / 1e3 / (reps * replays)
    return bfun3_flops(r, n, r, r, n, r, ra, ra) * nvec, dt


def _timed(torch, fn):
    """fn() bracketed by CUDA events on the current (library) stream."""
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    r = fn()
    e1.record()
    torch.cuda.synchronize()
    return r, e0.elapsed_time(e1) / 1e3


def config_block(args, torch, ttgpu, ctx):
    """The metric's other configurations, one timed run per method after a
    warm-up, each with its error against FP64 and against an oracle sample:

      ksl16  ztt_ksl, d=16, n=32, A = -(Dirichlet Laplacian) + rank-4
             N(0, 0.01^2) TT-matrix, x0 rank 8 of norm 1, 200 steps of 1e-3;
             oracle: 10 steps of the restatement against 10 PLAIN steps
      amen10 dtt_amen_solve, d=10, n=64, Laplacian + Gaussian potential,
             rhs rank 4, tol 1e-9, rmax 128, 20 sweeps; oracle: 6 sweeps of
             the restatement against 6 PLAIN sweeps from the same start
      xxz100 tt_eigb, XXZ d=100, delta=1, B=8, rmax 256, 2 sweeps per method
             (a converged run takes minutes: bench.py --workload xxz100)
    Differences of TT tensors are 2-norms of the difference tensor by QR
    sweeps.  CPU legs run only without --no-cpu."""
    from ttgpu.operators import (ksl_operator, random_tt_complex, tt_dot, tt_rel_diff,
                                 amen_operator, random_tt, xxz_mpo)
    out = {}
    def ksl16():
        d, nn = 16, 32
        n_, m_, ra, crA = ksl_operator(d=d, n=nn, rank=4, std=0.01, seed=1)
        _, ry, y = random_tt_complex(d, nn, 8, seed=2)
        y = y.copy()
        y[:ry[1] * nn] /= np.sqrt(tt_dot(d, n_, ry, y, ry, y).real)
        res = {}
        for meth in ("split", "plain"):
            ttgpu.ztt_ksl(d, n_, m_, ra, crA, y, ry, 1e-3, 64, nsteps=2, method=meth, ctx=ctx)
            (c, r), t = _timed(torch, lambda: ttgpu.ztt_ksl(d, n_, m_, ra, crA, y, ry, 1e-3, 64,
                                                             nsteps=args.ksl_steps, method=meth,
                                                             ctx=ctx))
            res[meth] = {"cores": c, "ry": r, "time": t, "launches": ctx.stats()["launches"]}
        sp, pl = res["split"], res["plain"]
        e = {"workload": f"ztt_ksl d=16 n=32 ra=6 ry=8 tau=1e-3 nsteps={args.ksl_steps}",
             "chosen_s": sp["time"], "plain_s": pl["time"], "plain_over_chosen": pl["time"] / sp["time"],
             "gpu_launches": {"chosen": int(sp["launches"]), "plain": int(pl["launches"])},
             "chosen_vs_fp64": tt_rel_diff(d, n_, sp["ry"], sp["cores"], pl["ry"], pl["cores"])}
        if not args.no_cpu:
            from oracle.ksl import ztt_ksl as oracle_ksl
            c_, r_ = y, list(ry)
            t0 = time.perf_counter()
            for _ in range(10):
                o = oracle_ksl(d, n_, m_, ra, crA, c_, r_, 1e-3, 64)
                c_, r_ = o["cores"], o["ry"]
            tc = time.perf_counter() - t0
            g10, gr10 = ttgpu.ztt_ksl(d, n_, m_, ra, crA, y, ry, 1e-3, 64, nsteps=10, method="plain",
                                      ctx=ctx)
            s10, sr10 = ttgpu.ztt_ksl(d, n_, m_, ra, crA, y, ry, 1e-3, 64, nsteps=10, method="split",
                                      ctx=ctx)
            e["oracle_sample"] = {"steps": 10, "seconds": tc, "cores": os.cpu_count(),
                                  "plain_vs_oracle": tt_rel_diff(d, n_, gr10, g10, r_, c_),
                                  "chosen_vs_oracle": tt_rel_diff(d, n_, sr10, s10, r_, c_)}
        return e

    def amen10():
        d, nn = 10, 64
        n_, m_, ra, crA = amen_operator(d=d, n=nn)
        _, ry, y = random_tt(d, nn, 4, seed=3)
        _, rx, x0 = random_tt(d, nn, 2, seed=7)
        res = {}
        for meth in ("split", "plain"):
            ttgpu.dtt_amen_solve(d, n_, m_, ry, ra, crA, y, x0, rx, 1e-9, rmax=128, nswp=2,
                                 method=meth, ctx=ctx)
            (c, r), t = _timed(torch, lambda: ttgpu.dtt_amen_solve(d, n_, m_, ry, ra, crA, y, x0, rx,
                                                                    1e-9, rmax=128, nswp=20,
                                                                    method=meth, ctx=ctx))
            st = ctx.stats()
            res[meth] = {"cores": c, "rx": r, "time": t, "res": st["res"], "sweeps": st["sweeps"],
                         "launches": st["launches"]}
        sp, pl = res["split"], res["plain"]
        e = {"workload": "dtt_amen_solve d=10 n=64 ra=3 ry=4 rx0=2 tol=1e-9 rmax=128 nswp=20",
             "chosen_s": sp["time"], "plain_s": pl["time"], "plain_over_chosen": pl["time"] / sp["time"],
             "sweeps": {"chosen": sp["sweeps"], "plain": pl["sweeps"]},
             "local_residual_max": {"chosen": sp["res"], "plain": pl["res"]},
             "max_rank": {"chosen": max(sp["rx"]), "plain": max(pl["rx"])},
             "chosen_vs_fp64": tt_rel_diff(d, n_, sp["rx"], sp["cores"], pl["rx"], pl["cores"])}
        if not args.no_cpu:
            from oracle.amen import tt_amen_solve as oracle_amen
            t0 = time.perf_counter()
            o = oracle_amen(d, n_, ra, crA, ry, y, rx, x0, 1e-9, nswp=6)
            tc = time.perf_counter() - t0
            g6, gr6 = ttgpu.dtt_amen_solve(d, n_, m_, ry, ra, crA, y, x0, rx, 1e-9, rmax=128, nswp=6,
                                           ctx=ctx)
            e["oracle_sample"] = {"sweeps": 6, "seconds": tc, "cores": os.cpu_count(),
                                  "plain_vs_oracle": tt_rel_diff(d, n_, gr6, g6, o["rx"], o["cores"]),
                                  "same_ranks": list(gr6) == list(o["rx"])}
        return e

    def xxz100():
        if not args.no_xxz:
            d, Bx = 100, 8
            n_, m_, ra, crA = xxz_mpo(d, delta=1.0)
            _, ry, cr = random_tt(d, 2, 16, last=Bx, seed=5)
            res = {}
            for meth in ("split", "plain"):
                (lam, _, r), t = _timed(torch, lambda: ttgpu.tt_eigb(d, n_, m_, ra, crA, cr, ry, 1e-10,
                                                                      256, Bx, nswp=2,
                                                                      max_full_size=200, method=meth,
                                                                      ctx=ctx))
                res[meth] = {"lambda": np.asarray(lam), "time": t, "max_rank": max(r[:d]),
                             "matvecs": ctx.stats()["matvecs"]}
            sp, pl = res["split"], res["plain"]
            out["xxz100"] = {
                "workload": "tt_eigb xxz d=100 n=2 ra=5 delta=1 B=8 start_rank=16 rmax=256 eps=1e-10 "
                            "nswp=2 max_full_size=200",
                "chosen_s": sp["time"], "plain_s": pl["time"],
                "plain_over_chosen": pl["time"] / sp["time"], "max_rank": int(sp["max_rank"]),
                "matvecs": {"chosen": sp["matvecs"], "plain": pl["matvecs"]},
                "chosen_vs_fp64_lambda": float(np.max(np.abs(sp["lambda"] - pl["lambda"]) /
                                                      np.abs(pl["lambda"])))}

    # a configuration that fails is reported in its entry; the line (and the
    # headline measurement) still prints
    for name, fn in (("ksl16", ksl16), ("amen10", amen10), ("xxz100", xxz100)):
        try:
            r = fn()
            if r is not None:
                out[name] = r
        except Exception as exc:   # noqa: BLE001
            out[name] = {"error": f"{type(exc).__name__}: {exc}"[:400]}
            torch.cuda.synchronize()
    return out


def batch_chains(count, seed=4):
    """The first `count` of the 256 chains of the batched configuration: XXZ,
    d ~ U{16..64}, delta ~ U[0.5, 1.5], B = 4, random rank-16 start (seeded),
    rank cap ~ U{32..128}."""
    from ttgpu.operators import xxz_mpo, random_tt
    rng = np.random.default_rng(seed)
    ds = rng.integers(16, 65, size=256)
    deltas = rng.uniform(0.5, 1.5, size=256)
    caps = rng.integers(32, 129, size=256)
    out = []
    for c in range(count):
        d = int(ds[c])
        n, m, ra, crA = xxz_mpo(d, delta=float(deltas[c]))
        _, ry, cr = random_tt(d, 2, 16, last=4, seed=1000 + c)
        out.append((d, n, m, ra, crA, cr, ry, int(caps[c])))
    return out


def bench_matvec(args, torch, ttgpu, ctx):
    """Split and plain local matvecs (prepared operators, CUDA-graph replays)
    at the d=20 Heisenberg local size (r=64, block 5) and the d=100 XXZ one
    (r=256, block 8); one JSON line."""
    peaks, src = measured_peaks()
    out = {"metric": "local matvec TFLOP/s (algorithmic)", "peak_bf16_tflops": peaks["bf16_tflops"],
           "peak_source": src, "shapes": {}}
    for r, nv in ((64, 5), (256, 8)):
        row = {}
        for meth in ("split", "plain"):
            fl, dt = matvec_roofline(torch, ctx, split=meth == "split", r=r, nvec=nv)
            row[meth] = {"us": dt * 1e6, "tflops": fl / dt / 1e12}
        fl = row["split"]["tflops"]
        row["split"]["bf16_issued_frac"] = 3 * fl / peaks["bf16_tflops"]
        out["shapes"]["r%d_b%d" % (r, nv)] = row
    print(json.dumps(out))


def bench_svd(args, torch, ttgpu, ctx):
    """The truncation SVD alone (ttg_dgesvd: QR with column sorting, one-sided
    Jacobi on R^T) on graded matrices of the sweeps' shapes: 320 x 128 (the
    d=20 Heisenberg block, B ry x n ry = 5*64 x 2*64) and 2048 x 512 (the d=100
    XXZ block, 8*256 x 2*256); mean of 5 calls after a warm-up, CUDA events."""
    out = {"metric": "truncation SVD time (ms)", "shapes": {}}
    for p, q in ((320, 128), (2048, 512)):
        rng = np.random.default_rng(p + q)
        r = min(p, q)
        U0 = np.linalg.qr(rng.standard_normal((p, r)))[0]
        V0 = np.linalg.qr(rng.standard_normal((q, r)))[0]
        M = (U0 * np.logspace(0, -13, r)) @ V0.T
        Md = torch.from_numpy(np.asfortranarray(M).ravel(order="F")).cuda()
        U = torch.zeros(p * r, dtype=torch.float64, device="cuda")
        sv = torch.zeros(r, dtype=torch.float64, device="cuda")
        Vt = torch.zeros(r * q, dtype=torch.float64, device="cuda")
        ttgpu.dgesvd(p, q, Md, U, sv, Vt, ctx=ctx)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            ttgpu.dgesvd(p, q, Md, U, sv, Vt, ctx=ctx)
        e1.record()
        torch.cuda.synchronize()
        s_ref = np.linalg.svd(M, compute_uv=False)
        out["shapes"]["%dx%d" % (p, q)] = {
            "ms": e0.elapsed_time(e1) / 5,
            "sigma_maxabs_err": float(np.abs(sv.cpu().numpy() - s_ref).max())}
    print(json.dumps(out))


def bench_batch(args, torch, ttgpu, ctx):
    """The batched configuration: independent chains queued on the batch
    runner (worker threads, one non-blocking stream each, longest first),
    chosen method, eps 1e-8, at most 20 sweeps; wall time of the whole batch
    (CUDA events around run())."""
    chains = batch_chains(args.batch_chains)
    batch = ttgpu.EigbBatch(nworkers=args.batch_workers, ctx=ctx)
    for (d, n, m, ra, crA, cr, ry, cap) in chains:
        batch.add(d, n, m, ra, crA, cr, ry, 1e-8, cap, 4, nswp=20, max_full_size=200,
                  method="split")
    with ClockSampler() as clk:
        _, t = _timed(torch, batch.run)
    mv = []
    sec = []
    for i in range(len(chains)):
        lam, _, ry_out, st = batch.result(i)
        mv.append(st["matvecs"])
        sec.append(st["seconds"])
    batch.close()
    line = {"metric": f"batched tt_eigb time, {len(chains)} of the 256 XXZ chains",
            "value": t, "unit": "s", "n_gpus": 1, "higher_is_better": False,
            "dtype": "bf16x3+f64", "data": "synthetic (seeded)", "method": "split",
            "config": {"workload": "batch: XXZ d~U{16..64} delta~U[0.5,1.5] B=4 start_rank=16 "
                                   "rmax~U{32..128} eps=1e-8 nswp=20 (seed 4)",
                       "chains": len(chains), "workers": args.batch_workers},
            "chain_seconds": {"sum": float(np.sum(sec)), "max": float(np.max(sec))},
            "matvecs": int(np.sum(mv)), "d_sum": int(sum(c[0] for c in chains)),
            "clocks": clk.summary()}
    print(json.dumps(line))


def one_core_baseline(timeout=300):
    """The same oracle solve on one core (one BLAS/OpenMP thread), in a child
    process so the thread count is fixed before numpy loads; None when it does
    not finish within the timeout."""
    code = ("import sys, time; sys.path[:0] = [%r, %r]\n"
            "import bench\n"
            "from oracle.eigb import tt_eigb\n"
            "n, m, ra, crA, ry, cr = bench.workload()\n"
            "t0 = time.perf_counter()\n"
            "tt_eigb(bench.D, n, m, ra, crA, cr, ry, bench.EPS, bench.RMAX, bench.B, nswp=20, "
            "max_full_size=bench.MFS)\n"
            "print(time.perf_counter() - t0)\n") % (ROOT, os.path.join(ROOT, "tt-fort_gb300"))
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1", MKL_NUM_THREADS="1")
    try:
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                           timeout=timeout)
        v = float(r.stdout.strip().splitlines()[-1])
    except Exception:
        return None
    return {"value": v, "unit": "s", "cores": 1,
            "sample": "one full solve with the oracle restatement, one BLAS/OpenMP thread"}


def run_reference(args):
    from oracle.eigb import tt_eigb as oracle_eigb
    n, m, ra, crA, ry, cr = workload()
    steps = max(1, min(args.steps, 2))
    warm = min(args.warmup, 1)
    for _ in range(warm):
        oracle_eigb(D, n, m, ra, crA, cr, ry, EPS, RMAX, B, nswp=20, max_full_size=MFS)
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        out = oracle_eigb(D, n, m, ra, crA, cr, ry, EPS, RMAX, B, nswp=20, max_full_size=MFS)
        ts.append(time.perf_counter() - t0)
    v_all = float(np.mean(ts))
    all_threads = {"value": v_all, "unit": "s", "cores": os.cpu_count(),
                   "sample": f"{steps} full solve(s) of the workload with the oracle "
                             "restatement (numpy + OpenBLAS on all host threads)"}
    # the same solve on one thread: the workload's dense products are small,
    # and on some hosts threading costs more than it gains; the faster of the
    # two is the reference arm's value
    one = one_core_baseline()
    best = one if one is not None and one["value"] < v_all else all_threads
    v = best["value"]
    line = {"metric": "tt_eigb sweep time to convergence (d=20 Heisenberg, B=5)",
            "value": v, "unit": "s", "n_gpus": args.gpus, "steps": steps, "warmup": warm,
            "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
            "config": config(),
            "cpu_baseline": {"value": v, "unit": "s", "cores": best["cores"], "kind": "port",
                             "sample": best["sample"] + " (the faster of all host threads and "
                                                        "one thread)",
                             "all_threads": all_threads, "one_core": one},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "lambda": out["lambda"].tolist()}
    print(json.dumps(line))


def bench_extra(args, torch, ttgpu, ctx):
    """The larger workloads: chosen (split) and plain methods, one timed run
    each (CUDA events on the library's stream) after a warm-up solve."""
    from ttgpu.operators import (xxz_mpo, random_tt, amen_operator, ksl_operator,
                                 random_tt_complex, tt_dot, tt_rel_diff)
    n, m, ra, crA, ry, cr = workload()
    ttgpu.tt_eigb(D, n, m, ra, crA, cr, ry, EPS, RMAX, B, nswp=20, max_full_size=MFS,
                  method="split", ctx=ctx)
    if args.workload == "ksl16":
        n_, m_, ra_, crA_ = ksl_operator(d=16, n=32, rank=4, std=0.01, seed=1)
        _, ry_, y_ = random_tt_complex(16, 32, 8, seed=2)
        for meth in ("split", "plain"):
            ttgpu.ztt_ksl(16, n_, m_, ra_, crA_, y_, ry_, 1e-3, 64, nsteps=2, method=meth, ctx=ctx)
    res = {}
    methods = args.methods.split(",")
    with ClockSampler() as clk:
        for meth in methods:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            l0 = ttgpu.launch_count()
            torch.cuda.profiler.start()   # the region a profiler started with capture off records
            e0.record()
            if args.workload == "xxz100":
                d, Bx = 100, 8
                n, m, ra, crA = xxz_mpo(d, delta=1.0)
                _, ry, cr = random_tt(d, 2, 16, last=Bx, seed=5)
                lam, _, ry_out = ttgpu.tt_eigb(d, n, m, ra, crA, cr, ry, 1e-10, 256, Bx,
                                               nswp=args.xxz_sweeps, max_full_size=200,
                                               method=meth, ctx=ctx)
                out = {"lambda": np.asarray(lam), "max_rank": max(ry_out[:d]),
                       "sweeps": ctx.stats()["sweeps"], "res": ctx.stats()["res"]}
            elif args.workload == "ksl16":
                d, nn, r = 16, 32, 8
                n_, m_, ra, crA = ksl_operator(d=d, n=nn, rank=4, std=0.01, seed=1)
                _, ry, y = random_tt_complex(d, nn, r, seed=2)
                y = y.copy()
                y[:ry[1] * nn] /= np.sqrt(tt_dot(d, n_, ry, y, ry, y).real)
                cores, ry_out = ttgpu.ztt_ksl(d, n_, m_, ra, crA, y, ry, 1e-3, 64,
                                              nsteps=args.ksl_steps, method=meth, ctx=ctx)
                out = {"cores": cores, "ry": ry_out, "n": n_, "max_rank": max(ry_out)}
            else:
                d, nn = 10, 64
                n_, m_, ra, crA = amen_operator(d=d, n=nn)
                _, ry, y = random_tt(d, nn, 4, seed=3)
                _, rx, x0 = random_tt(d, nn, 2, seed=7)
                _, rx_out = ttgpu.dtt_amen_solve(d, n_, m_, ry, ra, crA, y, x0, rx, 1e-9,
                                                 rmax=128, nswp=20, method=meth, ctx=ctx)
                out = {"max_rank": max(rx_out), "res": ctx.stats()["res"]}
            e1.record()
            torch.cuda.synchronize()
            torch.cuda.profiler.stop()
            out["time"] = e0.elapsed_time(e1) / 1e3
            out["launches"] = ttgpu.launch_count() - l0
            out["matvecs"] = ctx.stats()["matvecs"]
            res[meth] = out
    if len(methods) != 2:
        # one method only (profiling runs): its time and launches
        print(json.dumps({"workload": args.workload, "ksl_steps": args.ksl_steps,
                          **{m: {"time": res[m]["time"], "gpu_launches": int(res[m]["launches"])}
                             for m in methods}}))
        return
    sp, pl = res["split"], res["plain"]
    if args.workload == "xxz100":
        ns = args.xxz_sweeps
        metric = f"tt_eigb time to convergence, at most {ns} sweeps (d=100 XXZ, delta=1, B=8, rmax=256)"
        cfg = {"workload": "tt_eigb xxz d=100 n=2 ra=5 delta=1 B=8 start_rank=16 rmax=256 "
                           f"eps=1e-10 nswp={ns} max_full_size=200"}
        agree = float(np.max(np.abs(sp["lambda"] - pl["lambda"]) / np.abs(pl["lambda"])))
        extra = {"lambda_maxrel_vs_plain": agree, "lambda": sp["lambda"].tolist(),
                 "sweeps": {"split": sp["sweeps"], "plain": pl["sweeps"]},
                 "res": {"split": sp["res"], "plain": pl["res"]}}
    elif args.workload == "ksl16":
        ns = args.ksl_steps
        metric = f"ztt_ksl time of {ns} steps (d=16, n=32, -Laplacian + rank-4 N(0,0.01^2), rank 8)"
        cfg = {"workload": f"ztt_ksl d=16 n=32 ra=6 ry=8 tau=1e-3 nsteps={ns} typ=2 order=8"}
        extra = {"err_vs_fp64": tt_rel_diff(16, sp["n"], sp["ry"], sp["cores"], pl["ry"],
                                            pl["cores"])}
        if not args.no_cpu:
            # the oracle restatement on a bounded sample (10 of the 200 steps),
            # scaled to the workload, and its state against the plain method's
            from oracle.ksl import ztt_ksl as oracle_ksl
            n_, m_, ra_, crA_ = ksl_operator(d=16, n=32, rank=4, std=0.01, seed=1)
            _, ry_, y_ = random_tt_complex(16, 32, 8, seed=2)
            y_ = y_.copy()
            y_[:ry_[1] * 32] /= np.sqrt(tt_dot(16, n_, ry_, y_, ry_, y_).real)
            c_, r_ = y_, list(ry_)
            t0 = time.perf_counter()
            for _ in range(10):
                o = oracle_ksl(16, n_, m_, ra_, crA_, c_, r_, 1e-3, 64)
                c_, r_ = o["cores"], o["ry"]
            tc = time.perf_counter() - t0
            g10, gr10 = ttgpu.ztt_ksl(16, n_, m_, ra_, crA_, y_, ry_, 1e-3, 64, nsteps=10,
                                      method="plain", ctx=ctx)
            extra["cpu_baseline"] = {
                "value": tc * ns / 10, "unit": "s", "cores": os.cpu_count(), "kind": "port",
                "sample": f"10 of the {ns} steps with the oracle restatement (numpy + OpenBLAS "
                          f"threads), time x {ns / 10:g}",
                "plain_vs_oracle_10_steps": tt_rel_diff(16, n_, gr10, g10, r_, c_)}
        for o in (sp, pl):
            for k in ("cores", "ry", "n"):
                o.pop(k)
    else:
        metric = "ttamen solve time, 20 sweeps (d=10, n=64 Laplacian + potential, tol 1e-9)"
        cfg = {"workload": "dtt_amen_solve d=10 n=64 ra=3 ry=4 rx0=2 tol=1e-9 rmax=128 nswp=20"}
        extra = {"res_split": sp["res"], "res_plain": pl["res"]}
    line = {"metric": metric, "value": sp["time"], "unit": "s", "n_gpus": 1, "steps": 1,
            "warmup": 1, "higher_is_better": False, "dtype": "bf16x3+f64", "data": "synthetic (seeded)",
            "method": "split", "config": cfg, "gpu_launches": int(sp["launches"]),
            "matvecs": sp["matvecs"], "max_rank": int(sp["max_rank"]),
            "plain": {"value": pl["time"], "gpu_launches": int(pl["launches"]),
                      "matvecs": pl["matvecs"], "plain_over_chosen": pl["time"] / sp["time"]},
            "clocks": clk.summary()}
    line.update(extra)
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours")
    ap.add_argument("--method", default="split", choices=["split", "plain"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--methods", default="split,plain",
                    help="larger workloads: the methods to time (one method: profiling runs)")
    ap.add_argument("--profile-matvec", nargs=2, type=int, metavar=("R", "B"),
                    help="only apply the prepared split local operator (r = R, n = 2, ra = 5, "
                         "block of B) four times, for a profiler capture")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the block of the metric's other configurations")
    ap.add_argument("--no-xxz", action="store_true",
                    help="leave the d=100 XXZ entry out of that block")
    ap.add_argument("--xxz-sweeps", type=int, default=20,
                    help="sweep cap of the xxz100 workload (the reference's default nswp)")
    ap.add_argument("--ksl-steps", type=int, default=200,
                    help="ksl16: time steps (the workload is 200)")
    ap.add_argument("--workload", default="heisenberg20",
                    choices=["heisenberg20", "xxz100", "amen10", "ksl16", "batch256", "matvec",
                             "svd"])
    ap.add_argument("--batch-chains", type=int, default=256,
                    help="batch256: solve the first K of the 256 chains")
    ap.add_argument("--batch-workers", type=int, default=16)
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    import torch
    import ttgpu
    if args.gpus > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    ctx = ttgpu.Context(torch.cuda.current_device())
    # a non-blocking stream of our own (the legacy default stream serialises
    # with every other stream and cannot be captured into CUDA graphs); it is
    # torch's current stream from here on, so events and flushes use it too
    bench_stream = torch.cuda.Stream()
    torch.cuda.set_stream(bench_stream)
    ctx.bind_torch_stream()
    if args.profile_matvec:
        r, nv = args.profile_matvec
        rng = np.random.default_rng(0)
        t = lambda a: torch.from_numpy(a).cuda()
        phi1, A, phi2 = (t(rng.standard_normal(r * r * 5)), t(rng.standard_normal(5 * 2 * 2 * 5)),
                         t(rng.standard_normal(r * 5 * r)))
        X = t(rng.standard_normal(r * 2 * r * nv))
        Y = torch.zeros(r * 2 * r * nv, dtype=torch.float64, device="cuda")
        op = ttgpu.LocalOp(r, 2, r, r, 2, r, 5, 5, phi1, A, phi2, nvec_max=nv, method="split",
                           ctx=ctx)
        for _ in range(4):
            op.apply(X, Y, nv)
        torch.cuda.synchronize()
        op.close()
        return
    if args.workload == "matvec":
        if rank == 0:
            bench_matvec(args, torch, ttgpu, ctx)
        return
    if args.workload == "svd":
        if rank == 0:
            bench_svd(args, torch, ttgpu, ctx)
        return
    if args.workload == "batch256":
        if rank == 0:
            bench_batch(args, torch, ttgpu, ctx)
        return
    if args.workload != "heisenberg20":
        if rank == 0:
            bench_extra(args, torch, ttgpu, ctx)
        return
    n, m, ra, crA, ry, cr = workload()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def solve(method):
        return ttgpu.tt_eigb(D, n, m, ra, crA, cr, ry, EPS, RMAX, B, nswp=20, max_full_size=MFS,
                             method=method, ctx=ctx)

    def timed(method, steps):
        """steps solves, L2 flushed before each (untimed); CUDA events on the
        library's stream (bound to torch's current stream) and wall clock."""
        times, walls = [], []
        launches0 = ttgpu.launch_count()
        if args.gpus > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        out = None
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            w0 = time.perf_counter()
            e0.record()
            out = solve(method)
            e1.record()
            torch.cuda.synchronize()
            walls.append(time.perf_counter() - w0)
            times.append(e0.elapsed_time(e1) / 1e3)
        launches = (ttgpu.launch_count() - launches0) // max(1, steps)
        return float(np.mean(times)), float(np.mean(walls)), launches, out, ctx.stats()

    meth = args.method
    for _ in range(max(3, args.warmup)):
        solve(meth)
    with ClockSampler() as clk:
        t, tw, launches, (lam, cores, ry_out), st = timed(meth, args.steps)
    if args.gpus > 1:
        from ttgpu.replicas import max_over_ranks
        t, tw = max_over_ranks([t, tw])
    plain = None
    if meth != "plain" and not args.no_plain:
        solve("plain")
        tp, twp, lp, (lam_p, _, _), stp = timed("plain", max(1, min(args.steps, 2)))
        plain = {"value": tp, "unit": "s", "e2e": twp, "gpu_launches": int(lp),
                 "matvecs": stp["matvecs"], "plain_over_chosen": tp / t,
                 "lambda_maxrel_vs_chosen": float(np.max(np.abs(lam_p - lam) / np.abs(lam_p)))}
    ablation = None
    if meth == "split" and not args.no_plain:
        # the chosen method's local solver (Jacobi-Davidson + CG) on FP64
        # products: what split precision buys beyond the algorithm
        solve("jd64")
        tj, twj, lj, (lam_j, _, _), stj = timed("jd64", 1)
        ablation = {"jd64": {"value": tj, "unit": "s", "matvecs": stj["matvecs"],
                             "gpu_launches": int(lj), "jd64_over_chosen": tj / t,
                             "lambda_maxrel_vs_chosen":
                                 float(np.max(np.abs(lam_j - lam) / np.abs(lam_j)))}}
    if rank != 0:
        return
    peaks, kind = measured_peaks()
    split = meth == "split"
    fl, dt = matvec_roofline(torch, ctx, split=split)
    if split:
        peak, unit, bound = peaks["bf16_tflops"], "TFLOP/s", "tensor"
        peak_note = (f"bf16 dense burst ({kind}); the BF16x3 matvec issues 3 bf16 products "
                     "per algorithmic product, so the attainable algorithmic rate is peak/3")
    else:
        peak, unit, bound = fp64_peak_tflops(torch), "TFLOP/s", "tensor"
        peak_note = "fp64: cuBLAS DGEMM 4096^3 measured in this run"
    ach = fl / dt / 1e12
    big = None
    if split:
        flb, dtb = matvec_roofline(torch, ctx, split=True, r=256, nvec=8)
        big = {"kernel": "local matvec r=256 n=2 ra=5 block 8 (the d=100 XXZ local size)",
               "achieved": flb / dtb / 1e12, "bf16_issued": 3 * flb / dtb / 1e12,
               "frac": flb / dtb / 1e12 / peak, "launch_us": dtb * 1e6}
    configs = None if args.no_configs else config_block(args, torch, ttgpu, ctx)
    h2d = (len(crA) + len(cr)) * 8 + (len(n) * 3 + 2 * len(ry)) * 8
    d2h = len(cores) * 8 + B * 8
    cpu = None
    if not args.no_cpu:
        from oracle.eigb import tt_eigb as oracle_eigb
        t0 = time.perf_counter()
        ref = oracle_eigb(D, n, m, ra, crA, cr, ry, EPS, RMAX, B, nswp=20, max_full_size=MFS)
        tc = time.perf_counter() - t0
        all_threads = {"value": tc, "unit": "s", "cores": os.cpu_count(),
                       "sample": "one full solve of the workload with the oracle restatement "
                                 "(numpy + OpenBLAS on all host threads)"}
        one = one_core_baseline()
        best = one if one is not None and one["value"] < tc else all_threads
        cpu = {"value": best["value"], "unit": "s", "cores": best["cores"], "kind": "port",
               "sample": best["sample"] + " (the faster of all host threads and one thread)",
               "lambda_maxrel_vs_gpu": float(np.max(np.abs(ref["lambda"] - lam) / np.abs(ref["lambda"]))),
               "all_threads": all_threads, "one_core": one}
    line = {"metric": "tt_eigb sweep time to convergence (d=20 Heisenberg, B=5)",
            "value": t, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": t * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if meth == "plain" else "bf16x3+f64",
            "data": "synthetic (seeded)", "method": meth, "config": config(),
            "e2e": {"value": tw, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "roofline": {"kernel": f"local matvec bfun3 ({'BF16x3 tcgen05' if split else 'FP64'}, "
                                   f"r=64, n=2, ra=5, block 5)",
                         "bound": bound, "achieved": ach, "peak": peak, "unit": unit,
                         "frac": ach / peak, "traffic": SPLIT_MV_TRAFFIC if split else None,
                         "traffic_source": (SPLIT_MV_TRAFFIC_NOTE if split else None),
                         "peak_source": peak_note,
                         "launch_us": dt * 1e6, "flops_per_launch": fl, "large_local": big},
            "clocks": clk.summary(), "cpu_baseline": cpu, "plain": plain, "ablation": ablation,
            "configs": configs,
            "solve": {"lambda": lam.tolist(), "matvecs": st["matvecs"], "sweeps": st["sweeps"],
                      "max_rank": max(ry_out[:D])}}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
