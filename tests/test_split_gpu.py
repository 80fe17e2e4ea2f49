"""GPU parity of the split-precision (BF16x3, FP32 accumulate) tensor-core
local operator against the FP64 oracle.

Tolerance: relative 2-norm error <= 5e-5.  BF16x3 keeps ~16 significand bits
per operand (a_hi + a_lo) and drops a_lo*b_lo (<= 2^-18 |ab|); with FP32
accumulation and two GEMM stages plus the core stage the measured error is a
few 1e-6, so 5e-5 leaves head-room without hiding a wrong tile or index."""
import numpy as np
import pytest

from oracle import ops

pytestmark = pytest.mark.gpu
TOL_SPLIT = 5e-5

SHAPES = [
    (1, 2, 2, 1, 2, 2, 1, 4, 1),
    (16, 2, 16, 16, 2, 16, 5, 5, 5),
    (64, 2, 64, 64, 2, 64, 5, 5, 5),        # the d=20 Heisenberg local problem
    (7, 3, 11, 5, 2, 9, 2, 3, 2),           # ragged
    (130, 2, 70, 130, 2, 70, 5, 5, 3),      # crosses a 128-row tile
    (8, 32, 8, 8, 32, 8, 6, 6, 1),          # KSL-like
    (32, 64, 24, 32, 64, 24, 3, 3, 1),      # AMEn-like n = 64
    (256, 2, 256, 256, 2, 256, 5, 5, 8),    # the d=100 XXZ local problem (r = 256, B = 8)
    # single-launch fused path (rx1*m <= 128, rx2 <= 64, ry1 <= 128, n == m,
    # small core): ragged blocks of c2 and K tiles, boundary cores, m = 4 and
    # m = 1 with eight K tiles of GEMM3 (narrow-tile plan)
    (37, 2, 50, 45, 2, 61, 5, 5, 3),
    (64, 2, 64, 64, 2, 64, 1, 5, 2),        # left boundary core (ra1 = 1)
    (64, 2, 64, 64, 2, 64, 5, 1, 2),        # right boundary core (ra2 = 1)
    (32, 4, 16, 40, 4, 16, 2, 3, 2),
    (64, 1, 64, 100, 1, 64, 8, 8, 4),
    (60, 2, 33, 128, 2, 20, 3, 4, 9),
    # core-contracted path (rx1 % 8 == 0, n*m <= 4) with ragged other sizes
    (40, 2, 24, 48, 2, 56, 3, 4, 3),
    (8, 1, 5, 7, 2, 6, 1, 5, 2),
    (24, 2, 8, 16, 2, 8, 5, 1, 2),
]


@pytest.mark.parametrize("shape", SHAPES)
def test_dbfun3_split_vs_oracle(torch_cuda, ctx, shape):
    import ttgpu
    torch = torch_cuda
    rx1, m, rx2, ry1, n, ry2, ra1, ra2, nvec = shape
    rng = np.random.default_rng(sum(shape))
    phi1 = rng.standard_normal(ry1 * rx1 * ra1)
    A = rng.standard_normal(ra1 * n * m * ra2)
    phi2 = rng.standard_normal(rx2 * ra2 * ry2)
    X = rng.standard_normal(rx1 * m * rx2 * nvec)
    ref = ops.bfun3_block(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, X, nvec)
    t = lambda a: torch.from_numpy(a).cuda()
    Y = torch.full((ry1 * n * ry2 * nvec,), float("nan"), dtype=torch.float64, device="cuda")
    ttgpu.dbfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, t(phi1), t(A), t(phi2), t(X), Y,
                 nvec=nvec, split=True)
    ctx.synchronize()
    y = Y.cpu().numpy()
    assert np.all(np.isfinite(y))
    for v in range(nvec):
        sl = slice(v * ry1 * n * ry2, (v + 1) * ry1 * n * ry2)
        err = np.linalg.norm(y[sl] - ref[sl]) / np.linalg.norm(ref[sl])
        assert err < TOL_SPLIT, (v, err)


@pytest.mark.parametrize("method,tol", [("plain", 1e-12), ("split", TOL_SPLIT)])
def test_prepared_localop(torch_cuda, ctx, method, tol):
    import ttgpu
    torch = torch_cuda
    rx1, m, rx2, ry1, n, ry2, ra1, ra2 = 24, 2, 40, 24, 2, 40, 5, 4
    rng = np.random.default_rng(9)
    t = lambda a: torch.from_numpy(a).cuda()
    phi1 = t(rng.standard_normal(ry1 * rx1 * ra1))
    A = t(rng.standard_normal(ra1 * n * m * ra2))
    phi2 = t(rng.standard_normal(rx2 * ra2 * ry2))
    op = ttgpu.LocalOp(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, nvec_max=4,
                       method=method, ctx=ctx)
    for nvec in (4, 1, 3):     # the operator is reused for several block sizes
        X = rng.standard_normal(rx1 * m * rx2 * nvec)
        ref = ops.bfun3_block(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1.cpu().numpy(),
                              A.cpu().numpy(), phi2.cpu().numpy(), X, nvec)
        Y = torch.zeros(ry1 * n * ry2 * nvec, dtype=torch.float64, device="cuda")
        op.apply(t(X), Y, nvec)
        ctx.synchronize()
        y = Y.cpu().numpy()
        assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < tol
    op.close()


FUSED_SHAPES = [s for s in SHAPES if s[1] == s[4] and s[0] * s[1] <= 128 and s[2] <= 64
                and s[3] <= 128 and s[1] * s[7] <= 16 and s[4] * s[6] <= 16]

_FUSED_CHILD = r'''
import json, sys
import numpy as np, torch
import ttgpu
from oracle import ops
shapes = json.loads(sys.argv[1])
ctx = ttgpu.Context(0)
errs = []
for rx1, m, rx2, ry1, n, ry2, ra1, ra2, nvec in shapes:
    rng = np.random.default_rng(rx1 + 7 * ry2 + nvec)
    phi1 = rng.standard_normal(ry1 * rx1 * ra1)
    A = rng.standard_normal(ra1 * n * m * ra2)
    phi2 = rng.standard_normal(rx2 * ra2 * ry2)
    X = rng.standard_normal(rx1 * m * rx2 * nvec)
    ref = ops.bfun3_block(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, X, nvec)
    t = lambda a: torch.from_numpy(a).cuda()
    Y = torch.full((ry1 * n * ry2 * nvec,), float("nan"), dtype=torch.float64, device="cuda")
    ttgpu.dbfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, t(phi1), t(A), t(phi2), t(X), Y,
                 nvec=nvec, split=True, ctx=ctx)
    ctx.synchronize()
    y = Y.cpu().numpy()
    errs.append(float(np.linalg.norm(y - ref) / np.linalg.norm(ref)) if np.all(np.isfinite(y))
                else float("inf"))
print(json.dumps(errs))
'''


def test_fused_single_launch_path_vs_oracle(torch_cuda):
    """The opt-in single-launch operator (TTG_FUSED=1, read once per process,
    so it runs in a child process) on every shape it accepts."""
    import json
    import os
    import subprocess
    import sys
    from conftest import ROOT
    assert len(FUSED_SHAPES) >= 6
    env = dict(os.environ, TTG_FUSED="1",
               PYTHONPATH=os.pathsep.join([ROOT, os.path.join(ROOT, "tt-fort_gb300")]))
    out = subprocess.run([sys.executable, "-c", _FUSED_CHILD, json.dumps(FUSED_SHAPES)],
                         capture_output=True, text=True, env=env, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    errs = json.loads(out.stdout.strip().splitlines()[-1])
    assert max(errs) < TOL_SPLIT, errs


# products with several output tiles per CTA of the persistent GEMM (both
# TMEM accumulators reused, ragged K and tile edges), run at each fixed tile
# width in a child process (TTG_SPLIT_BN is read once per process)
WIDE_SHAPES = [
    (256, 2, 256, 256, 2, 256, 5, 5, 8),
    (256, 2, 200, 250, 2, 190, 5, 5, 7),
    (130, 2, 70, 130, 2, 70, 5, 5, 3),
    (7, 3, 11, 5, 2, 9, 2, 3, 2),
]


@pytest.mark.parametrize("bn", ["64", "128", "256"])
def test_split_gemm_each_tile_width_vs_oracle(torch_cuda, bn):
    import json
    import os
    import subprocess
    import sys
    from conftest import ROOT
    env = dict(os.environ, TTG_SPLIT_BN=bn,
               PYTHONPATH=os.pathsep.join([ROOT, os.path.join(ROOT, "tt-fort_gb300")]))
    out = subprocess.run([sys.executable, "-c", _FUSED_CHILD, json.dumps(WIDE_SHAPES)],
                         capture_output=True, text=True, env=env, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    errs = json.loads(out.stdout.strip().splitlines()[-1])
    assert max(errs) < TOL_SPLIT, errs


_PDL_CHILD = r'''
import json, sys
import numpy as np, torch
import ttgpu
shapes = json.loads(sys.argv[1])
ctx = ttgpu.Context(0)
out = []
for rx1, m, rx2, ry1, n, ry2, ra1, ra2, nvec in shapes:
    rng = np.random.default_rng(rx1 + 3 * ry2 + nvec)
    t = lambda a: torch.from_numpy(a).cuda()
    phi1, A = t(rng.standard_normal(ry1 * rx1 * ra1)), t(rng.standard_normal(ra1 * n * m * ra2))
    phi2 = t(rng.standard_normal(rx2 * ra2 * ry2))
    op = ttgpu.LocalOp(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, nvec_max=nvec,
                       method="split", ctx=ctx)
    ys = []
    for rep in range(3):   # back-to-back applies: each launch overlaps the one before
        X = t(rng.standard_normal(rx1 * m * rx2 * nvec))
        Y = torch.zeros(ry1 * n * ry2 * nvec, dtype=torch.float64, device="cuda")
        op.apply(X, Y, nvec)
        ys.append(Y)
    ctx.synchronize()
    out.append([y.cpu().numpy().tolist() for y in ys])
    op.close()
print(json.dumps(out))
'''


def test_programmatic_dependent_launch_changes_no_result(torch_cuda):
    """Programmatic dependent launch lets a kernel's prologue overlap the
    kernel before it; every kernel waits for its predecessor before touching
    memory, so results must be bit-identical with it switched off
    (TTG_PDL=0, read once per process: child processes)."""
    import json
    import os
    import subprocess
    import sys
    from conftest import ROOT
    shapes = [(64, 2, 64, 64, 2, 64, 5, 5, 5), (256, 2, 256, 256, 2, 256, 5, 5, 8),
              (8, 32, 8, 8, 32, 8, 6, 6, 1)]
    res = {}
    for mode in ("0", "1"):
        env = dict(os.environ, TTG_PDL=mode,
                   PYTHONPATH=os.pathsep.join([ROOT, os.path.join(ROOT, "tt-fort_gb300")]))
        out = subprocess.run([sys.executable, "-c", _PDL_CHILD, json.dumps(shapes)],
                             capture_output=True, text=True, env=env, timeout=600)
        assert out.returncode == 0, out.stderr[-2000:]
        res[mode] = json.loads(out.stdout.strip().splitlines()[-1])
    assert res["0"] == res["1"]
