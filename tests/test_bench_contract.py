"""The benchmark's output contract, on CPU: the reference arm's JSON line
(run on a small chain so the test stays fast) and the per-configuration error
capture of the GPU arm's configuration block."""
import io
import json
import types
from contextlib import redirect_stdout

import numpy as np


def test_reference_arm_line_contract(monkeypatch):
    import bench
    from ttgpu.operators import xxz_mpo, random_tt

    def small():
        n, m, ra, crA = xxz_mpo(6)
        _, ry, cr = random_tt(6, 2, 4, last=2, seed=0)
        return n, m, ra, crA, ry, cr

    monkeypatch.setattr(bench, "workload", small)
    monkeypatch.setattr(bench, "D", 6)
    monkeypatch.setattr(bench, "B", 2)
    monkeypatch.setattr(bench, "RMAX", 16)
    monkeypatch.setattr(bench, "MFS", 16)
    # the one-thread solve runs in a child process on the real workload; here
    # a fixed stand-in slower than any small-chain solve
    monkeypatch.setattr(bench, "one_core_baseline",
                        lambda: {"value": 1e9, "unit": "s", "cores": 1, "sample": "stand-in"})
    args = types.SimpleNamespace(steps=1, warmup=0, gpus=1)
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(args)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e", "impl"):
        assert k in line, k
    assert line["impl"] == "reference" and line["higher_is_better"] is False
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1
    assert cb["value"] == min(cb["all_threads"]["value"], cb["one_core"]["value"])
    assert "workload" in line["config"]
    assert np.all(np.isfinite(line["lambda"]))


def test_config_failures_are_reported_per_entry():
    """A configuration whose solver raises is reported in its own entry; the
    other entries and the line itself still come out."""
    import bench

    class NoGpu:
        def __getattr__(self, name):
            raise RuntimeError("unavailable: " + name)

    class Torch:
        class cuda:
            @staticmethod
            def synchronize():
                pass

    args = types.SimpleNamespace(no_xxz=False, no_cpu=True, ksl_steps=2)
    out = bench.config_block(args, Torch, NoGpu(), NoGpu())
    assert set(out) == {"ksl16", "amen10", "xxz100"}
    assert all("error" in v for v in out.values())
