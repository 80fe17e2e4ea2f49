"""The .sdv TT file format (dtt_write/ztt_write, dtt_read/ztt_read,
ttio.f90:29-399) through the C ABI, on the host (no GPU needed).

Pins: the library's writer reproduces the reference's Heisen_20.sdv byte for
byte after the 128-byte header (hash recorded by tests/golden/make_golden.py)
and the same first 16 header bytes; the oracle's reader (checked against the
reference file when the golden was made) reads what the library writes; real
and complex round trips; a file that is not a TT file is rejected."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle.ttio import read_sdv

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_writer_reproduces_the_reference_fixture(tmp_path):
    import ttgpu
    f = np.load(os.path.join(GOLDEN, "heisen20_sdv.npz"))
    lay = json.load(open(os.path.join(GOLDEN, "heisen20_sdv_layout.json")))
    path = tmp_path / "heisen20.sdv"
    ttgpu.sdv_write(path, f["n"], f["r"], f["cores"])
    raw = path.read_bytes()
    assert len(raw) == lay["size"]
    assert raw[:16].hex() == lay["head16_hex"]
    assert hashlib.sha256(raw[128:]).hexdigest() == lay["body_sha256"]
    n, r, cores = ttgpu.sdv_read(path)
    assert n == list(f["n"]) and r == list(f["r"])
    assert np.array_equal(cores, f["cores"])
    n2, r2, c2 = read_sdv(path)
    assert n2 == n and r2 == r and np.array_equal(c2, cores)


@pytest.mark.parametrize("complex_", [False, True])
def test_round_trip(tmp_path, complex_):
    import ttgpu
    rng = np.random.default_rng(5)
    n = [3, 4, 2, 5]
    r = [1, 2, 3, 4, 1]
    sz = sum(r[k] * n[k] * r[k + 1] for k in range(4))
    cores = rng.standard_normal(sz)
    if complex_:
        cores = cores + 1j * rng.standard_normal(sz)
    path = tmp_path / "x.sdv"
    ttgpu.sdv_write(path, n, r, cores, complex_=complex_)
    n1, r1, c1 = ttgpu.sdv_read(path, complex_=complex_)
    assert (n1, r1) == (n, r) and np.array_equal(c1, cores)
    n2, r2, c2 = read_sdv(path, complex_=complex_)
    assert (n2, r2) == (n, r) and np.array_equal(c2, cores)


def test_rejects_files_that_are_not_tt(tmp_path):
    import ttgpu
    path = tmp_path / "bad.sdv"
    path.write_bytes(b"XX" + bytes(200))
    with pytest.raises(RuntimeError):
        ttgpu.sdv_read(path)
    with pytest.raises(RuntimeError):
        ttgpu.sdv_read(tmp_path / "missing.sdv")
