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


def _good_file(tmp_path, complex_=False):
    import ttgpu
    rng = np.random.default_rng(3)
    n, r = [2, 3, 2], [1, 2, 2, 1]
    size = sum(r[k] * n[k] * r[k + 1] for k in range(3))
    cores = rng.standard_normal(size) + (1j * rng.standard_normal(size) if complex_ else 0)
    path = tmp_path / "good.sdv"
    ttgpu.sdv_write(path, n, r, cores, complex_=complex_)
    return path, n, r, cores


def test_rejects_corrupted_headers_and_bodies(tmp_path):
    """Corrupted .sdv files are errors, never partial reads: wrong magic,
    wrong version, truncated header, a mode or rank record that is zero or
    negative, a first mode after the last, and a body shorter than the ranks
    say."""
    import struct
    import ttgpu
    path, n, r, cores = _good_file(tmp_path)
    raw = path.read_bytes()
    ttgpu.sdv_read(path)                                        # the intact file reads

    def bad(data, name):
        p = tmp_path / name
        p.write_bytes(data)
        with pytest.raises(RuntimeError):
            ttgpu.sdv_read(p)

    bad(b"TX" + raw[2:], "magic.sdv")
    bad(raw[:8] + struct.pack("<i", 2) + raw[12:], "version.sdv")
    bad(raw[:100], "short_header.sdv")
    bad(raw[:128] + struct.pack("<ii", 3, 1) + raw[136:], "l_after_m.sdv")
    off_n = 128 + 8                                             # n(1:d), then r(0:d)
    bad(raw[:off_n] + struct.pack("<i", 0) + raw[off_n + 4:], "zero_mode.sdv")
    off_r = off_n + 4 * len(n)
    bad(raw[:off_r + 4] + struct.pack("<i", -2) + raw[off_r + 8:], "negative_rank.sdv")
    bad(raw[:-8], "short_body.sdv")
    bad(raw[:off_r], "no_ranks.sdv")


def test_complex_file_read_as_real_is_short(tmp_path):
    """The file does not say whether it holds float64 or complex128 cores; a
    real file read as complex runs out of body and is an error."""
    import ttgpu
    path, n, r, cores = _good_file(tmp_path, complex_=False)
    with pytest.raises(RuntimeError):
        ttgpu.sdv_read(path, complex_=True)
    n1, r1, c1 = ttgpu.sdv_read(path, complex_=False)
    assert np.array_equal(c1, cores)


def test_writer_rejects_bad_sizes(tmp_path):
    import ctypes as C
    import ttgpu
    with pytest.raises(ValueError):
        ttgpu.sdv_write(tmp_path / "a.sdv", [2, 0], [1, 1, 1], np.zeros(2))
    with pytest.raises(ValueError):
        ttgpu.sdv_write(tmp_path / "b.sdv", [2, 2], [1, -1, 1], np.zeros(4))
    with pytest.raises(RuntimeError):
        ttgpu.sdv_write(tmp_path / "no_such_dir" / "c.sdv", [2], [1, 1], np.zeros(2))
    # the C entry point checks the same itself
    lib = ttgpu.lib()
    buf = np.zeros(4)
    n0, r0 = np.array([2, 0], dtype=np.int64), np.array([1, 1, 1], dtype=np.int64)
    path = str(tmp_path / "d.sdv").encode()
    assert lib.ttg_sdv_write(path, C.c_int64(2), n0.ctypes.data_as(C.c_void_p),
                             r0.ctypes.data_as(C.c_void_p), buf.ctypes.data_as(C.c_void_p),
                             C.c_int(0)) != 0
    assert lib.ttg_sdv_write(path, C.c_int64(0), n0.ctypes.data_as(C.c_void_p),
                             r0.ctypes.data_as(C.c_void_p), buf.ctypes.data_as(C.c_void_p),
                             C.c_int(0)) != 0


def test_writer_checks_the_core_count_against_the_ranks(tmp_path):
    import ttgpu
    with pytest.raises(ValueError):
        ttgpu.sdv_write(tmp_path / "d.sdv", [2, 2], [1, 2, 1], np.zeros(7))
    with pytest.raises(ValueError):
        ttgpu.sdv_write(tmp_path / "e.sdv", [2, 2], [1, 2], np.zeros(8))
