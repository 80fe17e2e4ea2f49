"""Readers for the reference's binary fixtures (oracle / test infrastructure).

``read_sdv`` follows ``dtt_read`` ttio.f90:196-296: a 128-byte header
('TT' magic, version (1,0), info, comment, 8 ints), then int32 l, m, then
int32 n(l:m) and r(l-1:m), then the cores as float64 in column-major order.
``read_ksl_dat`` follows the stream reader of test_ksl.f90:9-33.
"""
import numpy as np


def read_sdv(path, complex_=False):
    with open(path, "rb") as f:
        head = f.read(128)
        if head[:2] != b"TT":
            raise ValueError("not a TT file")
        ver = np.frombuffer(head[8:16], dtype=np.int32)
        if ver[0] != 1:
            raise ValueError(f"bad TT version {ver}")
        l, m = np.frombuffer(f.read(8), dtype=np.int32)
        d = m - l + 1
        n = np.frombuffer(f.read(4 * d), dtype=np.int32).astype(int)
        r = np.frombuffer(f.read(4 * (d + 1)), dtype=np.int32).astype(int)
        sz = int(sum(r[k] * n[k] * r[k + 1] for k in range(d)))
        dt = np.complex128 if complex_ else np.float64
        cores = np.frombuffer(f.read(sz * np.dtype(dt).itemsize), dtype=dt).copy()
    return list(n), list(r), cores


def read_ksl_dat(path):
    """test_ksl.f90:9-33 layout: d, n, m, ra, ry, Asize, crA, Ysize, crY, tau, ..."""
    buf = open(path, "rb").read()
    off = 0

    def ints(k):
        nonlocal off
        v = np.frombuffer(buf, dtype=np.int32, count=k, offset=off).astype(int)
        off += 4 * k
        return v

    def cplx(k):
        nonlocal off
        v = np.frombuffer(buf, dtype=np.complex128, count=k, offset=off).copy()
        off += 16 * k
        return v

    d = int(ints(1)[0])
    n = ints(d); m = ints(d); ra = ints(d + 1); ry = ints(d + 1)
    Asize = int(ints(1)[0]); crA = cplx(Asize)
    Ysize = int(ints(1)[0]); crY = cplx(Ysize)
    tau = float(np.frombuffer(buf, dtype=np.float64, count=1, offset=off)[0]); off += 8
    rmax, kickrank, nswp, verb = ints(4)
    return dict(d=d, n=list(n), m=list(m), ra=list(ra), ry=list(ry), crA=crA, crY=crY,
                tau=tau, rmax=int(rmax), kickrank=int(kickrank), nswp=int(nswp), verb=int(verb))
