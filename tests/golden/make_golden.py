"""Generate the committed golden fixtures from the reference's own fixture files.

Run once where the reference tree is available:
    python tests/golden/make_golden.py /path/to/tt-fort
It reads the reference fixtures (``Heisen_20.sdv``, ``test_ksl.dat``,
``test_eye_ksl.dat``) with the oracle's readers and writes small .npz copies
here, plus the exact-diagonalisation spectrum of the Heisenberg chain stored
in ``Heisen_20.sdv`` (sparse Lanczos on the 2^20 space, tol 1e-13).
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.ttio import read_sdv, read_ksl_dat  # noqa: E402


def heisenberg_ed(d, k=8):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    N = 1 << d
    idx = np.arange(N, dtype=np.int64)
    diag = np.zeros(N)
    rows, cols, vals = [], [], []
    for q in range(d - 1):
        a = (idx >> q) & 1
        b = (idx >> (q + 1)) & 1
        diag += np.where(a == b, 0.25, -0.25)
        flip = a != b
        rows.append(idx[flip])
        cols.append(idx[flip] ^ ((1 << q) | (1 << (q + 1))))
        vals.append(np.full(flip.sum(), 0.5))
    rows.append(idx); cols.append(idx); vals.append(diag)
    H = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(N, N))
    w = sla.eigsh(H, k=k, which="SA", tol=1e-13, return_eigenvectors=False)
    return np.sort(w).tolist()


def sdv_layout(ref):
    """The byte layout of the reference's Heisen_20.sdv: its first 16 header
    bytes ('TT' magic and version) and a hash of everything after the
    128-byte header (l, m, n, r and the cores)."""
    raw = open(os.path.join(ref, "Heisen_20.sdv"), "rb").read()
    with open(os.path.join(HERE, "heisen20_sdv_layout.json"), "w") as f:
        json.dump({"source": "Heisen_20.sdv", "size": len(raw), "head16_hex": raw[:16].hex(),
                   "body_sha256": hashlib.sha256(raw[128:]).hexdigest()}, f, indent=1)


def cme_fixture(ref):
    """The chemical-master-equation KSL case of test_ksl_cme.f90: operator
    cme20_A.sdv (TT-matrix, mode sizes n*n) and start cme20_u0.sdv, both
    complex files with zero imaginary parts, stored here as real arrays with
    the mode sizes n = sqrt(A's mode sizes) (test_ksl_cme.f90:71-79) and
    tau = T / Nt from test_ksl_cme.inp."""
    nA, rA, cA = read_sdv(os.path.join(ref, "cme20_A.sdv"), complex_=True)
    nu, ru, cu = read_sdv(os.path.join(ref, "cme20_u0.sdv"), complex_=True)
    assert np.abs(cA.imag).max() == 0.0 and np.abs(cu.imag).max() == 0.0
    n = np.array([int(round(np.sqrt(v))) for v in nA])
    assert list(n) == list(nu)
    lines = open(os.path.join(ref, "test_ksl_cme.inp")).read().split()
    T, Nt = float(lines[3]), int(lines[4])
    np.savez_compressed(os.path.join(HERE, "cme20_ksl.npz"), n=n, ra=np.array(rA),
                        crA=cA.real.copy(), ry=np.array(ru), crY=cu.real.copy(),
                        tau=np.array(T / Nt), nsteps_reference=np.array(Nt))


def main(ref):
    n, r, cores = read_sdv(os.path.join(ref, "Heisen_20.sdv"))
    np.savez_compressed(os.path.join(HERE, "heisen20_sdv.npz"), n=np.array(n), r=np.array(r),
                        cores=cores)
    sdv_layout(ref)
    cme_fixture(ref)
    for name in ("test_ksl.dat", "test_eye_ksl.dat"):
        D = read_ksl_dat(os.path.join(ref, name))
        np.savez_compressed(os.path.join(HERE, name.replace(".dat", "_dat.npz")),
                            **{k: np.asarray(v) for k, v in D.items()})
    ed = heisenberg_ed(20)
    with open(os.path.join(HERE, "heisen20_ed.json"), "w") as f:
        json.dump({"source": "Heisen_20.sdv (d=20 OBC spin-1/2 Heisenberg), sparse ED",
                   "eigenvalues": ed}, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path of the tt-fort source tree>")
    main(sys.argv[1])
