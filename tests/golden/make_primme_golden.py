"""Golden fixtures from the reference's own PRIMME eigensolver.

Runs tt-fort's vendored PRIMME C code (built unchanged by oracle/build_ref.py)
as the local eigensolver of the oracle's tt_eigb sweep, with tt_eigb's
settings (tt_eigb.f90:252-283), on the d=20 Heisenberg workload (the
operator of Heisen_20.sdv, B=5, start ranks 16 seed 0, rmax 64, eps 1e-8,
max_full_size 200):

  eigb_heisen20_primme.json  eigenvalues, sweeps, ranks and matvecs of the
                             sweep with PRIMME pinned to GD+k (deterministic)
                             and with the reference's DYNAMIC method
  primme_local_heisen20.npz  two local problems recorded from that sweep (the
                             largest, N = 64*2*64, and one of N = 32*2*64):
                             Phi1, A, Phi2, a seeded N(0,1) start block, the
                             tolerance, and PRIMME's (GD+k) eigenvalues and
                             residual norms from that start

Needs the tt-fort source tree (for PRIMME's sources):
  python tests/golden/make_primme_golden.py <path of the tt-fort source tree>
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "tt-fort_gb300")]


def main(src):
    os.environ["TT_FORT_SRC"] = src
    from oracle import primme
    from oracle.eigb import tt_eigb
    from oracle.ops import bfun3_block, flat, F
    from ttgpu.operators import xxz_mpo, random_tt
    D, B = 20, 5
    n, m, ra, crA = xxz_mpo(D)
    _, ry, cr = random_tt(D, 2, 16, last=B, seed=0)
    out = {"source": "oracle tt_eigb sweep with tt-fort's PRIMME (primme/*.c, unchanged) as the "
                     "local eigensolver, tt_eigb.f90:252-283 settings",
           "workload": "heisenberg d=20 n=2 ra=5 B=5 start_rank=16 seed=0 rmax=64 eps=1e-8 "
                       "max_full_size=200"}
    recorded = []
    for meth in ("GD_plusK", "DYNAMIC"):
        st = []
        rec = recorded if meth == "GD_plusK" else None
        r = tt_eigb(D, n, m, ra, crA, cr, ry, 1e-8, 64, B, nswp=20, max_full_size=200,
                    local_solver=primme.local_solver(meth, st), record=rec)
        out[meth] = {"lambda": r["lambda"].tolist(), "sweeps": r["sweeps"], "ry": r["ry"],
                     "matvecs": r["matvecs"], "local_solves": len(st),
                     "ierr": sorted(set(int(s[2]) for s in st))}
    with open(os.path.join(HERE, "eigb_heisen20_primme.json"), "w") as f:
        json.dump(out, f, indent=1)
    # two local problems: the largest and one of the next size down
    sizes = [p["dims"][0] * p["dims"][1] * p["dims"][2] for p in recorded]
    pick = [sizes.index(max(sizes))]
    pick.append(next(k for k, s in enumerate(sizes) if s == 32 * 2 * 64))
    arrays = {}
    rng = np.random.default_rng(2024)
    for q, k in enumerate(pick):
        p = recorded[k]
        r1, nn, r2, ra1, ra2 = p["dims"]
        N = r1 * nn * r2
        X0 = rng.standard_normal((N, B))

        def mv(X, p=p, r1=r1, nn=nn, r2=r2, ra1=ra1, ra2=ra2, N=N):
            k_ = X.shape[1]
            return F(bfun3_block(r1, nn, r2, r1, nn, r2, ra1, ra2, p["phi1"], p["A"], p["phi2"],
                                 flat(X), k_), N, k_)
        lam, V, rn, nmv, ierr = primme.dprimme(mv, N, B, X0, p["tol"], method="GD_plusK")
        assert ierr == 0, ierr
        arrays.update({f"p{q}_dims": np.array(p["dims"]), f"p{q}_phi1": p["phi1"],
                       f"p{q}_A": p["A"], f"p{q}_phi2": p["phi2"], f"p{q}_X0": flat(X0),
                       f"p{q}_tol": np.array(p["tol"]), f"p{q}_lambda": lam,
                       f"p{q}_rnorms": rn, f"p{q}_matvecs": np.array(nmv)})
    np.savez_compressed(os.path.join(HERE, "primme_local_heisen20.npz"), **arrays)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_primme_golden.py <path of the tt-fort source tree>")
    main(sys.argv[1])
