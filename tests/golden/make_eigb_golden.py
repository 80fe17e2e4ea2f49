"""Oracle result of the d=20 Heisenberg tt_eigb workload (committed fixture).

    python tests/golden/make_eigb_golden.py
Inputs: the reference operator ``Heisen_20.sdv`` (heisen20_sdv.npz), start
block random_tt(20, 2, 16, last=5, seed=0), eps 1e-8, rmax 64, B 5,
max_full_size 200 -- the same call the GPU test makes.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "tt-fort_gb300")]

from oracle.eigb import tt_eigb  # noqa: E402
from ttgpu.operators import random_tt  # noqa: E402

f = np.load(os.path.join(HERE, "heisen20_sdv.npz"))
d, B = 20, 5
r = [int(v) for v in f["r"]]
_, ry, cr = random_tt(d, 2, 16, last=B, seed=0)
out = tt_eigb(d, [2] * d, [2] * d, r, f["cores"], cr, ry, 1e-8, 64, B, nswp=20, max_full_size=200)
with open(os.path.join(HERE, "eigb_heisen20_oracle.json"), "w") as fh:
    json.dump({"lambda": out["lambda"].tolist(), "ry": out["ry"], "sweeps": out["sweeps"],
               "matvecs": out["matvecs"]}, fh, indent=1)
print(out["lambda"], out["sweeps"])
