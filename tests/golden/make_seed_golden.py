"""Generate tests/golden/seeds_dichotomy.npz: the reference's own dichotomy
seed initialiser (backend/main.py:83-91, 252-326) run on a seeded network
with its global RNGs seeded -- the fixture that pins
analyticmesh_gb300.seeds.dichotomy (same draws, same points).

    python tests/golden/make_seed_golden.py

Reads the reference checkout (AM_REFERENCE_ROOT); the reference's functions
are taken from its source and run on the CPU (its `.cuda()` calls become no-
ops for the run).  Test infrastructure only.
"""
import ast
import os
import random
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from analyticmesh_gb300 import workloads as wl  # noqa: E402
from oracle import build_ref  # noqa: E402

NAMES = ("constraints_filter", "init_within_ball", "dichotomy")
CASES = [  # (network seed, widths, iso, init_num, try_pts_num, rng seed)
    (7, [32, 32], 0.0, 256, 1024, 5),
    (12, [48, 48, 48], 0.05, 200, 2048, 9),
]


def reference_functions():
    src = open(os.path.join(build_ref.REF_ROOT, "backend", "main.py")).read()
    tree = ast.parse(src)
    body = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in NAMES]
    ns = {"torch": torch, "random": random, "time": time, "np": np}
    exec(compile(ast.Module(body=body, type_ignores=[]), "reference_main", "exec"), ns)
    return ns


def main():
    ns = reference_functions()
    cuda = torch.Tensor.cuda
    torch.Tensor.cuda = lambda self, *a, **k: self  # CPU run of the reference's code
    out = {}
    try:
        for c, (nseed, widths, iso, n, tries, seed) in enumerate(CASES):
            model = wl.geometric(widths, nseed, perturb=0.05 if len(widths) > 2 else 0.0).float().eval()
            random.seed(seed)
            torch.manual_seed(seed)
            with torch.no_grad():
                pts = ns["dichotomy"](model, iso, n, None, None, tries, 1.0, 100, 1e-3, 60)
            out["points%d" % c] = pts.numpy()
    finally:
        torch.Tensor.cuda = cuda
    np.savez_compressed(os.path.join(HERE, "seeds_dichotomy.npz"), **out)
    print("wrote", os.path.join(HERE, "seeds_dichotomy.npz"))


if __name__ == "__main__":
    main()
