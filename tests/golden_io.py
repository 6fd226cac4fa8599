"""Loader for the golden fixtures in tests/golden (written by tests/golden/make_golden.py)."""

import glob
import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    runs = []
    for r in meta["runs"]:
        r = dict(r)
        r["idx"] = z[r["tag"] + "_idx"]
        r["dist"] = z[r["tag"] + "_dist"]
        runs.append(r)
    return dict(name=meta["name"], k=meta["k"], max_dist2=meta["max_dist2"],
                points=z["points"], queries=z["queries"], runs=runs)
