"""Writes sample_task_digests.json.gz: compact golden vectors derived from
CP2K's recorded single-task fixtures (src/grid/sample_tasks/*.task), so that
tests running without the CP2K tree (e.g. on the GPU host) can still check
against them.  Per task: the full task description (parameters and the pab
block), the expected hab / forces / virial, and a digest of the expected grid
(sum, sum of squares, max |value|, and 96 sampled points including the
largest ones).

Run from the repository root:  python tests/golden/make_sample_digests.py
"""
import gzip
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from sample_tasks import DIGEST_FILE, SAMPLE_TASKS, load_sample  # noqa: E402


def main():
    out = {}
    rng = np.random.default_rng(7)
    for name in SAMPLE_TASKS:
        t = load_sample(name)
        g = t["grid"]
        top = np.argsort(-np.abs(g))[:48]
        nz = np.flatnonzero(g)
        rand = rng.choice(nz, size=min(48, nz.size), replace=False) if nz.size else np.zeros(0, int)
        idx = np.unique(np.concatenate([top, rand])).astype(int)
        inputs = {k: v for k, v in t.items() if k not in ("grid", "hab", "force_a", "force_b", "virial")}
        inputs["pab"] = t["pab"].tolist()
        out[name] = {
            "inputs": inputs,
            "hab": t["hab"].tolist(),
            "forces": [t["force_a"], t["force_b"]],
            "virial": t["virial"],
            "grid_sum": float(g.sum()),
            "grid_sumsq": float((g * g).sum()),
            "grid_maxabs": float(np.abs(g).max()),
            "grid_idx": idx.tolist(),
            "grid_val": g[idx].tolist(),
        }
    with gzip.open(DIGEST_FILE, "wt") as fh:
        json.dump(out, fh)
    print("wrote", DIGEST_FILE, os.path.getsize(DIGEST_FILE), "bytes")


if __name__ == "__main__":
    main()
