"""Reader for CP2K's recorded single-task fixtures ("#Grid task v10" files,
src/grid/sample_tasks/*.task, format written by
src/grid/cpu/grid_cpu_collocate.c:196-219 and read by
src/grid/grid_replay.c:216-300), and for the compact digests of them that
tests/golden/make_sample_digests.py commits for runs without the CP2K tree."""
from __future__ import annotations

import gzip
import json
import os

import numpy as np



def _reference_root() -> str:
    """The CP2K source tree: CP2K_REFERENCE_ROOT, else the location the
    oracle's Makefile builds the reference library from."""
    root = os.environ.get("CP2K_REFERENCE_ROOT")
    if root:
        return root
    oracle_dir = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle")
    try:
        import subprocess
        r = subprocess.run(["make", "-s", "-C", oracle_dir, "print-ref-root"],
                           capture_output=True, text=True, timeout=30)
        return r.stdout.strip()
    except Exception:
        return ""


REFERENCE_ROOT = _reference_root()
SAMPLE_DIR = os.path.join(REFERENCE_ROOT, "src", "grid", "sample_tasks")
GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DIGEST_FILE = os.path.join(GOLDEN_DIR, "sample_task_digests.json.gz")

# the 13 tasks the reference unit test runs (src/grid/grid_unittest.c:96-108)
SAMPLE_TASKS = [
    "ortho_density_l0000", "ortho_density_l0122", "ortho_density_l2200",
    "ortho_density_l3300", "ortho_density_l3333", "ortho_density_l0505",
    "ortho_non_periodic", "ortho_tau", "general_density", "general_tau",
    "general_subpatch0", "general_subpatch16", "general_overflow",
]


def have_reference() -> bool:
    return os.path.isdir(SAMPLE_DIR)


def parse_task_file(path: str) -> dict:
    with open(path) as fh:
        lines = fh.read().splitlines()
    if lines[0] != "#Grid task v10" or lines[-1] != "#THE_END":
        raise ValueError(f"{path}: not a v10 task file")
    it = iter(lines[1:-1])
    t: dict = {}

    def nxt(key):
        parts = next(it).split()
        assert parts[0] == key, (parts[0], key)
        return parts[1:]

    for k in ("orthorhombic", "border_mask", "func", "la_max", "la_min", "lb_max", "lb_min"):
        t[k] = int(nxt(k)[0])
    for k in ("zeta", "zetb", "rscale"):
        t[k] = float(nxt(k)[0])
    for k in ("dh", "dh_inv"):
        t[k] = [[float(x) for x in nxt(k)[1:]] for _ in range(3)]
    for k in ("ra", "rab"):
        t[k] = [float(x) for x in nxt(k)]
    for k in ("npts_global", "npts_local", "shift_local", "border_width"):
        t[k] = [int(x) for x in nxt(k)]
    t["radius"] = float(nxt("radius")[0])
    for k in ("o1", "o2", "n1", "n2"):
        t[k] = int(nxt(k)[0])
    pab = np.zeros((t["n2"], t["n1"]))
    for i in range(t["n2"]):
        for j in range(t["n1"]):
            p = nxt("pab")
            assert int(p[0]) == i and int(p[1]) == j
            pab[i, j] = float(p[2])
    t["pab"] = pab
    nl = t["npts_local"]
    grid = np.zeros(nl[0] * nl[1] * nl[2])
    for _ in range(int(nxt("ngrid_nonzero")[0])):
        p = nxt("grid")
        i, j, k = int(p[0]), int(p[1]), int(p[2])
        grid[k * nl[1] * nl[0] + j * nl[0] + i] = float(p[3])
    t["grid"] = grid
    from cp2k_gb300.tasklist import ncoset
    hab = np.zeros((t["n2"], t["n1"]))
    for i in range(t["o2"], ncoset(t["lb_max"]) + t["o2"]):
        for j in range(t["o1"], ncoset(t["la_max"]) + t["o1"]):
            p = nxt("hab")
            assert int(p[0]) == i and int(p[1]) == j
            hab[i, j] = float(p[2])
    t["hab"] = hab
    t["force_a"] = [float(x) for x in nxt("force_a")]
    t["force_b"] = [float(x) for x in nxt("force_b")]
    t["virial"] = [[float(x) for x in nxt("virial")[1:]] for _ in range(3)]
    return t


def load_sample(name: str) -> dict:
    return parse_task_file(os.path.join(SAMPLE_DIR, name + ".task"))


def rel_diff(test, ref) -> float:
    """Max |test-ref| / max(1, |ref|): the reference's comparison measure
    (src/grid/grid_replay.c:443-502, grid_task_list.c:249-252)."""
    test = np.asarray(test, np.float64)
    ref = np.asarray(ref, np.float64)
    if ref.size == 0:
        return 0.0
    return float(np.max(np.abs(test - ref) / np.maximum(1.0, np.abs(ref))))


# ---------------------------------------------------------------- digests --
def load_digests() -> dict:
    with gzip.open(DIGEST_FILE, "rt") as fh:
        return json.load(fh)


def digest_task(d: dict) -> dict:
    """Task-description dict from a committed digest entry (inputs in full)."""
    t = dict(d["inputs"])
    t["pab"] = np.asarray(t["pab"], np.float64)
    return t
