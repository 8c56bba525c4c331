"""In-tree build of the package's native libraries.

* ``libgb300grid.so``  -- the CUDA backend and its C ABI (nvcc, sm_103a only;
  linked with cuFFT for the plane-wave transfer of the level grids);
* ``libgb300workload.so`` -- the host-only synthetic task-list generator (gcc).

Both land next to this file (``cp2k_gb300/``) and are git-ignored.  Builds run
in parallel and are skipped when the library is newer than its sources.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")

GRID_LIB = os.path.join(HERE, "libgb300grid.so")
WORKLOAD_LIB = os.path.join(HERE, "libgb300workload.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"build failed: {' '.join(cmd[:3])} ...")


def build_workload(force: bool = False) -> str:
    src = os.path.join(CSRC, "workload.c")
    if force or _stale(WORKLOAD_LIB, [src]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-o", WORKLOAD_LIB,
              src, "-lm"])
    return WORKLOAD_LIB


def grid_sources() -> tuple[list[str], list[str]]:
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    deps = cu + sorted(glob.glob(os.path.join(CSRC, "*.h"))) + sorted(
        glob.glob(os.path.join(CSRC, "*.cuh"))) + sorted(glob.glob(os.path.join(INCLUDE, "*.h")))
    return cu, deps


def build_grid(force: bool = False, verbose_ptxas: bool = False) -> str:
    cu, deps = grid_sources()
    if not cu:
        raise RuntimeError("no CUDA sources found")
    if not (force or _stale(GRID_LIB, deps)):
        return GRID_LIB
    objdir = os.path.join(HERE, "_build")
    os.makedirs(objdir, exist_ok=True)
    nvcc = _nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                    "-Xcompiler", "-ffp-contract=off",
                    "-Xcompiler", "-fvisibility=hidden", "-I", INCLUDE, "-I", CSRC,
                    "--expt-relaxed-constexpr"]
    if verbose_ptxas:
        flags += ["-Xptxas", "-v"]
    objs = [os.path.join(objdir, os.path.basename(s) + ".o") for s in cu]

    def compile_one(pair):
        src, obj = pair
        _run([nvcc, *flags, "-c", src, "-o", obj])

    with ThreadPoolExecutor(max_workers=max(1, len(cu))) as ex:
        list(ex.map(compile_one, zip(cu, objs)))
    _run([nvcc, *ARCH, "-shared", "-o", GRID_LIB, *objs, "-lcudart", "-lcuda", "-lcufft",
          "-lpthread"])
    return GRID_LIB


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        futs = [ex.submit(build_workload, force), ex.submit(build_grid, force)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
