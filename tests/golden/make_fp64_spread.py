"""Writes fp64_spread.json: how far two FP64 implementations of CP2K's REF
algorithm drift apart on the full-size synthetic workloads, in the
reference's own measure max |a - b| / max(1, |b|)
(src/grid/grid_task_list.c:249-262).

The two implementations are CP2K's REF backend itself (compiled from the CP2K
sources into oracle/_ref by `make -C oracle ref`) and the oracle (its C
restatement, oracle/grid_oracle.c).  They evaluate the same formulas; they
differ only in the order of FP64 operations (thread-local grid copies and
their reduction, loop nests).  Where this spread exceeds 1e-12, the
reference measure cannot resolve 1e-12 on that input, and the GPU parity
tests bound the FP64 path by a small multiple of the spread instead
(tests/test_parity_fullsize.py).

Inputs: cp2k_gb300.workload.config(name, seed=5) with density_blocks() and
potential_grids() -- the inputs of the full-size GPU parity tests.

Run from the repository root:  python tests/golden/make_fp64_spread.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from cp2k_gb300 import workload as W  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import refgrid as R  # noqa: E402
from sample_tasks import rel_diff  # noqa: E402

OUT = os.path.join(HERE, "fp64_spread.json")

CASES = {
    "c1_64atoms": (100, 200, 302, 412, 503, 602, 703, 801, 902, 906, 1003),
    "c2_512atoms": (100, 200),
    "c3_256atoms_triclinic": (100, 200),
}


def spread(name, funcs):
    inp = W.config(name, seed=5)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    ot = O.OracleTaskList(inp)
    rt = R.RefTaskList(inp, backend=R.BACKEND_REF)
    out = {"ntasks": int(inp.ntasks)}
    for func in funcs:
        a = rt.collocate(func, pab)
        b = ot.collocate(func, pab)
        out[f"rho{func}"] = max(rel_diff(x, y) for x, y in zip(a, b))
    for tau in (0, 1):
        h1, f1, v1 = rt.integrate(V, pab, compute_tau=bool(tau), forces=True, virial=True)
        h2, f2, v2 = ot.integrate(V, pab, compute_tau=bool(tau), forces=True, virial=True)
        out[f"hab_tau{tau}"] = rel_diff(h1, h2)
        out[f"forces_tau{tau}"] = rel_diff(f1, f2)
        out[f"virial_tau{tau}"] = rel_diff(v1, v2)
    rt.close()
    ot.close()
    return out


def main():
    if not R.available():
        sys.exit("oracle/_ref/libcp2kgrid_ref.so is missing: run `make -C oracle ref` first")
    res = {name: spread(name, funcs) for name, funcs in CASES.items()}
    with open(OUT, "w") as fh:
        json.dump(res, fh, indent=1, sort_keys=True)
        fh.write("\n")
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
