"""Writes ref_golden.npz: outputs of CP2K's own REF grid backend (compiled from
the CP2K sources into oracle/_ref by `make -C oracle ref`) on two tiny seeded
synthetic task lists, so that the oracle restatement and the GPU backend can be
checked against the reference itself where the CP2K tree is absent.

Cases (seeded, see cp2k_gb300.workload.generate):
  ortho   6 atoms, 6 A cubic cell, levels 24^3/16^3/12^3, sets l<=2 / l<=1
  tricl   4 atoms, 7 A cell with angles 80/95/110 deg, levels 24^3/16^3, l<=3
Stored per case: the task-list inputs, the density-matrix blocks, the
potential grids, and REF's outputs: rho for GRID_FUNC_AB and GRID_FUNC_DADB,
hab / forces / virial for compute_tau false and true.

Run from the repository root:  python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cp2k_gb300 import workload as W  # noqa: E402
from oracle import refgrid as R  # noqa: E402

OUT = os.path.join(HERE, "ref_golden.npz")


def cases():
    ortho = W.generate(6, W.cubic_cell(6.0), [24, 16, 12], [(0.5, [2, 1]), (0.5, [1])],
                       (0.1, 20.0), seed=21)
    tricl = W.generate(4, W.triclinic_cell(7.0, 7.0, 7.0, 80.0, 95.0, 110.0), [24, 16],
                       [(1.0, [3, 1])], (0.2, 20.0), seed=22)
    return {"ortho": ortho, "tricl": tricl}


INPUT_KEYS = ("block_offsets", "atom_positions", "atom_kinds", "level_list", "iatom_list",
              "jatom_list", "iset_list", "jset_list", "ipgf_list", "jpgf_list",
              "border_mask_list", "block_num_list", "radius_list", "rab_list", "npts_global",
              "npts_local", "shift_local", "border_width", "dh", "dh_inv")


def main():
    out = {}
    for name, inp in cases().items():
        pab = W.density_blocks(inp, seed=31)
        V = W.potential_grids(inp, seed=32)
        rt = R.RefTaskList(inp)
        for k in INPUT_KEYS:
            out[f"{name}/{k}"] = getattr(inp, k)
        out[f"{name}/orthorhombic"] = np.array(inp.orthorhombic)
        out[f"{name}/buffer_size"] = np.array(inp.buffer_size)
        for i, b in enumerate(inp.basis_sets):
            for f in ("lmin", "lmax", "npgf", "nsgf_set", "first_sgf", "sphi", "zet"):
                out[f"{name}/basis{i}/{f}"] = getattr(b, f)
            out[f"{name}/basis{i}/dims"] = np.array([b.nset, b.nsgf, b.maxco, b.maxpgf])
        out[f"{name}/pab"] = pab
        for l, v in enumerate(V):
            out[f"{name}/V{l}"] = v
        for func in (100, 200):
            for l, g in enumerate(rt.collocate(func, pab)):
                out[f"{name}/rho{func}_{l}"] = g
        for tau in (0, 1):
            h, f, v = rt.integrate(V, pab, compute_tau=bool(tau), forces=True, virial=True)
            out[f"{name}/hab_tau{tau}"] = h
            out[f"{name}/forces_tau{tau}"] = f
            out[f"{name}/virial_tau{tau}"] = v
        rt.close()
        print(name, inp.ntasks, "tasks")
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
