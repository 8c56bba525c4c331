"""Loader for tests/golden/ref_golden.npz (outputs of CP2K's REF backend on
tiny seeded task lists; written by tests/golden/make_ref_golden.py)."""
import os

import numpy as np

from cp2k_gb300.tasklist import BasisSet, TaskListInputs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_golden.npz")
CASES = ("ortho", "tricl")


def load(name: str):
    z = np.load(GOLDEN)
    g = lambda k: z[f"{name}/{k}"]
    basis = []
    i = 0
    while f"{name}/basis{i}/dims" in z:
        nset, nsgf, maxco, maxpgf = [int(x) for x in g(f"basis{i}/dims")]
        basis.append(BasisSet(nset=nset, nsgf=nsgf, maxco=maxco, maxpgf=maxpgf,
                              **{f: g(f"basis{i}/{f}") for f in
                                 ("lmin", "lmax", "npgf", "nsgf_set", "first_sgf", "sphi",
                                  "zet")}))
        i += 1
    keys = ("block_offsets", "atom_positions", "atom_kinds", "level_list", "iatom_list",
            "jatom_list", "iset_list", "jset_list", "ipgf_list", "jpgf_list",
            "border_mask_list", "block_num_list", "radius_list", "rab_list", "npts_global",
            "npts_local", "shift_local", "border_width", "dh", "dh_inv")
    kw = {k: g(k) for k in keys}
    inp = TaskListInputs(orthorhombic=bool(g("orthorhombic")), natoms=len(kw["atom_kinds"]),
                         nkinds=len(basis), nblocks=len(kw["block_offsets"]),
                         nlevels=len(kw["npts_global"]), basis_sets=basis,
                         buffer_size=int(g("buffer_size")), **kw)
    nl = inp.nlevels
    exp = {
        "rho100": [g(f"rho100_{l}") for l in range(nl)],
        "rho200": [g(f"rho200_{l}") for l in range(nl)],
    }
    for tau in (0, 1):
        for q in ("hab", "forces", "virial"):
            exp[f"{q}_tau{tau}"] = g(f"{q}_tau{tau}")
    return inp, g("pab"), [g(f"V{l}") for l in range(nl)], exp
