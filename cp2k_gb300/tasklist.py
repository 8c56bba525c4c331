"""Host-side description of a grid task list: exactly the arrays that
``grid_create_task_list`` takes (src/grid/grid_task_list.h:59-72 of CP2K), as
numpy arrays, plus the basis sets (src/grid/common/grid_basis_set.h:52-61).

Conventions kept from the reference interface:
  * task lists are 1-based (level, atoms, sets, pgfs, block numbers);
  * ``block_offsets`` are 0-based element offsets into the pab/hab buffers;
  * ``atom_positions`` / ``rab_list`` are [n][3]; ``dh``/``dh_inv`` [nlevels][3][3]
    with the rows of dh being the grid step vectors;
  * a matrix block of atom pair (i <= j) is stored [nsgf_j][nsgf_i] (C order),
    i.e. Fortran column-major (nsgf_i, nsgf_j).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def ncoset(l: int) -> int:
    """Number of Cartesian functions with angular momentum <= l."""
    return 0 if l < 0 else (l + 1) * (l + 2) * (l + 3) // 6


@dataclass
class BasisSet:
    nset: int
    nsgf: int
    maxco: int
    maxpgf: int
    lmin: np.ndarray
    lmax: np.ndarray
    npgf: np.ndarray
    nsgf_set: np.ndarray
    first_sgf: np.ndarray  # 1-based
    sphi: np.ndarray  # [nsgf][maxco]
    zet: np.ndarray  # [nset][maxpgf]


@dataclass
class TaskListInputs:
    orthorhombic: bool
    natoms: int
    nkinds: int
    nblocks: int
    nlevels: int
    block_offsets: np.ndarray
    atom_positions: np.ndarray
    atom_kinds: np.ndarray
    basis_sets: list
    level_list: np.ndarray
    iatom_list: np.ndarray
    jatom_list: np.ndarray
    iset_list: np.ndarray
    jset_list: np.ndarray
    ipgf_list: np.ndarray
    jpgf_list: np.ndarray
    border_mask_list: np.ndarray
    block_num_list: np.ndarray
    radius_list: np.ndarray
    rab_list: np.ndarray
    npts_global: np.ndarray
    npts_local: np.ndarray
    shift_local: np.ndarray
    border_width: np.ndarray
    dh: np.ndarray
    dh_inv: np.ndarray
    buffer_size: int  # doubles in the pab/hab block buffer
    meta: dict = field(default_factory=dict)

    @property
    def ntasks(self) -> int:
        return int(len(self.level_list))

    def grid_sizes(self):
        return [int(np.prod(n)) for n in self.npts_local]


def identity_basis(n: int, lmin: int, lmax: int, zet: float) -> BasisSet:
    """One-set basis with an identity contraction matrix and npgf equal
    exponents, as the reference's replay harness builds it
    (src/grid/grid_replay.c:114-148)."""
    npgf = n // ncoset(lmax)
    assert npgf * ncoset(lmax) == n
    return BasisSet(
        nset=1, nsgf=n, maxco=n, maxpgf=npgf,
        lmin=np.array([lmin], np.int32), lmax=np.array([lmax], np.int32),
        npgf=np.array([npgf], np.int32), nsgf_set=np.array([n], np.int32),
        first_sgf=np.array([1], np.int32), sphi=np.eye(n),
        zet=np.full((1, npgf), zet))


def single_task_list(t: dict, ntasks: int = 1) -> TaskListInputs:
    """Task list holding ``ntasks`` copies of one recorded task, with two atoms
    and dummy identity basis sets, as the reference replays a .task file in
    batched mode (src/grid/grid_replay.c:154-214).  All blocks share offset 0."""
    ra = np.asarray(t["ra"], np.float64)
    rab = np.asarray(t["rab"], np.float64)
    la_max, lb_max = t["la_max"], t["lb_max"]
    ipgf = t["o1"] // ncoset(la_max) + 1
    jpgf = t["o2"] // ncoset(lb_max) + 1
    ba = identity_basis(t["n1"], t["la_min"], la_max, t["zeta"])
    bb = identity_basis(t["n2"], t["lb_min"], lb_max, t["zetb"])
    one = np.ones(ntasks, np.int32)
    return TaskListInputs(
        orthorhombic=bool(t["orthorhombic"]), natoms=2, nkinds=2, nblocks=1,
        nlevels=1, block_offsets=np.zeros(1, np.int32),
        atom_positions=np.stack([ra, ra + rab]), atom_kinds=np.array([1, 2], np.int32),
        basis_sets=[ba, bb], level_list=one.copy(), iatom_list=one.copy(),
        jatom_list=2 * one, iset_list=one.copy(), jset_list=one.copy(),
        ipgf_list=ipgf * one, jpgf_list=jpgf * one,
        border_mask_list=int(t["border_mask"]) * one, block_num_list=one.copy(),
        radius_list=np.full(ntasks, float(t["radius"])), rab_list=np.tile(rab, (ntasks, 1)),
        npts_global=np.array([t["npts_global"]], np.int32),
        npts_local=np.array([t["npts_local"]], np.int32),
        shift_local=np.array([t["shift_local"]], np.int32),
        border_width=np.array([t["border_width"]], np.int32),
        dh=np.array([t["dh"]], np.float64).reshape(1, 3, 3),
        dh_inv=np.array([t["dh_inv"]], np.float64).reshape(1, 3, 3),
        buffer_size=int(t["n1"] * t["n2"]))
