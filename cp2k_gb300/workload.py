"""Seeded synthetic GPW workloads (task lists, density-matrix blocks, potential
grids) with the shapes of the benchmark configurations.

The task-list arrays come from ``csrc/workload.c`` (a restatement of
Quickstep's screening, radius and grid-level rules); blocks and grids are
uniform in [-1, 1] from numpy's PCG64 with fixed seeds, diagonal blocks
symmetrised.  Lengths are in bohr.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import build
from .tasklist import BasisSet, TaskListInputs

ANGSTROM = 1.8897261246  # bohr per angstrom

_MAXL, _MAXE, _MAXS = 8, 2, 4


class _Params(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64), ("natoms", C.c_int), ("cell", C.c_double * 9),
        ("nlevels", C.c_int), ("npts", C.c_int * (3 * _MAXL)), ("cutoff", C.c_double * _MAXL),
        ("rel_cutoff", C.c_double), ("eps", C.c_double), ("nelem", C.c_int),
        ("elem_fraction", C.c_double * _MAXE), ("nsets", C.c_int * _MAXE),
        ("set_lmax", C.c_int * (_MAXE * _MAXS)), ("zet_min", C.c_double),
        ("zet_max", C.c_double), ("random_sphi", C.c_int), ("npgf", C.c_int * _MAXE),
        ("screen", C.c_int), ("eps_pgf_orb", C.c_double),
    ]


_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)


class _Out(C.Structure):
    _fields_ = [
        ("natoms", C.c_int), ("nkinds", C.c_int), ("ntasks", C.c_int),
        ("nblocks", C.c_int), ("nlevels", C.c_int), ("buffer_size", C.c_longlong),
        ("atom_positions", _dp), ("atom_kinds", _ip),
        ("nset", _ip), ("nsgf", _ip), ("maxco", _ip), ("maxpgf", _ip), ("set_off", _ip),
        ("lmin", _ip), ("lmax", _ip), ("npgf", _ip), ("nsgf_set", _ip), ("first_sgf", _ip),
        ("sphi_off", _ip), ("sphi", _dp), ("zet", _dp), ("maxpgf_all", C.c_int),
        ("block_offsets", _ip),
        ("level", _ip), ("iatom", _ip), ("jatom", _ip), ("iset", _ip), ("jset", _ip),
        ("ipgf", _ip), ("jpgf", _ip), ("border_mask", _ip), ("block_num", _ip),
        ("radius", _dp), ("rab", _dp),
        ("dh", C.c_double * (_MAXL * 9)), ("dh_inv", C.c_double * (_MAXL * 9)),
        ("nimg", C.c_int * 3), ("rmax", C.c_double),
        ("rpgf", _dp), ("set_radius", _dp), ("kind_radius", _dp),
    ]


_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(build.build_workload())
        L.wl_generate.restype = C.POINTER(_Out)
        L.wl_generate.argtypes = [C.POINTER(_Params)]
        L.wl_free.argtypes = [C.POINTER(_Out)]
        L.wl_retask.restype = C.c_int
        L.wl_retask.argtypes = [C.POINTER(_Out), C.POINTER(_Params), C.c_void_p]
        _LIB = L
    return _LIB


def cubic_cell(edge_angstrom: float) -> np.ndarray:
    return np.eye(3) * edge_angstrom * ANGSTROM


def triclinic_cell(a, b, c, alpha, beta, gamma) -> np.ndarray:
    """Cell rows (a along x, b in the xy plane), angles in degrees, lengths in
    angstrom; returned in bohr."""
    al, be, ga = (math.radians(x) for x in (alpha, beta, gamma))
    va = [a, 0.0, 0.0]
    vb = [b * math.cos(ga), b * math.sin(ga), 0.0]
    cx = math.cos(be)
    cy = (math.cos(al) - math.cos(be) * math.cos(ga)) / math.sin(ga)
    vc = [c * cx, c * cy, c * math.sqrt(1.0 - cx * cx - cy * cy)]
    return np.array([va, vb, vc]) * ANGSTROM


def _cutoffs(cell: np.ndarray, npts) -> list:
    """Level cutoffs (Ry) at the spacing of the 280 Ry / 128-point / 12.4 A
    grid: E = 280 * (h_ref / h)^2 with h the longest step vector."""
    h_ref = 12.4 * ANGSTROM / 128.0
    out = []
    for n in npts:
        h = max(np.linalg.norm(cell[d]) / n[d] for d in range(3))
        out.append(280.0 * (h_ref / h) ** 2)
    return out


# name -> generator settings.  elements: (fraction, [set lmax...], primitives
# per set).  "water" = O:H 1:2, O 3 sets up to l=2, H 2 sets up to l=1, two
# primitive exponents per set; every set spans l = 0..lmax.
CONFIGS = {
    "c1_64atoms": dict(natoms=64, cell=("cubic", 12.4), npts=[128, 96, 64, 48],
                       elements=[(1.0, [2, 2])], zet=(0.05, 30.0)),
    "c2_512atoms": dict(natoms=512, cell=("cubic", 24.8), npts=[216, 152, 108, 76, 54],
                        elements=[(1.0 / 3.0, [2, 2, 2], 2), (2.0 / 3.0, [1, 1], 2)],
                        zet=(0.04, 40.0)),
    "c3_256atoms_triclinic": dict(natoms=256, cell=("triclinic", 18.0, 18.0, 18.0, 80.0, 95.0, 110.0),
                                  npts=[180, 125, 87, 60], elements=[(1.0, [2, 4])],
                                  zet=(0.1, 80.0)),
    "c4_1024atoms": dict(natoms=1024, cell=("cubic", 31.2), npts=[272, 192, 136, 96, 68],
                         elements=[(1.0 / 3.0, [2, 2, 2], 2), (2.0 / 3.0, [1, 1], 2)],
                         zet=(0.04, 40.0)),
    "c4_2048atoms": dict(natoms=2048, cell=("cubic", 39.3), npts=[342, 242, 171, 121, 86],
                         elements=[(1.0 / 3.0, [2, 2, 2], 2), (2.0 / 3.0, [1, 1], 2)],
                         zet=(0.04, 40.0)),
    "c5_6144atoms": dict(natoms=6144, cell=("cubic", 56.7), npts=[480, 340, 240, 170, 120],
                         elements=[(1.0 / 3.0, [2, 2, 2], 2), (2.0 / 3.0, [1, 1], 2)],
                         zet=(0.04, 40.0)),
}


def make_cell(spec) -> np.ndarray:
    if spec[0] == "cubic":
        return cubic_cell(spec[1])
    return triclinic_cell(*spec[1:])


def generate(natoms: int, cell: np.ndarray, npts, elements, zet, seed: int = 1,
             rel_cutoff: float = 40.0, eps: float = 1e-10, random_sphi: bool = False,
             cutoffs=None, positions=None, screen: str = "prefactor",
             eps_pgf_orb: float = 1e-5) -> TaskListInputs:
    """Build a task list.  ``npts`` is a list of per-level point counts (int or
    3-tuple), finest first; ``elements`` a list of (fraction, [set lmax...]).
    ``positions`` ([natoms][3], bohr) replaces the seeded atom positions
    (same basis sets): the task list of a moved geometry.  ``screen``:
    "prefactor" keeps primitive pairs whose Gaussian-product prefactor
    exceeds eps (the benchmark workloads); "radius" screens by the basis
    radii as Quickstep's task_list_inner_loop does (radii from exp_radius
    at threshold ``eps_pgf_orb``)."""
    npts = [(n, n, n) if np.isscalar(n) else tuple(n) for n in npts]
    cell = np.asarray(cell, np.float64)
    p = _Params()
    p.seed = seed
    p.natoms = natoms
    p.cell[:] = list(cell.ravel())
    p.nlevels = len(npts)
    for l, n in enumerate(npts):
        for d in range(3):
            p.npts[3 * l + d] = int(n[d])
    cut = cutoffs if cutoffs is not None else _cutoffs(cell, npts)
    for l, c in enumerate(cut):
        p.cutoff[l] = c
    p.rel_cutoff = rel_cutoff
    p.eps = eps
    p.nelem = len(elements)
    for e, el in enumerate(elements):
        frac, lmaxs = el[0], el[1]
        p.npgf[e] = el[2] if len(el) > 2 else 1
        p.elem_fraction[e] = frac
        p.nsets[e] = len(lmaxs)
        for k, L in enumerate(lmaxs):
            p.set_lmax[e * _MAXS + k] = L
    p.zet_min, p.zet_max = zet
    p.random_sphi = int(random_sphi)
    if screen not in ("prefactor", "radius"):
        raise ValueError("screen must be 'prefactor' or 'radius'")
    p.screen = 1 if screen == "radius" else 0
    p.eps_pgf_orb = eps_pgf_orb
    L = _lib()
    op = L.wl_generate(C.byref(p))
    if not op:
        raise ValueError("invalid workload parameters")
    try:
        if positions is not None:
            pos = np.ascontiguousarray(positions, np.float64).reshape(natoms, 3)
            if L.wl_retask(op, C.byref(p), pos.ctypes.data_as(C.c_void_p)) != 0:
                raise ValueError("positions do not match the workload")
        o = op.contents
        nsets = int(np.ctypeslib.as_array(o.nset, shape=(o.natoms,)).sum())
        radii = dict(rpgf=_arr(o.rpgf, nsets * o.maxpgf_all, np.float64).reshape(nsets, -1),
                     set_radius=_arr(o.set_radius, nsets, np.float64),
                     kind_radius=_arr(o.kind_radius, o.nkinds, np.float64))
        return _to_inputs(o, cell, npts, cut, dict(natoms=natoms, seed=seed, zet=zet,
                                                   elements=elements, rel_cutoff=rel_cutoff,
                                                   eps=eps, nimg=list(o.nimg), rmax=o.rmax,
                                                   screen=screen, eps_pgf_orb=eps_pgf_orb,
                                                   **radii))
    finally:
        L.wl_free(op)


def _arr(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def _to_inputs(o, cell, npts, cutoffs, meta) -> TaskListInputs:
    na, nt, nb, nl = o.natoms, o.ntasks, o.nblocks, o.nlevels
    nset = _arr(o.nset, na, np.int32)
    nsgf = _arr(o.nsgf, na, np.int32)
    maxco = _arr(o.maxco, na, np.int32)
    set_off = _arr(o.set_off, na, np.int32)
    sphi_off = _arr(o.sphi_off, na, np.int64)
    tot_sets = int(nset.sum())
    lmax_all = _arr(o.lmax, tot_sets, np.int32)
    lmin_all = _arr(o.lmin, tot_sets, np.int32)
    npgf_all = _arr(o.npgf, tot_sets, np.int32)
    nsgfset_all = _arr(o.nsgf_set, tot_sets, np.int32)
    first_all = _arr(o.first_sgf, tot_sets, np.int32)
    mp = int(o.maxpgf_all)
    zet_all = _arr(o.zet, tot_sets * mp, np.float64).reshape(tot_sets, mp)
    sphi_all = _arr(o.sphi, int((nsgf.astype(np.int64) * maxco).sum()), np.float64)
    basis = []
    for k in range(na):
        s0, s1 = set_off[k], set_off[k] + nset[k]
        sp = sphi_all[sphi_off[k]: sphi_off[k] + nsgf[k] * maxco[k]].reshape(nsgf[k], maxco[k])
        basis.append(BasisSet(
            nset=int(nset[k]), nsgf=int(nsgf[k]), maxco=int(maxco[k]), maxpgf=mp,
            lmin=lmin_all[s0:s1].copy(), lmax=lmax_all[s0:s1].copy(),
            npgf=npgf_all[s0:s1].copy(), nsgf_set=nsgfset_all[s0:s1].copy(),
            first_sgf=first_all[s0:s1].copy(), sphi=sp.copy(),
            zet=zet_all[s0:s1].copy()))
    dh = np.ctypeslib.as_array(o.dh).reshape(-1, 3, 3)[:nl].copy()
    dh_inv = np.ctypeslib.as_array(o.dh_inv).reshape(-1, 3, 3)[:nl].copy()
    npts_arr = np.array(npts, np.int32)
    meta = dict(meta)
    meta["cutoffs_ry"] = list(cutoffs)
    meta["cell_bohr"] = cell.tolist()
    return TaskListInputs(
        orthorhombic=bool(np.allclose(cell - np.diag(np.diag(cell)), 0.0)),
        natoms=na, nkinds=na, nblocks=nb, nlevels=nl,
        block_offsets=_arr(o.block_offsets, nb, np.int32),
        atom_positions=_arr(o.atom_positions, 3 * na, np.float64).reshape(na, 3),
        atom_kinds=_arr(o.atom_kinds, na, np.int32), basis_sets=basis,
        level_list=_arr(o.level, nt, np.int32), iatom_list=_arr(o.iatom, nt, np.int32),
        jatom_list=_arr(o.jatom, nt, np.int32), iset_list=_arr(o.iset, nt, np.int32),
        jset_list=_arr(o.jset, nt, np.int32), ipgf_list=_arr(o.ipgf, nt, np.int32),
        jpgf_list=_arr(o.jpgf, nt, np.int32),
        border_mask_list=_arr(o.border_mask, nt, np.int32),
        block_num_list=_arr(o.block_num, nt, np.int32),
        radius_list=_arr(o.radius, nt, np.float64),
        rab_list=_arr(o.rab, 3 * nt, np.float64).reshape(nt, 3),
        npts_global=npts_arr.copy(), npts_local=npts_arr.copy(),
        shift_local=np.zeros((nl, 3), np.int32), border_width=np.zeros((nl, 3), np.int32),
        dh=dh, dh_inv=dh_inv, buffer_size=int(o.buffer_size), meta=meta)


def config(name: str, seed: int = 1, scale: float = 1.0, random_sphi: bool = False,
           positions=None, screen: str = "prefactor", **overrides) -> TaskListInputs:
    """A named benchmark configuration.  ``scale`` < 1 shrinks the atom count,
    the cell edge (at fixed density) and the grid point counts (at fixed
    spacing) for quick parity runs.  ``positions`` moves the atoms (see
    ``generate``)."""
    c = dict(CONFIGS[name])
    c.update(overrides)
    natoms = max(2, int(round(c["natoms"] * scale)))
    lin = (natoms / c["natoms"]) ** (1.0 / 3.0)
    cell = make_cell(c["cell"])
    npts = [max(8, int(round(n * lin))) for n in c["npts"]]
    cutoffs = _cutoffs(cell, [(n, n, n) for n in c["npts"]])
    return generate(natoms, cell * lin, npts, c["elements"], c["zet"], seed=seed,
                    random_sphi=random_sphi, cutoffs=cutoffs, positions=positions,
                    screen=screen)


def density_blocks(inp: TaskListInputs, seed: int = 2) -> np.ndarray:
    """Density-matrix block buffer: entries uniform in [-1, 1]; diagonal blocks
    (iatom == jatom) symmetrised."""
    rng = np.random.default_rng(seed)
    buf = rng.uniform(-1.0, 1.0, size=inp.buffer_size)
    # symmetrise diagonal blocks: find them from the tasks
    diag = np.unique(inp.block_num_list[inp.iatom_list == inp.jatom_list]) - 1
    atoms = {}
    for b, ia in zip(inp.block_num_list - 1, inp.iatom_list - 1):
        atoms.setdefault(int(b), int(ia))
    for b in diag:
        n = inp.basis_sets[inp.atom_kinds[atoms[int(b)]] - 1].nsgf
        off = inp.block_offsets[b]
        m = buf[off: off + n * n].reshape(n, n)
        buf[off: off + n * n] = (0.5 * (m + m.T)).ravel()
    return buf


def potential_grids(inp: TaskListInputs, seed: int = 3) -> list:
    rng = np.random.default_rng(seed)
    return [rng.uniform(-1.0, 1.0, size=n) for n in inp.grid_sizes()]
