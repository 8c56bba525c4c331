"""TEST INFRASTRUCTURE -- Python handle on the CPU oracle (liboracle.so).

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s cpu_baseline and
reference legs may import this module, and only as the checker or as the timed
CPU baseline.  The oracle is a plain-C FP64 restatement of CP2K's REF grid
backend (src/grid/ref/*); see grid_oracle.h.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_LOCK = threading.Lock()

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    path = os.path.join(_HERE, "liboracle.so")
    if force or not os.path.exists(path) or os.path.getmtime(path) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("grid_oracle.c", "grid_oracle.h")
    ):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return path


def lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            L = C.CDLL(build())
            vp = C.c_void_p
            L.oracle_create_basis_set.argtypes = [C.c_int] * 4 + [_ip] * 5 + [_dp, _dp, C.POINTER(vp)]
            L.oracle_free_basis_set.argtypes = [vp]
            L.oracle_create_task_list.argtypes = (
                [C.c_bool] + [C.c_int] * 5 + [_ip, _dp, _ip, C.POINTER(vp)]
                + [_ip] * 9 + [_dp, _dp] + [_ip] * 4 + [_dp, _dp, C.POINTER(vp)]
            )
            L.oracle_free_task_list.argtypes = [vp]
            L.oracle_collocate_task_list.argtypes = [vp, C.c_int, C.c_int, _dp, C.POINTER(C.POINTER(C.c_double))]
            L.oracle_integrate_task_list.argtypes = [
                vp, C.c_bool, C.c_int, C.c_int, vp, C.POINTER(C.POINTER(C.c_double)),
                _dp, C.c_size_t, vp, vp]
            L.oracle_collocate_pgf_product.argtypes = (
                [C.c_bool, C.c_int, C.c_int] + [C.c_int] * 4 + [C.c_double] * 3
                + [_dp] * 4 + [_ip] * 4 + [C.c_double] + [C.c_int] * 4 + [_dp, _dp])
            L.oracle_integrate_pgf_product.argtypes = (
                [C.c_bool, C.c_bool, C.c_int] + [C.c_int] * 4 + [C.c_double] * 2
                + [_dp] * 4 + [_ip] * 4 + [C.c_double] + [C.c_int] * 4
                + [_dp, _dp, vp, vp, vp, vp, vp, vp])
            L.oracle_count_task_points.restype = C.c_longlong
            L.oracle_count_task_points.argtypes = [vp, C.c_int, vp, vp]
            _LIB = L
    return _LIB


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# --------------------------------------------------------------------------
# single-task (pgf product) entry points
# --------------------------------------------------------------------------
def collocate_pgf_product(t: dict) -> np.ndarray:
    """Collocate one task description (keys as in a CP2K .task file)."""
    nl = t["npts_local"]
    grid = np.zeros(int(nl[0] * nl[1] * nl[2]), dtype=np.float64)
    lib().oracle_collocate_pgf_product(
        bool(t["orthorhombic"]), int(t["border_mask"]), int(t["func"]),
        t["la_max"], t["la_min"], t["lb_max"], t["lb_min"],
        t["zeta"], t["zetb"], t["rscale"], _f64(t["dh"]), _f64(t["dh_inv"]),
        _f64(t["ra"]), _f64(t["rab"]), _i32(t["npts_global"]), _i32(nl),
        _i32(t["shift_local"]), _i32(t["border_width"]), t["radius"],
        t["o1"], t["o2"], t["n1"], t["n2"], _f64(t["pab"]), grid)
    return grid


def integrate_pgf_product(t: dict, grid: np.ndarray, compute_tau: bool,
                          forces: bool = True, virial: bool = True, derivatives: bool = False):
    """Integrate one task; returns (hab[n2][n1], forces[2][3], virials[2][3][3])
    and, with derivatives=True, also (hdab[n2][n1][3], hadb[n2][n1][3],
    a_hdab[n2][n1][3][3]) (grid_ref_integrate.c:121-145; not with tau)."""
    hab = np.zeros((t["n2"], t["n1"]), dtype=np.float64)
    f = np.zeros((2, 3)) if forces else None
    v = np.zeros((2, 3, 3)) if virial else None
    hd = np.zeros((t["n2"], t["n1"], 3)) if derivatives else None
    ha = np.zeros((t["n2"], t["n1"], 3)) if derivatives else None
    ahd = np.zeros((t["n2"], t["n1"], 3, 3)) if derivatives else None
    pab = _f64(t["pab"]) if (forces or virial) else None
    lib().oracle_integrate_pgf_product(
        bool(t["orthorhombic"]), bool(compute_tau), int(t["border_mask"]),
        t["la_max"], t["la_min"], t["lb_max"], t["lb_min"], t["zeta"], t["zetb"],
        _f64(t["dh"]), _f64(t["dh_inv"]), _f64(t["ra"]), _f64(t["rab"]),
        _i32(t["npts_global"]), _i32(t["npts_local"]), _i32(t["shift_local"]),
        _i32(t["border_width"]), t["radius"], t["o1"], t["o2"], t["n1"], t["n2"],
        _f64(grid), hab, _ptr(pab), _ptr(f), _ptr(v), _ptr(hd), _ptr(ha), _ptr(ahd))
    if derivatives:
        return hab, f, v, hd, ha, ahd
    return hab, f, v


# --------------------------------------------------------------------------
# task lists
# --------------------------------------------------------------------------
class OracleTaskList:
    """Oracle twin of a grid task list built from a ``TaskListInputs``
    (cp2k_gb300.tasklist) -- same arrays as grid_create_task_list."""

    def __init__(self, inp):
        L = lib()
        self._keep = []
        self._basis = []
        for b in inp.basis_sets:
            h = C.c_void_p()
            L.oracle_create_basis_set(
                b.nset, b.nsgf, b.maxco, b.maxpgf, _i32(b.lmin), _i32(b.lmax),
                _i32(b.npgf), _i32(b.nsgf_set), _i32(b.first_sgf),
                _f64(b.sphi), _f64(b.zet), C.byref(h))
            self._basis.append(h)
        arr = (C.c_void_p * len(self._basis))(*[h.value for h in self._basis])
        self._keep.append(arr)
        self.inp = inp
        self.h = C.c_void_p()
        L.oracle_create_task_list(
            bool(inp.orthorhombic), inp.ntasks, inp.nlevels, inp.natoms, inp.nkinds,
            inp.nblocks, _i32(inp.block_offsets), _f64(inp.atom_positions),
            _i32(inp.atom_kinds), C.cast(arr, C.POINTER(C.c_void_p)),
            _i32(inp.level_list), _i32(inp.iatom_list), _i32(inp.jatom_list),
            _i32(inp.iset_list), _i32(inp.jset_list), _i32(inp.ipgf_list),
            _i32(inp.jpgf_list), _i32(inp.border_mask_list), _i32(inp.block_num_list),
            _f64(inp.radius_list), _f64(inp.rab_list), _i32(inp.npts_global),
            _i32(inp.npts_local), _i32(inp.shift_local), _i32(inp.border_width),
            _f64(inp.dh), _f64(inp.dh_inv), C.byref(self.h))

    def close(self):
        L = lib()
        if self.h:
            L.oracle_free_task_list(self.h)
            self.h = C.c_void_p()
        for h in self._basis:
            L.oracle_free_basis_set(h)
        self._basis = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def collocate(self, func: int, pab_blocks: np.ndarray) -> list:
        grids = [np.zeros(int(np.prod(n)), dtype=np.float64) for n in self.inp.npts_local]
        ptrs = (C.POINTER(C.c_double) * len(grids))(
            *[g.ctypes.data_as(C.POINTER(C.c_double)) for g in grids])
        lib().oracle_collocate_task_list(self.h, int(func), len(grids), _f64(pab_blocks), ptrs)
        return grids

    def integrate(self, grids, pab_blocks=None, compute_tau=False, forces=False,
                  virial=False):
        """Returns (hab_blocks, forces[natoms][3] or None, virial[3][3] or None)."""
        inp = self.inp
        gl = [_f64(g) for g in grids]
        ptrs = (C.POINTER(C.c_double) * len(gl))(
            *[g.ctypes.data_as(C.POINTER(C.c_double)) for g in gl])
        hab = np.zeros(int(inp.buffer_size), dtype=np.float64)
        f = np.zeros((inp.natoms, 3)) if forces else None
        v = np.zeros((3, 3)) if virial else None
        pab = _f64(pab_blocks) if pab_blocks is not None else None
        lib().oracle_integrate_task_list(
            self.h, bool(compute_tau), inp.natoms, len(gl), _ptr(pab), ptrs, hab,
            hab.size, _ptr(f), _ptr(v))
        return hab, f, v

    def count_points(self, func: int = 100):
        """Per-task grid points visited and contraction order lp (input order)."""
        n = self.inp.ntasks
        pts = np.zeros(n, dtype=np.int64)
        lp = np.zeros(n, dtype=np.int32)
        lib().oracle_count_task_points(self.h, int(func), _ptr(pts), _ptr(lp))
        return pts, lp
