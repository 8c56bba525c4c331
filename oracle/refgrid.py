"""TEST INFRASTRUCTURE -- ctypes handle on CP2K's own grid library, compiled
from the reference sources into oracle/_ref/libcp2kgrid_ref.so by
``make -C oracle ref``.  Exists only where the CP2K tree was available at
build time; used to pin the oracle restatement and to produce the committed
golden fixtures, never by product code.

Calls go through the reference's public task-list API
(src/grid/grid_task_list.h) with GRID_BACKEND_REF or GRID_BACKEND_CPU selected
by grid_library_set_config (src/grid/common/grid_library.h).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libcp2kgrid_ref.so")
BACKEND_REF, BACKEND_CPU = 11, 12

_LIB = None


class OffloadBuffer(C.Structure):
    _fields_ = [("size", C.c_size_t), ("host_buffer", C.POINTER(C.c_double)),
                ("device_buffer", C.POINTER(C.c_double))]


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(LIB_PATH)
        L.grid_library_init()
        vp = C.c_void_p
        L.grid_library_set_config.argtypes = [C.c_int, C.c_bool, C.c_bool]
        L.offload_create_buffer.argtypes = [C.c_int, C.POINTER(C.POINTER(OffloadBuffer))]
        L.offload_free_buffer.argtypes = [C.POINTER(OffloadBuffer)]
        L.grid_create_basis_set.argtypes = [C.c_int] * 4 + [vp] * 7 + [C.POINTER(vp)]
        L.grid_free_basis_set.argtypes = [vp]
        L.grid_create_task_list.argtypes = [C.c_bool] + [C.c_int] * 5 + [vp] * 21 + [C.POINTER(vp)]
        L.grid_free_task_list.argtypes = [vp]
        L.grid_collocate_task_list.argtypes = [vp, C.c_int, C.c_int, vp, C.POINTER(OffloadBuffer),
                                               C.POINTER(C.POINTER(OffloadBuffer))]
        L.grid_integrate_task_list.argtypes = [vp, C.c_bool, C.c_int, C.c_int, vp,
                                               C.POINTER(OffloadBuffer),
                                               C.POINTER(C.POINTER(OffloadBuffer)),
                                               C.POINTER(OffloadBuffer), vp, vp]
        _LIB = L
    return _LIB


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class _Buf:
    def __init__(self, n):
        self.ptr = C.POINTER(OffloadBuffer)()
        lib().offload_create_buffer(max(int(n), 1), C.byref(self.ptr))
        self.n = int(n)

    def view(self):
        return np.ctypeslib.as_array(self.ptr.contents.host_buffer, shape=(max(self.n, 1),))[: self.n]

    def free(self):
        if self.ptr:
            lib().offload_free_buffer(self.ptr)
            self.ptr = C.POINTER(OffloadBuffer)()


class RefTaskList:
    """The reference's grid task list for a ``TaskListInputs``."""

    def __init__(self, inp, backend: int = BACKEND_REF):
        L = lib()
        L.grid_library_set_config(backend, False, False)
        self.inp = inp
        self._keep = []
        self._basis = []
        for b in inp.basis_sets:
            arrs = [np.ascontiguousarray(x, np.int32) for x in
                    (b.lmin, b.lmax, b.npgf, b.nsgf_set, b.first_sgf)]
            arrs += [np.ascontiguousarray(b.sphi, np.float64), np.ascontiguousarray(b.zet, np.float64)]
            self._keep.append(arrs)
            h = C.c_void_p()
            L.grid_create_basis_set(b.nset, b.nsgf, b.maxco, b.maxpgf, *[_p(a) for a in arrs], C.byref(h))
            self._basis.append(h)
        bs = (C.c_void_p * len(self._basis))(*[h.value for h in self._basis])
        self._keep.append(bs)
        i32 = lambda a: np.ascontiguousarray(a, np.int32)
        f64 = lambda a: np.ascontiguousarray(a, np.float64)
        arrays = [i32(inp.block_offsets), f64(inp.atom_positions), i32(inp.atom_kinds)]
        lists = [i32(inp.level_list), i32(inp.iatom_list), i32(inp.jatom_list), i32(inp.iset_list),
                 i32(inp.jset_list), i32(inp.ipgf_list), i32(inp.jpgf_list),
                 i32(inp.border_mask_list), i32(inp.block_num_list), f64(inp.radius_list),
                 f64(inp.rab_list)]
        levels = [i32(inp.npts_global), i32(inp.npts_local), i32(inp.shift_local),
                  i32(inp.border_width), f64(inp.dh), f64(inp.dh_inv)]
        self._keep += arrays + lists + levels
        self.h = C.c_void_p()
        L.grid_create_task_list(
            bool(inp.orthorhombic), inp.ntasks, inp.nlevels, inp.natoms, inp.nkinds,
            inp.nblocks, _p(arrays[0]), _p(arrays[1]), _p(arrays[2]),
            C.cast(bs, C.c_void_p), *[_p(a) for a in lists], *[_p(a) for a in levels],
            C.byref(self.h))
        self.npts_local = levels[1]

    def close(self):
        L = lib()
        if self.h:
            L.grid_free_task_list(self.h)
            self.h = C.c_void_p()
        for h in self._basis:
            L.grid_free_basis_set(h)
        self._basis = []

    def collocate(self, func, pab_blocks):
        inp = self.inp
        pab = _Buf(inp.buffer_size)
        pab.view()[:] = pab_blocks
        grids = [_Buf(n) for n in inp.grid_sizes()]
        arr = (C.POINTER(OffloadBuffer) * len(grids))(*[g.ptr for g in grids])
        lib().grid_collocate_task_list(self.h, int(func), inp.nlevels, _p(self.npts_local),
                                       pab.ptr, arr)
        out = [g.view().copy() for g in grids]
        for g in grids:
            g.free()
        pab.free()
        return out

    def integrate(self, grids, pab_blocks=None, compute_tau=False, forces=False, virial=False):
        inp = self.inp
        pab = None
        if pab_blocks is not None:
            pab = _Buf(inp.buffer_size)
            pab.view()[:] = pab_blocks
        gb = [_Buf(n) for n in inp.grid_sizes()]
        for b, g in zip(gb, grids):
            b.view()[:] = g
        arr = (C.POINTER(OffloadBuffer) * len(gb))(*[b.ptr for b in gb])
        hab = _Buf(inp.buffer_size)
        f = np.zeros((inp.natoms, 3)) if forces else None
        v = np.zeros((3, 3)) if virial else None
        lib().grid_integrate_task_list(
            self.h, bool(compute_tau), inp.natoms, inp.nlevels, _p(self.npts_local),
            pab.ptr if pab is not None else None, arr, hab.ptr,
            _p(f) if f is not None else None, _p(v) if v is not None else None)
        h = hab.view().copy()
        for b in gb:
            b.free()
        hab.free()
        if pab is not None:
            pab.free()
        return h, f, v
