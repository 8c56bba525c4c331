"""Python mirror of CP2K's grid API (src/grid/grid_api.F) over the C ABI of
libgb300grid.so (include/grid_gb300.h).

The classes follow the Fortran wrappers' argument meaning:
  * ``BasisSet``      -> grid_create_basis_set / grid_free_basis_set
  * ``GridTaskList``  -> grid_create_task_list / grid_collocate_task_list /
                         grid_integrate_task_list / grid_free_task_list
with host buffers passed as CP2K's offload buffers (pinned host + device
copies).  Device-resident variants take torch CUDA tensors and call the
``grid_gb300_*_device_async`` entry points.  There is no CPU path: loading
fails loudly when the CUDA library is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build
from .tasklist import TaskListInputs

GRID_FUNC_AB = 100
GRID_FUNC_DADB = 200
GRID_BACKEND_AUTO, GRID_BACKEND_REF, GRID_BACKEND_CPU = 10, 11, 12
GRID_BACKEND_DGEMM, GRID_BACKEND_GPU, GRID_BACKEND_GB300 = 13, 14, 15
FP64, MIXED, FP32 = 0, 1, 2
SCHEDULE_SIZE, SCHEDULE_MODEL, SCHEDULE_INPUT = 0, 1, 2

# every grid_func value (src/grid/common/grid_constants.h:10-46)
GRID_FUNCS = [100, 200, 301, 302, 303, 411, 412, 413, 421, 422, 423, 431, 432, 433,
              501, 502, 503, 601, 602, 603, 701, 702, 703, 801, 802, 803,
              901, 902, 903, 904, 905, 906, 1001, 1002, 1003]


class OffloadBuffer(C.Structure):
    _fields_ = [("size", C.c_size_t), ("host_buffer", C.POINTER(C.c_double)),
                ("device_buffer", C.POINTER(C.c_double))]


_LIB = None
vp = C.c_void_p


def lib_path() -> str:
    return build.GRID_LIB


def lib():
    """Load libgb300grid.so.  Raises if it has not been built."""
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run cp2k_gb300.build.build_all() first")
        L = C.CDLL(path)
        L.offload_create_buffer.argtypes = [C.c_int, C.POINTER(C.POINTER(OffloadBuffer))]
        L.offload_free_buffer.argtypes = [C.POINTER(OffloadBuffer)]
        L.offload_get_buffer_host_pointer.argtypes = [C.POINTER(OffloadBuffer)]
        L.offload_get_buffer_host_pointer.restype = C.POINTER(C.c_double)
        L.grid_create_basis_set.argtypes = [C.c_int] * 4 + [vp] * 7 + [C.POINTER(vp)]
        L.grid_free_basis_set.argtypes = [vp]
        L.grid_library_init.argtypes = []
        L.grid_library_finalize.argtypes = []
        L.grid_library_set_config.argtypes = [C.c_int, C.c_bool, C.c_bool]
        create_args = [C.c_bool] + [C.c_int] * 5 + [vp] * 21 + [C.POINTER(vp)]
        L.grid_create_task_list.argtypes = create_args
        L.grid_gb300_create_task_list.argtypes = create_args
        L.grid_free_task_list.argtypes = [vp]
        L.grid_gb300_free_task_list.argtypes = [vp]
        L.grid_collocate_task_list.argtypes = [vp, C.c_int, C.c_int, vp, C.POINTER(OffloadBuffer),
                                               C.POINTER(C.POINTER(OffloadBuffer))]
        L.grid_integrate_task_list.argtypes = [vp, C.c_bool, C.c_int, C.c_int, vp,
                                               C.POINTER(OffloadBuffer),
                                               C.POINTER(C.POINTER(OffloadBuffer)),
                                               C.POINTER(OffloadBuffer), vp, vp]
        L.grid_gb300_collocate_task_list.argtypes = [vp, C.c_int, C.c_int, C.POINTER(OffloadBuffer),
                                                     C.POINTER(C.POINTER(OffloadBuffer))]
        L.grid_gb300_integrate_task_list.argtypes = [vp, C.c_bool, C.c_int, C.POINTER(OffloadBuffer),
                                                     C.POINTER(C.POINTER(OffloadBuffer)),
                                                     C.POINTER(OffloadBuffer), vp, vp]
        L.grid_gb300_collocate_device_async.argtypes = [vp, C.c_int, vp, vp, vp]
        L.grid_gb300_integrate_device_async.argtypes = [vp, C.c_bool, vp, vp, vp, vp, vp, vp]
        L.grid_gb300_set_precision.argtypes = [vp, C.c_int]
        L.grid_gb300_get_precision.argtypes = [vp]
        L.grid_gb300_set_schedule.argtypes = [vp, C.c_int]
        L.grid_gb300_set_mixed_threshold.argtypes = [vp, C.c_double]
        L.grid_gb300_mixed_split.argtypes = [vp, vp, vp]
        L.grid_gb300_task_list_info.argtypes = [vp, vp, vp, vp, vp]
        L.grid_gb300_task_sizes.argtypes = [vp, vp, vp]
        L.grid_gb300_last_timings.argtypes = [vp, vp]
        L.grid_gb300_collocate_pgf_product_static.restype = C.c_int
        L.grid_gb300_collocate_pgf_product_static.argtypes = (
            [C.c_bool, C.c_int, C.c_int] + [C.c_int] * 4 + [C.c_double] * 3 + [vp] * 4
            + [vp] * 4 + [C.c_double] + [C.c_int] * 4 + [vp, vp, vp])
        L.grid_gb300_static_scratch_bytes.restype = C.c_size_t
        L.grid_gb300_static_scratch_error.restype = C.c_char_p
        L.grid_gb300_backend_handle.argtypes = [vp]
        L.grid_gb300_backend_handle.restype = vp
        L.grid_gb300_kernel_launches.restype = C.c_longlong
        L.grid_gb300_capture_step.argtypes = [vp, C.c_int, vp, vp, C.c_bool, vp, vp, vp, vp, vp]
        L.grid_gb300_capture_step.restype = vp
        L.grid_gb300_step_graph_launch.argtypes = [vp, vp]
        L.grid_gb300_step_graph_wait.argtypes = [vp, vp]
        L.grid_gb300_step_graph_kernels.argtypes = [vp]
        L.grid_gb300_step_graph_kernels.restype = C.c_longlong
        L.grid_gb300_step_graph_free.argtypes = [vp]
        L.grid_gb300_autotune.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp]
        L.grid_gb300_autotune.restype = C.c_double
        L.grid_gb300_set_collocate_variant.argtypes = [vp, C.c_int]
        L.grid_gb300_set_model_bin_width.argtypes = [vp, C.c_double]
        L.grid_gb300_set_transform_variant.argtypes = [vp, C.c_int]
        L.grid_gb300_set_copy_chunks.argtypes = [vp, C.c_int]
        L.grid_gb300_set_queue_streams.argtypes = [vp, C.c_int]
        L.grid_gb300_set_tensor_integrate.argtypes = [vp, C.c_int]
        L.grid_gb300_set_row_split.argtypes = [vp, C.c_int]
        L.grid_gb300_set_tensor_collocate.argtypes = [vp, C.c_int]
        L.grid_gb300_row_split_stats.argtypes = [vp, vp, vp]
        L.grid_gb300_tuned_split.argtypes = [vp]
        L.grid_gb300_tuned_split.restype = C.c_int
        L.grid_gb300_set_launch_timing.argtypes = [vp, C.c_int]
        L.grid_gb300_launch_timings.argtypes = [vp, C.c_int, vp]
        L.grid_gb300_launch_timings.restype = C.c_int
        L.grid_gb300_set_task_timing.argtypes = [vp, C.c_int]
        L.grid_gb300_task_cycles.argtypes = [vp, vp]
        L.grid_gb300_task_features.argtypes = [vp, vp]
        L.grid_gb300_cost_model_nparams.restype = C.c_int
        L.grid_gb300_cost_model_work_floats.argtypes = [C.c_int]
        L.grid_gb300_cost_model_work_floats.restype = C.c_size_t
        L.grid_gb300_cost_model_loss_grad.argtypes = [vp, vp, vp, C.c_int, vp, vp, vp, vp]
        L.grid_gb300_cost_model_adam.argtypes = [vp, vp, vp, vp, C.c_int] + [C.c_float] * 4 + [vp]
        L.grid_gb300_cost_model_predict.argtypes = [vp, vp, C.c_int, vp, vp, vp]
        L.grid_gb300_apply_cost_model.argtypes = [vp, vp, vp, vp]
        L.grid_gb300_last_error.restype = C.c_char_p
        L.grid_library_init()
        _LIB = L
    return _LIB


class LaunchInfo(C.Structure):
    _fields_ = [("phase", C.c_int), ("precision", C.c_int), ("general", C.c_int),
                ("lp_bucket", C.c_int), ("ntasks", C.c_int), ("warps_per_block", C.c_int),
                ("blocks", C.c_int), ("points", C.c_longlong), ("flops", C.c_double),
                ("ms", C.c_double), ("work_items", C.c_int)]


def kernel_launches() -> int:
    return int(lib().grid_gb300_kernel_launches())


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Buffer:
    """CP2K offload buffer: pinned host memory + device memory of n doubles."""

    def __init__(self, n: int):
        self.n = int(n)
        self.ptr = C.POINTER(OffloadBuffer)()
        lib().offload_create_buffer(max(self.n, 0), C.byref(self.ptr))

    @property
    def host(self) -> np.ndarray:
        if self.n == 0:
            return np.zeros(0)
        return np.ctypeslib.as_array(self.ptr.contents.host_buffer, shape=(self.n,))

    @property
    def device_ptr(self) -> int:
        return C.cast(self.ptr.contents.device_buffer, C.c_void_p).value

    def free(self):
        if self.ptr:
            lib().offload_free_buffer(self.ptr)
            self.ptr = C.POINTER(OffloadBuffer)()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class BasisSet:
    def __init__(self, b):
        self._arrays = [np.ascontiguousarray(x, np.int32) for x in
                        (b.lmin, b.lmax, b.npgf, b.nsgf_set, b.first_sgf)]
        self._arrays += [np.ascontiguousarray(b.sphi, np.float64),
                         np.ascontiguousarray(b.zet, np.float64)]
        self.h = C.c_void_p()
        lib().grid_create_basis_set(b.nset, b.nsgf, b.maxco, b.maxpgf,
                                    *[_p(a) for a in self._arrays], C.byref(self.h))

    def free(self):
        if self.h:
            lib().grid_free_basis_set(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def host_digest(inp: TaskListInputs) -> np.ndarray:
    """grid_gb300_host_digest: hashes of the host-side task-list preparation
    (no GPU needed); 12 unsigned 64-bit words."""
    L = lib()
    basis = [BasisSet(b) for b in inp.basis_sets]
    bs = (C.c_void_p * max(1, len(basis)))(*[b.h.value for b in basis])
    i32 = lambda a: np.ascontiguousarray(a, np.int32)
    f64 = lambda a: np.ascontiguousarray(a, np.float64)
    head = [i32(inp.block_offsets), f64(inp.atom_positions), i32(inp.atom_kinds)]
    lists = [i32(inp.level_list), i32(inp.iatom_list), i32(inp.jatom_list),
             i32(inp.iset_list), i32(inp.jset_list), i32(inp.ipgf_list), i32(inp.jpgf_list),
             i32(inp.border_mask_list), i32(inp.block_num_list), f64(inp.radius_list),
             f64(inp.rab_list)]
    levels = [i32(inp.npts_global), i32(inp.npts_local), i32(inp.shift_local),
              i32(inp.border_width), f64(inp.dh), f64(inp.dh_inv)]
    out = np.zeros(12, np.uint64)
    L.grid_gb300_host_digest(bool(inp.orthorhombic), inp.ntasks, inp.nlevels, inp.natoms,
                             inp.nkinds, inp.nblocks, *[_p(a) for a in head],
                             C.cast(bs, C.c_void_p), *[_p(a) for a in lists],
                             *[_p(a) for a in levels], _p(out))
    for b in basis:
        b.free()
    return out


class GridTaskList:
    """A GB300 task list for ``TaskListInputs`` (see cp2k_gb300.tasklist).

    ``api="cp2k"`` goes through grid_create_task_list & co. (the CP2K surface),
    ``api="backend"`` through grid_gb300_* (what CP2K's dispatcher binds)."""

    def __init__(self, inp: TaskListInputs, precision: int | None = FP64,
                 schedule: int | None = SCHEDULE_SIZE, api: str = "backend"):
        # precision / schedule None: keep what the library chose at creation
        # (at the CP2K surface the environment may set the precision)
        self.api = api
        self.h = C.c_void_p()
        self._create(inp)
        if precision is not None:
            self.set_precision(precision)
        if schedule is not None:
            self.set_schedule(schedule)

    def _create(self, inp: TaskListInputs):
        """grid_create_task_list (or grid_gb300_create_task_list) into self.h;
        a non-NULL handle is re-created in place, as CP2K does at every change
        of geometry (src/grid/grid_task_list.c:42-63)."""
        L = lib()
        old_basis = getattr(self, "basis", [])
        self.inp = inp
        self.basis = [BasisSet(b) for b in inp.basis_sets]
        self._bs = (C.c_void_p * max(1, len(self.basis)))(*[b.h.value for b in self.basis])
        i32 = lambda a: np.ascontiguousarray(a, np.int32)
        f64 = lambda a: np.ascontiguousarray(a, np.float64)
        self._arrays = [i32(inp.block_offsets), f64(inp.atom_positions), i32(inp.atom_kinds)]
        lists = [i32(inp.level_list), i32(inp.iatom_list), i32(inp.jatom_list),
                 i32(inp.iset_list), i32(inp.jset_list), i32(inp.ipgf_list), i32(inp.jpgf_list),
                 i32(inp.border_mask_list), i32(inp.block_num_list), f64(inp.radius_list),
                 f64(inp.rab_list)]
        levels = [i32(inp.npts_global), i32(inp.npts_local), i32(inp.shift_local),
                  i32(inp.border_width), f64(inp.dh), f64(inp.dh_inv)]
        self._arrays += lists + levels
        self.npts_local = levels[1]
        fn = L.grid_create_task_list if self.api == "cp2k" else L.grid_gb300_create_task_list
        fn(bool(inp.orthorhombic), inp.ntasks, inp.nlevels, inp.natoms, inp.nkinds,
           inp.nblocks, _p(self._arrays[0]), _p(self._arrays[1]), _p(self._arrays[2]),
           C.cast(self._bs, C.c_void_p), *[_p(a) for a in lists], *[_p(a) for a in levels],
           C.byref(self.h))
        self.impl = self._impl_handle()
        # the list kept pointers to the old basis sets until now
        for b in old_basis:
            b.free()
        for buf in ([getattr(self, "_pab", None), getattr(self, "_hab", None)]
                    + list(getattr(self, "_grids", None) or [])):
            if buf is not None:
                buf.free()
        self._pab = None
        self._hab = None
        self._grids = None

    @classmethod
    def from_generator(cls, gen: "TaskGenerator", positions=None, precision: int | None = FP64,
                       schedule: int | None = SCHEDULE_SIZE, existing: "GridTaskList" = None):
        """A backend task list from the generator's last run through
        grid_gb300_taskgen_create_task_list; ``existing`` is re-created in
        place (its settings kept), as at a change of geometry."""
        inp = gen.inputs(positions)
        self = existing if existing is not None else cls.__new__(cls)
        if existing is None:
            self.api = "backend"
            self.h = C.c_void_p()
        old_basis = getattr(self, "basis", [])
        old_inp = getattr(self, "inp", None)
        if old_basis and old_inp is not None and old_inp.basis_sets is inp.basis_sets:
            old_basis = []  # the same basis sets: keep their handles
        else:
            self.basis = [BasisSet(b) for b in inp.basis_sets]
            self._bs = (C.c_void_p * max(1, len(self.basis)))(*[b.h.value for b in self.basis])
        self.inp = inp
        i32 = lambda a: np.ascontiguousarray(a, np.int32)
        f64 = lambda a: np.ascontiguousarray(a, np.float64)
        levels = [i32(inp.npts_global), i32(inp.npts_local), i32(inp.shift_local),
                  i32(inp.border_width), f64(inp.dh), f64(inp.dh_inv)]
        self._arrays = levels
        self.npts_local = levels[1]
        import time
        t0 = time.perf_counter()
        lib().grid_gb300_taskgen_create_task_list(gen.h, bool(inp.orthorhombic), inp.nlevels,
                                                  C.cast(self._bs, C.c_void_p),
                                                  *[_p(a) for a in levels], C.byref(self.h))
        self.create_s = time.perf_counter() - t0  # the C call alone
        self.impl = self.h
        for b in old_basis:
            b.free()
        for buf in ([getattr(self, "_pab", None), getattr(self, "_hab", None)]
                    + list(getattr(self, "_grids", None) or [])):
            if buf is not None:
                buf.free()
        self._pab = None
        self._hab = None
        self._grids = None
        if existing is None:
            if precision is not None:
                self.set_precision(precision)
            if schedule is not None:
                self.set_schedule(schedule)
        return self

    def recreate(self, inp: TaskListInputs):
        """Re-create the task list through its existing handle for new inputs
        (a moved geometry); the backend keeps the settings made on it."""
        self._create(inp)

    def _impl_handle(self):
        if self.api == "cp2k":
            return C.c_void_p(lib().grid_gb300_backend_handle(self.h))
        return self.h

    # ------------------------------------------------------------ settings
    def set_precision(self, precision: int):
        lib().grid_gb300_set_precision(self.impl, int(precision))

    def set_schedule(self, schedule: int):
        lib().grid_gb300_set_schedule(self.impl, int(schedule))

    def set_mixed_threshold(self, tau: float):
        lib().grid_gb300_set_mixed_threshold(self.impl, float(tau))

    def mixed_split(self):
        ft, fp = C.c_double(), C.c_double()
        lib().grid_gb300_mixed_split(self.impl, C.byref(ft), C.byref(fp))
        return ft.value, fp.value

    def sizes(self):
        """(grid points visited, lp) per task in input order."""
        n = self.inp.ntasks
        pts = np.zeros(n, np.int64)
        lp = np.zeros(n, np.int32)
        lib().grid_gb300_task_sizes(self.impl, _p(pts), _p(lp))
        return pts, lp

    def set_launch_timing(self, enable: bool = True):
        lib().grid_gb300_set_launch_timing(self.impl, int(bool(enable)))

    def launch_timings(self):
        """Per grid-kernel launch of the last call (launch timing enabled):
        list of dicts with phase, precision, general, lp_bucket, ntasks,
        warps_per_block, blocks, points, flops, ms, work_items."""
        n = lib().grid_gb300_launch_timings(self.impl, 0, None)
        arr = (LaunchInfo * max(n, 1))()
        lib().grid_gb300_launch_timings(self.impl, n, C.cast(arr, C.c_void_p))
        return [{f: getattr(arr[i], f) for f, _ in LaunchInfo._fields_} for i in range(n)]

    def set_task_timing(self, enable: bool = True):
        lib().grid_gb300_set_task_timing(self.impl, int(bool(enable)))

    def task_cycles(self) -> np.ndarray:
        """clock64 cycles per task (input order) of the last call."""
        c = np.zeros(self.inp.ntasks, np.int64)
        lib().grid_gb300_task_cycles(self.impl, _p(c))
        return c

    def task_features(self) -> np.ndarray:
        """[ntasks][6] cost-model features in input order."""
        f = np.zeros((self.inp.ntasks, 6), np.float32)
        lib().grid_gb300_task_features(self.impl, _p(f))
        return f

    def timings(self):
        t = np.zeros(4)
        lib().grid_gb300_last_timings(self.impl, _p(t))
        return {"coef_ms": t[0], "grid_ms": t[1], "post_ms": t[2], "total_ms": t[3]}

    # ------------------------------------------------------ host buffers
    def _buffers(self):
        if self._grids is None:
            self._pab = Buffer(self.inp.buffer_size)
            self._hab = Buffer(self.inp.buffer_size)
            self._grids = [Buffer(n) for n in self.inp.grid_sizes()]
        return self._pab, self._hab, self._grids

    def host_buffers(self):
        """The pinned offload buffers (pab, hab, grids) the host calls use."""
        return self._buffers()

    def collocate(self, func: int, pab_blocks=None, copy_out: bool = True):
        """grid_collocate_task_list with host buffers.  pab_blocks=None uses the
        current content of the pab offload buffer; returns copies of the grids
        (or None with copy_out=False)."""
        L = lib()
        pab, _, grids = self._buffers()
        if pab_blocks is not None:
            pab.host[:] = pab_blocks
        arr = (C.POINTER(OffloadBuffer) * len(grids))(*[g.ptr for g in grids])
        if self.api == "cp2k":
            L.grid_collocate_task_list(self.h, int(func), self.inp.nlevels, _p(self.npts_local),
                                       pab.ptr, arr)
        else:
            L.grid_gb300_collocate_task_list(self.impl, int(func), self.inp.nlevels, pab.ptr, arr)
        return [g.host.copy() for g in grids] if copy_out else None

    def integrate(self, grids=None, pab_blocks=None, compute_tau=False, forces=False,
                  virial=False, copy_out: bool = True, use_pab: bool = None):
        """grid_integrate_task_list with host buffers; returns (hab, forces, virial).
        grids=None uses the current content of the grid offload buffers."""
        L = lib()
        pab, hab, gb = self._buffers()
        if grids is not None:
            for b, g in zip(gb, grids):
                b.host[:] = g
        if pab_blocks is not None:
            pab.host[:] = pab_blocks
        if use_pab is None:
            use_pab = pab_blocks is not None
        arr = (C.POINTER(OffloadBuffer) * len(gb))(*[b.ptr for b in gb])
        f = np.zeros((self.inp.natoms, 3)) if forces else None
        v = np.zeros((3, 3)) if virial else None
        fp = _p(f) if f is not None else None
        vp_ = _p(v) if v is not None else None
        pp = pab.ptr if use_pab else None
        if self.api == "cp2k":
            L.grid_integrate_task_list(self.h, bool(compute_tau), self.inp.natoms,
                                       self.inp.nlevels, _p(self.npts_local), pp, arr, hab.ptr,
                                       fp, vp_)
        else:
            L.grid_gb300_integrate_task_list(self.impl, bool(compute_tau), self.inp.nlevels, pp,
                                             arr, hab.ptr, fp, vp_)
        return (hab.host.copy() if copy_out else None), f, v

    # ---------------------------------------------------- device buffers
    def collocate_device(self, func: int, pab_dev, grids_dev, stream=None):
        """Enqueue collocation on device tensors (torch, float64, contiguous)."""
        ptrs = (C.c_void_p * len(grids_dev))(*[g.data_ptr() for g in grids_dev])
        lib().grid_gb300_collocate_device_async(self.impl, int(func), C.c_void_p(pab_dev.data_ptr()),
                                                C.cast(ptrs, C.c_void_p), _stream(stream))

    def integrate_device(self, grids_dev, hab_dev, pab_dev=None, forces_dev=None,
                         virial_dev=None, compute_tau=False, stream=None):
        ptrs = (C.c_void_p * len(grids_dev))(*[g.data_ptr() for g in grids_dev])
        dp = lambda x: C.c_void_p(x.data_ptr()) if x is not None else None
        lib().grid_gb300_integrate_device_async(
            self.impl, bool(compute_tau), dp(pab_dev), C.cast(ptrs, C.c_void_p), dp(hab_dev),
            dp(forces_dev), dp(virial_dev), _stream(stream))

    def autotune(self, func: int, pab_dev, rho_dev, V_dev, hab_dev, stream=None) -> float:
        """Measures and keeps the fastest size split and launch shapes for the
        current precision (grid_gb300_autotune); returns grid-kernel ms."""
        rp = (C.c_void_p * len(rho_dev))(*[g.data_ptr() for g in rho_dev])
        vp_ = (C.c_void_p * len(V_dev))(*[g.data_ptr() for g in V_dev])
        return float(lib().grid_gb300_autotune(self.impl, int(func), C.c_void_p(pab_dev.data_ptr()),
                                               C.cast(rp, C.c_void_p), C.cast(vp_, C.c_void_p),
                                               C.c_void_p(hab_dev.data_ptr()), _stream(stream)))

    def set_collocate_variant(self, variant: int):
        """0: row walk, 1: point list, -1: by arithmetic
        (grid_gb300_set_collocate_variant)."""
        lib().grid_gb300_set_collocate_variant(self.impl, int(variant))

    def set_transform_variant(self, variant: int):
        """C_ab <-> C_xyz transform: 0 direct, 1 staged, -1 staged in the
        coefficient kernel only
        (grid_gb300_set_transform_variant)."""
        lib().grid_gb300_set_transform_variant(self.impl, int(variant))

    def set_tensor_integrate(self, enable: bool):
        """FP32-class orthorhombic integration on the tensor cores
        (grid_gb300_set_tensor_integrate)."""
        lib().grid_gb300_set_tensor_integrate(self.impl, int(bool(enable)))

    def set_tensor_collocate(self, enable: bool):
        """FP32-class orthorhombic collocation on the tensor cores
        (grid_gb300_set_tensor_collocate)."""
        lib().grid_gb300_set_tensor_collocate(self.impl, int(bool(enable)))

    def set_row_split(self, enable: bool):
        """Mixed mode: run the outer rows of orthorhombic double-float tasks
        in FP32 (grid_gb300_set_row_split)."""
        lib().grid_gb300_set_row_split(self.impl, int(bool(enable)))

    def row_split_stats(self):
        """(share of tasks split, share of grid points in FP32) of a density
        collocation in the mixed mode (grid_gb300_row_split_stats)."""
        a, b = C.c_double(), C.c_double()
        lib().grid_gb300_row_split_stats(self.impl, C.byref(a), C.byref(b))
        return a.value, b.value

    def set_queue_streams(self, n: int):
        """Streams the grid launches of a phase alternate over (1 or 2;
        grid_gb300_set_queue_streams)."""
        lib().grid_gb300_set_queue_streams(self.impl, int(n))

    def set_copy_chunks(self, chunks: int):
        """Pieces of the pab / hab copies of the host-buffer calls
        (grid_gb300_set_copy_chunks)."""
        lib().grid_gb300_set_copy_chunks(self.impl, int(chunks))

    def set_model_bin_width(self, width: float):
        lib().grid_gb300_set_model_bin_width(self.impl, float(width))

    def tuned_split(self) -> int:
        return int(lib().grid_gb300_tuned_split(self.impl))

    def capture_step(self, func: int, pab_dev, rho_dev, V_dev, hab_dev, forces_dev=None,
                     virial_dev=None, compute_tau=False, stream=None):
        """CUDA graph of one SCF step (collocate func into rho_dev, integrate
        V_dev into hab_dev) on device tensors; `stream` must be a created
        torch.cuda.Stream.  Returns a StepGraph."""
        rp = (C.c_void_p * len(rho_dev))(*[g.data_ptr() for g in rho_dev])
        vp_ = (C.c_void_p * len(V_dev))(*[g.data_ptr() for g in V_dev])
        dp = lambda x: C.c_void_p(x.data_ptr()) if x is not None else None
        h = lib().grid_gb300_capture_step(self.impl, int(func), dp(pab_dev), C.cast(rp, C.c_void_p),
                                          bool(compute_tau), C.cast(vp_, C.c_void_p), dp(hab_dev),
                                          dp(forces_dev), dp(virial_dev), _stream(stream))
        return StepGraph(h, (rp, vp_, pab_dev, rho_dev, V_dev, hab_dev, forces_dev, virial_dev))

    def close(self):
        if self.h:
            fn = lib().grid_free_task_list if self.api == "cp2k" else lib().grid_gb300_free_task_list
            fn(self.h)
            self.h = C.c_void_p()
        for b in (self._pab, self._hab):
            if b is not None:
                b.free()
        for g in self._grids or []:
            g.free()
        self._grids = None
        for b in self.basis:
            b.free()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class StepGraph:
    """A captured SCF step (grid_gb300_capture_step); keeps the buffers it
    was captured on alive."""

    def __init__(self, handle, keep):
        self.h = C.c_void_p(handle)
        self._keep = keep

    @property
    def kernels(self) -> int:
        return int(lib().grid_gb300_step_graph_kernels(self.h))

    def launch(self, stream=None):
        lib().grid_gb300_step_graph_launch(self.h, _stream(stream))

    def wait(self, stream=None):
        lib().grid_gb300_step_graph_wait(self.h, _stream(stream))

    def free(self):
        if self.h:
            lib().grid_gb300_step_graph_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def collocate_pgf_product_static(t: dict, pab_dev, grid_dev, stream=None) -> int:
    """grid_gb300_collocate_pgf_product_static for a task description dict
    (keys as a CP2K .task file); pab_dev / grid_dev are torch CUDA float64
    tensors.  Returns the entry point's status (0 = ok)."""
    f64 = lambda x: np.ascontiguousarray(x, np.float64)
    i32 = lambda x: np.ascontiguousarray(x, np.int32)
    arrs = [f64(t["dh"]), f64(t["dh_inv"]), f64(t["ra"]), f64(t["rab"]), i32(t["npts_global"]),
            i32(t["npts_local"]), i32(t["shift_local"]), i32(t["border_width"])]
    return int(lib().grid_gb300_collocate_pgf_product_static(
        bool(t["orthorhombic"]), int(t["border_mask"]), int(t["func"]), t["la_max"], t["la_min"],
        t["lb_max"], t["lb_min"], t["zeta"], t["zetb"], t["rscale"], *[_p(a) for a in arrs],
        t["radius"], t["o1"], t["o2"], t["n1"], t["n2"], C.c_void_p(pab_dev.data_ptr()),
        C.c_void_p(grid_dev.data_ptr()), _stream(stream)))


def _stream(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


def _bind_taskgen(L):
    if hasattr(L, "_tg_bound"):
        return
    vp = C.c_void_p
    L.grid_gb300_taskgen_create.argtypes = ([C.c_int, C.c_int] + [vp] * 5 + [C.c_int, vp, vp, vp]
                                            + [C.c_double, C.c_double, C.c_int, vp, C.c_double,
                                               C.POINTER(vp)])
    L.grid_gb300_taskgen_free.argtypes = [vp]
    L.grid_gb300_taskgen_set_radius_screen.argtypes = [vp, vp, vp, vp]
    L.grid_gb300_taskgen_run.argtypes = [vp, vp, C.c_int, vp, vp, vp, vp]
    L.grid_gb300_taskgen_arrays.argtypes = [vp] + [vp] * 12
    L.grid_gb300_taskgen_copy.argtypes = [vp] + [vp] * 12
    L.grid_gb300_taskgen_create_task_list.argtypes = [vp, C.c_bool, C.c_int] + [vp] * 8
    L.grid_gb300_pack_blocks.argtypes = [C.c_longlong] + [vp] * 6
    L.grid_gb300_unpack_blocks.argtypes = [C.c_longlong] + [vp] * 6
    L.grid_gb300_find_blocks.restype = C.c_longlong
    L.grid_gb300_find_blocks.argtypes = [C.c_longlong, vp, vp, vp, C.c_longlong, vp, vp, vp, vp]
    L._tg_bound = True


_TASK_INT_FIELDS = ["level_list", "iatom_list", "jatom_list", "iset_list", "jset_list",
                    "ipgf_list", "jpgf_list", "border_mask_list", "block_num_list"]


class TaskGenerator:
    """Task-list generation on the device (grid_gb300_taskgen_*): the work of
    Quickstep's generate_qs_task_list (src/task_list_methods.F:117-501) for
    a geometry, with the basis and screening of ``like`` (a TaskListInputs
    from cp2k_gb300.workload, whose ``meta`` holds the cell, level cutoffs,
    rel_cutoff, eps, image range and pair cut)."""

    def __init__(self, like: TaskListInputs):
        L = lib()
        _bind_taskgen(L)
        m = like.meta
        self.like = like
        bs = like.basis_sets
        self.maxpgf = max(int(b.maxpgf) for b in bs)
        nset = np.array([b.nset for b in bs], np.int32)
        nsgf = np.array([b.nsgf for b in bs], np.int32)
        lmax = np.concatenate([np.asarray(b.lmax, np.int32) for b in bs]).astype(np.int32)
        npgf = np.concatenate([np.asarray(b.npgf, np.int32) for b in bs]).astype(np.int32)
        zet = np.zeros((int(nset.sum()), self.maxpgf))
        r = 0
        for b in bs:
            z = np.asarray(b.zet, np.float64).reshape(b.nset, -1)
            zet[r:r + b.nset, :z.shape[1]] = z
            r += b.nset
        kinds = np.ascontiguousarray(like.atom_kinds, np.int32)
        cell = np.ascontiguousarray(np.asarray(m["cell_bohr"], np.float64).reshape(3, 3))
        nimg = np.ascontiguousarray(m["nimg"], np.int32)
        cut = np.ascontiguousarray(m["cutoffs_ry"], np.float64)
        self._keep = [kinds, nset, nsgf, lmax, npgf, zet, cell, nimg, cut]
        self.h = C.c_void_p()
        L.grid_gb300_taskgen_create(like.natoms, len(bs), _p(kinds), _p(nset), _p(nsgf),
                                    _p(lmax), _p(npgf), self.maxpgf, _p(zet), _p(cell),
                                    _p(nimg), float(m["rmax"]), float(m["eps"]),
                                    len(cut), _p(cut), float(m["rel_cutoff"]),
                                    C.byref(self.h))
        if m.get("screen") == "radius":  # Quickstep's screening by basis radii
            rp = np.zeros((int(nset.sum()), self.maxpgf))
            src = np.asarray(m["rpgf"], np.float64)
            rp[:, :src.shape[1]] = src
            sr = np.ascontiguousarray(m["set_radius"], np.float64)
            kr = np.ascontiguousarray(m["kind_radius"], np.float64)
            self._keep += [rp, sr, kr]
            L.grid_gb300_taskgen_set_radius_screen(self.h, _p(rp), _p(sr), _p(kr))
        self.ntasks = self.nblocks = self.buffer_size = 0
        self.positions = None

    def run(self, positions, stream=None):
        """Generate for ``positions`` ([natoms][3] bohr: numpy, or a torch
        CUDA float64 tensor); returns (ntasks, nblocks, buffer_size)."""
        nt, nb, bsz = C.c_int(), C.c_int(), C.c_longlong()
        if hasattr(positions, "data_ptr"):
            self.positions = None
            lib().grid_gb300_taskgen_run(self.h, C.c_void_p(positions.data_ptr()), 1,
                                         _stream(stream), C.byref(nt), C.byref(nb),
                                         C.byref(bsz))
        else:
            pos = np.ascontiguousarray(positions, np.float64).reshape(-1, 3)
            self.positions = pos
            lib().grid_gb300_taskgen_run(self.h, _p(pos), 0, _stream(stream), C.byref(nt),
                                         C.byref(nb), C.byref(bsz))
        self.ntasks, self.nblocks, self.buffer_size = nt.value, nb.value, bsz.value
        return self.ntasks, self.nblocks, self.buffer_size

    def device_arrays(self) -> dict:
        """Device addresses of the last run's arrays."""
        ptrs = [C.c_void_p() for _ in range(12)]
        lib().grid_gb300_taskgen_arrays(self.h, *[C.byref(x) for x in ptrs])
        names = _TASK_INT_FIELDS + ["radius_list", "rab_list", "block_offsets"]
        return {k: v.value for k, v in zip(names, ptrs)}

    def host_arrays(self) -> dict:
        nt, nb = self.ntasks, self.nblocks
        out = {k: np.zeros(nt, np.int32) for k in _TASK_INT_FIELDS}
        out["radius_list"] = np.zeros(nt)
        out["rab_list"] = np.zeros((nt, 3))
        out["block_offsets"] = np.zeros(nb, np.int32)
        lib().grid_gb300_taskgen_copy(self.h, *[_p(out[k]) for k in _TASK_INT_FIELDS],
                                      _p(out["radius_list"]), _p(out["rab_list"]),
                                      _p(out["block_offsets"]))
        return out

    def inputs(self, positions=None) -> TaskListInputs:
        """``like`` with the last run's task arrays (and ``positions``)."""
        import dataclasses
        a = self.host_arrays()
        pos = self.positions if positions is None else positions
        if pos is None:
            raise ValueError("positions of a device run must be given")
        return dataclasses.replace(self.like, nblocks=self.nblocks,
                                   buffer_size=self.buffer_size,
                                   atom_positions=np.asarray(pos, np.float64).reshape(-1, 3),
                                   **a)

    def free(self):
        if self.h:
            lib().grid_gb300_taskgen_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def pack_blocks(src_offsets, dst_offsets, sizes, src, dst, stream=None):
    """rs_pack_buffer on torch CUDA tensors: dst[dst_off[b]:+sizes[b]] =
    src[src_off[b]:+sizes[b]] (src_offsets int64, dst_offsets / sizes int32)."""
    L = lib()
    _bind_taskgen(L)
    d = lambda t: C.c_void_p(t.data_ptr())
    L.grid_gb300_pack_blocks(int(sizes.numel()), d(src_offsets), d(dst_offsets), d(sizes),
                             d(src), d(dst), _stream(stream))


def unpack_blocks(buffer_offsets, block_offsets, sizes, buffer, blocks, stream=None):
    """rs_unpack_buffer on torch CUDA tensors: blocks[block_off[b]:+sizes[b]]
    += buffer[buffer_off[b]:+sizes[b]] (buffer_offsets / sizes int32,
    block_offsets int64)."""
    L = lib()
    _bind_taskgen(L)
    d = lambda t: C.c_void_p(t.data_ptr())
    L.grid_gb300_unpack_blocks(int(sizes.numel()), d(buffer_offsets), d(block_offsets),
                               d(sizes), d(buffer), d(blocks), _stream(stream))


def find_blocks(key_rows, key_cols, key_offsets, rows, cols, offsets, stream=None) -> int:
    """Block look-up by (row, col) in keys sorted by row then column (torch
    CUDA tensors; offsets int64, -1 where absent); returns the misses."""
    L = lib()
    _bind_taskgen(L)
    d = lambda t: C.c_void_p(t.data_ptr())
    return int(L.grid_gb300_find_blocks(int(key_rows.numel()), d(key_rows), d(key_cols),
                                        d(key_offsets), int(rows.numel()), d(rows), d(cols),
                                        d(offsets), _stream(stream)))


class PwTransfer:
    """Device-resident transfer of the level grids to the plane-wave grid and
    back (grid_gb300_pw_*): density_rs2pw / potential_pw2rs of CP2K's
    src/pw_env/rs_pw_interface.F on torch CUDA float64 tensors."""

    def __init__(self, npts):
        L = lib()
        if not hasattr(L, "_pw_bound"):
            L.grid_gb300_pw_create.argtypes = [C.c_int, vp, C.POINTER(vp)]
            L.grid_gb300_pw_free.argtypes = [vp]
            L.grid_gb300_pw_density_rs2pw.argtypes = [vp, vp, vp, vp, vp]
            L.grid_gb300_pw_potential_pw2rs.argtypes = [vp, vp, vp, vp]
            L.grid_gb300_pw_poisson.argtypes = [vp, vp, vp, vp, vp, vp, vp]
            L.grid_gb300_pw_potential_g2rs.argtypes = [vp, vp, vp, vp]
            L._pw_bound = True
        self.npts = [tuple(int(x) for x in n) for n in npts]
        arr = np.ascontiguousarray(np.array(self.npts, np.int32).ravel())
        self.h = C.c_void_p()
        L.grid_gb300_pw_create(len(self.npts), _p(arr), C.byref(self.h))

    def density_rs2pw(self, rs_grids, rho=None, rho_gspace=None, stream=None):
        ptrs = (C.c_void_p * len(rs_grids))(*[g.data_ptr() for g in rs_grids])
        dp = lambda x: C.c_void_p(x.data_ptr()) if x is not None else None
        lib().grid_gb300_pw_density_rs2pw(self.h, C.cast(ptrs, C.c_void_p), dp(rho),
                                          dp(rho_gspace), _stream(stream))

    def potential_pw2rs(self, v_rspace, rs_grids, stream=None):
        ptrs = (C.c_void_p * len(rs_grids))(*[g.data_ptr() for g in rs_grids])
        lib().grid_gb300_pw_potential_pw2rs(self.h, C.c_void_p(v_rspace.data_ptr()),
                                            C.cast(ptrs, C.c_void_p), _stream(stream))

    def potential_g2rs(self, v_gspace, rs_grids, stream=None):
        """The level grids from the finest grid's G-space coefficients
        (grid_gb300_pw_potential_g2rs)."""
        ptrs = (C.c_void_p * len(rs_grids))(*[g.data_ptr() for g in rs_grids])
        lib().grid_gb300_pw_potential_g2rs(self.h, C.c_void_p(v_gspace.data_ptr()),
                                           C.cast(ptrs, C.c_void_p), _stream(stream))

    def poisson(self, dh, rho_gspace, v_gspace, v_rspace=None, energy=False, stream=None):
        """Periodic Hartree solve in G space (grid_gb300_pw_poisson), with v in
        real space when a tensor is given; returns the Hartree energy when
        asked for (synchronising)."""
        dh = np.ascontiguousarray(dh, np.float64).reshape(9)
        e = C.c_double(0.0)
        lib().grid_gb300_pw_poisson(
            self.h, _p(dh), C.c_void_p(rho_gspace.data_ptr()), C.c_void_p(v_gspace.data_ptr()),
            C.c_void_p(v_rspace.data_ptr()) if v_rspace is not None else None,
            C.byref(e) if energy else None, _stream(stream))
        return e.value if energy else None

    def close(self):
        if self.h:
            lib().grid_gb300_pw_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _pgf_bind(L):
    if hasattr(L, "_pgf_bound"):
        return
    L.grid_cpu_collocate_pgf_product.argtypes = (
        [C.c_bool, C.c_int, C.c_int] + [C.c_int] * 4 + [C.c_double] * 3 + [vp] * 8
        + [C.c_double] + [C.c_int] * 4 + [vp, vp])
    L.grid_cpu_integrate_pgf_product.argtypes = (
        [C.c_bool, C.c_bool, C.c_int] + [C.c_int] * 4 + [C.c_double] * 2 + [vp] * 8
        + [C.c_double] + [C.c_int] * 4 + [vp] * 8)
    L._pgf_bound = True


def _task_arrays(t):
    f64 = lambda x: np.ascontiguousarray(x, np.float64)
    i32 = lambda x: np.ascontiguousarray(x, np.int32)
    return [f64(t["dh"]), f64(t["dh_inv"]), f64(t["ra"]), f64(t["rab"]), i32(t["npts_global"]),
            i32(t["npts_local"]), i32(t["shift_local"]), i32(t["border_width"])]


def collocate_pgf_product(t: dict, grid: np.ndarray = None) -> np.ndarray:
    """grid_cpu_collocate_pgf_product (CP2K's single-task collocate, run on the
    GPU) for a task description dict (keys as a CP2K .task file); the values
    are added into `grid` (zeros if not given), which is returned."""
    L = lib()
    _pgf_bind(L)
    nl = t["npts_local"]
    if grid is None:
        grid = np.zeros(int(nl[0] * nl[1] * nl[2]))
    grid = np.ascontiguousarray(grid, np.float64)
    arrs = _task_arrays(t)
    pab = np.ascontiguousarray(t["pab"], np.float64)
    L.grid_cpu_collocate_pgf_product(
        bool(t["orthorhombic"]), int(t["border_mask"]), int(t["func"]), t["la_max"], t["la_min"],
        t["lb_max"], t["lb_min"], t["zeta"], t["zetb"], t["rscale"], *[_p(a) for a in arrs],
        t["radius"], t["o1"], t["o2"], t["n1"], t["n2"], _p(pab), _p(grid))
    return grid


def integrate_pgf_product(t: dict, grid: np.ndarray, compute_tau: bool, forces: bool = True,
                          virial: bool = True, derivatives: bool = False):
    """grid_cpu_integrate_pgf_product (CP2K's single-task integrate, run on the
    GPU); returns (hab, forces[2][3], virials[2][3][3]) and, with
    derivatives, also (hdab, hadb, a_hdab)."""
    L = lib()
    _pgf_bind(L)
    hab = np.zeros((t["n2"], t["n1"]))
    f = np.zeros((2, 3)) if forces else None
    v = np.zeros((2, 3, 3)) if virial else None
    hd = np.zeros((t["n2"], t["n1"], 3)) if derivatives else None
    ha = np.zeros((t["n2"], t["n1"], 3)) if derivatives else None
    ahd = np.zeros((t["n2"], t["n1"], 3, 3)) if derivatives else None
    pab = np.ascontiguousarray(t["pab"], np.float64) if (forces or virial) else None
    g = np.ascontiguousarray(grid, np.float64)
    arrs = _task_arrays(t)
    pp = lambda a: _p(a) if a is not None else None
    L.grid_cpu_integrate_pgf_product(
        bool(t["orthorhombic"]), bool(compute_tau), int(t["border_mask"]), t["la_max"],
        t["la_min"], t["lb_max"], t["lb_min"], t["zeta"], t["zetb"], *[_p(a) for a in arrs],
        t["radius"], t["o1"], t["o2"], t["n1"], t["n2"], _p(g), _p(hab), pp(pab), pp(f), pp(v),
        pp(hd), pp(ha), pp(ahd))
    if derivatives:
        return hab, f, v, hd, ha, ahd
    return hab, f, v
