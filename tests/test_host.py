"""CPU-only checks of the host side: the C-ABI library exports exactly what
include/grid_gb300.h declares, the product path fails loudly without its
CUDA library or a GPU, the seeded workload generator is deterministic and
consistent, and the multi-process bench helpers work over gloo."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "grid_gb300.h")


def _declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    src = re.sub(r"^\s*#[^\n]*", "", src, flags=re.M)
    names = set()
    # top-level declarations "<type> name(" ending in ");"
    for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}]*)\)\s*;", src):
        name = m.group(1)
        if name not in ("sizeof", "if", "while", "return"):
            names.add(name)
    return names


@pytest.fixture(scope="module")
def grid_lib():
    from cp2k_gb300 import build
    if not os.path.exists(build.GRID_LIB):
        build.build_all()
    return build.GRID_LIB


def test_header_declares_the_cp2k_surface():
    d = _declared()
    # the entry points CP2K's Fortran binds (src/grid/grid_api.F:
    # grid_create_task_list, grid_collocate_task_list, grid_integrate_task_list,
    # grid_free_task_list, grid_create_basis_set, grid_free_basis_set,
    # grid_library_*) and the offload buffer (src/offload/offload_buffer.h)
    for name in ("grid_create_task_list", "grid_free_task_list", "grid_collocate_task_list",
                 "grid_integrate_task_list", "grid_create_basis_set", "grid_free_basis_set",
                 "grid_library_init", "grid_library_finalize", "grid_library_set_config",
                 "grid_library_get_config", "grid_library_print_stats",
                 "grid_library_counter_add", "offload_create_buffer", "offload_free_buffer",
                 "offload_get_buffer_host_pointer"):
        assert name in d, name


def test_struct_layouts_match_ctypes(tmp_path):
    """The ctypes mirrors of the header's structs (offload_buffer,
    grid_gb300_launch_info) have the C compiler's size and field offsets."""
    import ctypes as C
    from cp2k_gb300 import grid as G
    structs = {"offload_buffer": G.OffloadBuffer, "grid_gb300_launch_info": G.LaunchInfo}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "grid_gb300.h"',
             'int main(void) {']
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    seen = {}
    for line in out.splitlines():
        cname, field, value = line.split()
        seen[(cname, field)] = int(value)
    for cname, py in structs.items():
        assert seen[(cname, "sizeof")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert seen[(cname, f)] == getattr(py, f).offset, (cname, f)


@pytest.mark.parametrize("name,scale", [("c2_512atoms", 0.3), ("c3_256atoms_triclinic", 0.5)])
def test_host_preparation_independent_of_threads(grid_lib, name, scale, monkeypatch):
    """The host-side task-list preparation runs on several threads: its
    arrays (hashed by grid_gb300_host_digest, no GPU needed) are the same
    with one thread as with eight, and the class split is non-trivial."""
    from cp2k_gb300 import grid as G
    from cp2k_gb300 import workload as W
    inp = W.config(name, scale=scale, seed=3)
    assert inp.ntasks > 4096  # large enough for the threaded path
    monkeypatch.setenv("GRID_GB300_HOST_THREADS", "1")
    one = G.host_digest(inp)
    monkeypatch.setenv("GRID_GB300_HOST_THREADS", "8")
    eight = G.host_digest(inp)
    assert np.array_equal(one, eight)
    assert one[10] > 0                     # Cartesian scratch
    assert 0 < one[11] < inp.ntasks        # FP32-class tasks at the default bound


def test_library_exports_every_declared_symbol(grid_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", grid_lib], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.split()}
    declared = _declared()
    missing = declared - exported
    assert not missing, missing
    # every unmangled export is part of the declared interface
    extra = {s for s in exported if not s.startswith("_Z") and not s.startswith("_")} - declared
    assert not extra, extra


def test_library_loads_and_resolves_through_ctypes(grid_lib):
    import ctypes
    L = ctypes.CDLL(grid_lib)
    for name in _declared():
        assert getattr(L, name) is not None
    # pure host queries: no device work
    L.grid_gb300_static_scratch_bytes.restype = ctypes.c_size_t
    assert L.grid_gb300_static_scratch_bytes() == 256 * 1024
    L.grid_gb300_kernel_launches.restype = ctypes.c_longlong
    assert L.grid_gb300_kernel_launches() == 0


def test_missing_library_raises(monkeypatch, tmp_path):
    from cp2k_gb300 import grid
    monkeypatch.setattr(grid, "_LIB", None)
    monkeypatch.setattr(grid, "lib_path", lambda: str(tmp_path / "absent.so"))
    with pytest.raises(RuntimeError, match="missing"):
        grid.lib()


@pytest.mark.skipif(os.environ.get("CUDA_VISIBLE_DEVICES") is None and
                    os.path.exists("/dev/nvidia0"), reason="a GPU is present")
def test_no_gpu_fails_loudly(grid_lib):
    """Without a usable device the task-list constructor stops the process with
    a CUDA error message instead of falling back to any CPU path."""
    code = ("from cp2k_gb300 import workload as W, grid\n"
            "inp = W.config('c1_64atoms', scale=0.1, seed=3)\n"
            "grid.GridTaskList(inp)\n"
            "print('RETURNED')\n")
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode != 0
    assert "RETURNED" not in r.stdout
    assert "CUDA" in r.stderr or "cuda" in r.stderr


def test_generator_deterministic_and_consistent():
    from cp2k_gb300 import workload as W
    a = W.config("c1_64atoms", scale=0.2, seed=5)
    b = W.config("c1_64atoms", scale=0.2, seed=5)
    c = W.config("c1_64atoms", scale=0.2, seed=6)
    for k in ("atom_positions", "iatom_list", "jatom_list", "level_list", "radius_list",
              "rab_list", "block_offsets"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert not np.array_equal(a.atom_positions, c.atom_positions)
    n = a.ntasks
    assert n > 0
    assert np.all(a.radius_list > 0)
    assert np.all((a.level_list >= 1) & (a.level_list <= a.nlevels))
    # blocks are contiguous runs (CP2K's task lists are sorted by block,
    # src/grid/grid_task_list.c:82-118)
    blk = a.block_num_list
    assert np.all(np.diff(blk) >= 0)
    # rab = r_j - r_i up to a lattice vector; cell vector i = dh[i] * npts[i]
    pos = a.atom_positions.reshape(-1, 3)
    d = pos[a.jatom_list - 1] - pos[a.iatom_list - 1]
    dh = a.dh.reshape(-1, 3, 3)[0]
    npts = a.npts_global.reshape(-1, 3)[0]
    cell = dh * npts[:, None]
    frac = (a.rab_list.reshape(-1, 3) - d) @ np.linalg.inv(cell)
    assert np.allclose(frac, np.round(frac), atol=1e-9)
    # buffer holds every block
    sizes = [a.basis_sets[a.atom_kinds[i - 1] - 1].nsgf * a.basis_sets[a.atom_kinds[j - 1] - 1].nsgf
             for i, j in zip(a.iatom_list, a.jatom_list)]
    assert a.buffer_size >= max(o + s for o, s in zip(a.block_offsets[blk - 1], sizes))
    # density blocks: the diagonal ones are symmetric
    pab = W.density_blocks(a, seed=1)
    assert pab.shape == (a.buffer_size,)
    assert np.array_equal(pab, W.density_blocks(a, seed=1))


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    m = bench.max_over_ranks(10.0 + r, w)
    q.put((r, w, m))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_bench_ranks_over_gloo():
    """bench.py's replica path: each rank measures its own copy of the workload
    and rank 0 reports the slowest (max over ranks)."""
    import socket

    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 11.0), (1, 2, 11.0)]


def test_bench_reference_arm_replicas_exit_quietly():
    """Ranks other than 0 of the reference arm do no work."""
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup, gpus = 1, 1, 2
    assert bench.reference_arm(A, 2, 1) is None
