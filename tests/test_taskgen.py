"""Task-list generation on the device (grid_gb300_taskgen_*, the work of
CP2K's generate_qs_task_list, src/task_list_methods.F:117-501) against the
host generator (cp2k_gb300/csrc/workload.c, the same screening, radius and
level rules in C) on the same basis and positions: every array equal,
element for element (integer fields and the radii, which come out of the
same bisection); and the device block packing (rs_pack_buffer /
rs_unpack_buffer, :2593-2674) against numpy gathers, bit for bit."""
import numpy as np
import pytest

from cp2k_gb300 import workload as W

FIELDS = ["level_list", "iatom_list", "jatom_list", "iset_list", "jset_list", "ipgf_list",
          "jpgf_list", "border_mask_list", "block_num_list", "radius_list", "rab_list",
          "block_offsets"]


def _same_lists(host, arrays, nblocks, buffer_size):
    assert arrays["level_list"].shape[0] == host.ntasks
    assert nblocks == host.nblocks
    assert buffer_size == host.buffer_size
    for k in FIELDS:
        a = np.asarray(getattr(host, k)).reshape(arrays[k].shape)
        bad = np.flatnonzero((a != arrays[k]).reshape(len(a), -1).any(axis=1))
        assert bad.size == 0, (k, bad[:5], a[bad[:5]], arrays[k][bad[:5]])


def test_host_radius_screen_rules():
    """CPU: the host generator's radius screening keeps exactly the
    primitive pairs whose radii reach |rab| (Quickstep's four tests), and
    its radii are exp_radius maxima over the set's shells."""
    inp = W.config("c1_64atoms", scale=0.4, seed=3, screen="radius")
    m = inp.meta
    rp, sr, kr = m["rpgf"], m["set_radius"], m["kind_radius"]
    off = np.concatenate([[0], np.cumsum([b.nset for b in inp.basis_sets])])
    assert np.allclose(sr, rp.max(axis=1)) and np.all(sr > 0)
    for k in range(len(kr)):
        assert kr[k] == sr[off[k]:off[k + 1]].max()
    dab = np.linalg.norm(inp.rab_list, axis=1)
    gi = off[inp.atom_kinds[inp.iatom_list - 1] - 1] + inp.iset_list - 1
    gj = off[inp.atom_kinds[inp.jatom_list - 1] - 1] + inp.jset_list - 1
    assert np.all(rp[gi, inp.ipgf_list - 1] + rp[gj, inp.jpgf_list - 1] >= dab)
    assert np.all(sr[gi] + sr[gj] >= dab)


def test_host_retask_reproduces_and_moves():
    """CPU: re-tasking the host generator at its own positions gives the same
    arrays; moved atoms give another list of the same kind."""
    a = W.config("c1_64atoms", scale=0.3, seed=4)
    b = W.config("c1_64atoms", scale=0.3, seed=4, positions=a.atom_positions)
    for k in FIELDS:
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    rng = np.random.default_rng(1)
    moved = a.atom_positions + rng.normal(scale=0.4, size=a.atom_positions.shape)
    c = W.config("c1_64atoms", scale=0.3, seed=4, positions=moved)
    assert np.array_equal(c.atom_positions, moved)
    assert c.ntasks > 0
    assert not (c.ntasks == a.ntasks and np.array_equal(c.rab_list, a.rab_list))
    assert a.meta["nimg"] == c.meta["nimg"] and a.meta["rmax"] == c.meta["rmax"]


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale", [("c1_64atoms", 1.0), ("c3_256atoms_triclinic", 1.0),
                                        ("c2_512atoms", 1.0)])
def test_taskgen_matches_host(name, scale):
    from cp2k_gb300 import grid as G
    host = W.config(name, scale=scale)
    gen = G.TaskGenerator(host)
    nt, nb, bs = gen.run(host.atom_positions)
    assert nt == host.ntasks
    _same_lists(host, gen.host_arrays(), nb, bs)
    gen.free()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1_64atoms", "c3_256atoms_triclinic", "c2_512atoms"])
def test_taskgen_radius_screen_matches_host(name):
    """Quickstep's screening by the basis radii (task_list_methods.F:
    673-696) on the device against the host generator's."""
    from cp2k_gb300 import grid as G
    host = W.config(name, screen="radius")
    gen = G.TaskGenerator(host)
    nt, nb, bs = gen.run(host.atom_positions)
    assert nt == host.ntasks
    _same_lists(host, gen.host_arrays(), nb, bs)
    gen.free()


@pytest.mark.gpu
def test_taskgen_moved_geometry_and_device_positions():
    """Three geometries through one generator (an MD trajectory), positions
    from the host and from device memory."""
    import torch
    from cp2k_gb300 import grid as G
    base = W.config("c1_64atoms", seed=2)
    gen = G.TaskGenerator(base)
    rng = np.random.default_rng(7)
    pos = base.atom_positions.copy()
    for step in range(3):
        host = W.config("c1_64atoms", seed=2, positions=pos)
        if step == 1:
            nt, nb, bs = gen.run(torch.tensor(pos, device="cuda"))
        else:
            nt, nb, bs = gen.run(pos)
        _same_lists(host, gen.host_arrays(), nb, bs)
        # atoms may leave the cell: images are found all the same
        pos = pos + rng.normal(scale=0.5, size=pos.shape)
    gen.free()


@pytest.mark.gpu
def test_task_list_from_generator_collocates_like_host_list():
    """grid_gb300_taskgen_create_task_list: the task list made from the
    device arrays collocates like the one made from the host generator's
    arrays (to 1e-12), also when re-created in place at moved positions."""
    from cp2k_gb300 import grid as G
    base = W.config("c1_64atoms", scale=0.5, seed=3)
    gen = G.TaskGenerator(base)
    rng = np.random.default_rng(11)
    tl = None
    pos = base.atom_positions.copy()
    for step in range(2):
        host = W.config("c1_64atoms", scale=0.5, seed=3, positions=pos)
        gen.run(pos)
        tl = G.GridTaskList.from_generator(gen, precision=G.FP64, existing=tl)
        ref = G.GridTaskList(host, precision=G.FP64)
        pab = W.density_blocks(host, seed=5)
        a = tl.collocate(G.GRID_FUNC_AB, pab)
        b = ref.collocate(G.GRID_FUNC_AB, pab)
        # the grids accumulate through FP64 atomics: equal up to the order of
        # the additions
        for x, y in zip(a, b):
            assert np.abs(x - y).max() <= 1e-12 * max(1.0, np.abs(y).max())
        ref.close()
        pos = pos + rng.normal(scale=0.3, size=pos.shape)
    tl.close()
    gen.free()


def _block_store(inp, rng):
    """A block store in the manner of a sparse matrix library: the task
    list's blocks (row = iatom, col = jatom) at shuffled places in one
    arena, with a key table sorted by (row, col)."""
    blk = inp.block_num_list - 1
    first = np.unique(blk, return_index=True)[1]
    rows = inp.iatom_list[first].astype(np.int32)
    cols = inp.jatom_list[first].astype(np.int32)
    nsgf = np.array([inp.basis_sets[k - 1].nsgf for k in inp.atom_kinds])
    sizes = (nsgf[rows - 1] * nsgf[cols - 1]).astype(np.int32)
    perm = rng.permutation(len(rows))
    arena_off = np.zeros(len(rows), np.int64)
    arena_off[perm] = np.concatenate([[0], np.cumsum(sizes[perm])[:-1]]) + 3 * np.arange(len(rows))
    arena = rng.uniform(-1, 1, size=int(arena_off.max() + sizes.max() + 8))
    order = np.lexsort((cols, rows))
    return rows, cols, sizes, arena, arena_off, order


@pytest.mark.gpu
def test_pack_unpack_blocks():
    import torch
    from cp2k_gb300 import grid as G
    inp = W.config("c2_512atoms", scale=0.25)
    rng = np.random.default_rng(4)
    rows, cols, sizes, arena, arena_off, order = _block_store(inp, rng)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device=dev)
    # look the blocks up (dbcsr_get_block_p), plus two absent keys
    q_rows = np.concatenate([rows, [rows[0], 10 ** 6]]).astype(np.int32)
    q_cols = np.concatenate([cols, [10 ** 6, 1]]).astype(np.int32)
    off = torch.empty(len(q_rows), dtype=torch.int64, device=dev)
    miss = G.find_blocks(t(rows[order]), t(cols[order]), t(arena_off[order]), t(q_rows),
                         t(q_cols), off)
    assert miss == 2
    off = off.cpu().numpy()
    assert np.array_equal(off[:-2], arena_off) and np.all(off[-2:] == -1)
    # pack into the task list's buffer
    src = t(arena)
    dst = torch.full((inp.buffer_size,), np.nan, dtype=torch.float64, device=dev)
    boff = np.ascontiguousarray(inp.block_offsets, np.int32)
    G.pack_blocks(t(arena_off), t(boff), t(sizes), src, dst)
    want = np.full(inp.buffer_size, np.nan)
    for b in range(len(rows)):
        want[boff[b]:boff[b] + sizes[b]] = arena[arena_off[b]:arena_off[b] + sizes[b]]
    got = dst.cpu().numpy()
    assert np.array_equal(np.isnan(got), np.isnan(want))
    assert np.array_equal(got[~np.isnan(want)], want[~np.isnan(want)])
    # unpack adds into the store
    hab = rng.uniform(-1, 1, size=inp.buffer_size)
    store = t(arena)
    G.unpack_blocks(t(boff), t(arena_off), t(sizes), t(hab), store)
    want2 = arena.copy()
    for b in range(len(rows)):
        want2[arena_off[b]:arena_off[b] + sizes[b]] += hab[boff[b]:boff[b] + sizes[b]]
    assert np.array_equal(store.cpu().numpy(), want2)


@pytest.mark.gpu
def test_packed_pab_feeds_device_collocate():
    """Generation, block look-up, packing and collocation on the device give
    the grids of the host path (host generator, host pab buffer)."""
    import torch
    from cp2k_gb300 import grid as G
    host = W.config("c1_64atoms", scale=0.5, seed=8)
    gen = G.TaskGenerator(host)
    gen.run(host.atom_positions)
    tl = G.GridTaskList.from_generator(gen, precision=G.FP64)
    pab_h = W.density_blocks(host, seed=9)
    rng = np.random.default_rng(2)
    rows, cols, sizes, arena, arena_off, order = _block_store(host, rng)
    boff = np.ascontiguousarray(host.block_offsets, np.int32)
    for b in range(len(rows)):
        arena[arena_off[b]:arena_off[b] + sizes[b]] = pab_h[boff[b]:boff[b] + sizes[b]]
    dev = torch.device("cuda", 0)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device=dev)
    off = torch.empty(len(rows), dtype=torch.int64, device=dev)
    assert G.find_blocks(t(rows[order]), t(cols[order]), t(arena_off[order]), t(rows),
                         t(cols), off) == 0
    assert np.array_equal(gen.host_arrays()["block_offsets"], boff)
    pab = torch.zeros(host.buffer_size, dtype=torch.float64, device=dev)
    G.pack_blocks(off, t(boff), t(sizes), t(arena), pab)
    grids = [torch.zeros(int(np.prod(n)), dtype=torch.float64, device=dev)
             for n in host.npts_local]
    tl.collocate_device(G.GRID_FUNC_AB, pab, grids)
    torch.cuda.synchronize()
    ref = G.GridTaskList(host, precision=G.FP64).collocate(G.GRID_FUNC_AB, pab_h)
    for x, y in zip(grids, ref):
        assert np.abs(x.cpu().numpy() - y).max() <= 1e-12 * max(1.0, np.abs(y).max())
    assert all(v for v in gen.device_arrays().values())
    tl.close()
    gen.free()
