"""GPU parity: the CUDA backend, called through its C ABI, against the oracle
(the FP64 restatement of CP2K's REF backend) on the same seeded inputs.

FP64 path tolerance: max |test - ref| / max(1, |ref|) <= 1e-12 for grids and
hab (the reference's own validation measure and bound,
src/grid/grid_task_list.c:249-262, 353-370), 1e-8 for forces and virial (the
reference's bound for these, grid_task_list.c:386-387, 409)."""
import numpy as np
import pytest

from sample_tasks import SAMPLE_TASKS, digest_task, load_digests, rel_diff

pytestmark = pytest.mark.gpu

TOL_GRID, TOL_DERIV = 1e-12, 1e-8


@pytest.fixture(scope="module")
def G():
    from cp2k_gb300 import grid
    grid.lib()
    return grid


@pytest.fixture(scope="module")
def O():
    from oracle import oracle
    return oracle


@pytest.mark.parametrize("name", SAMPLE_TASKS)
def test_sample_task_fp64(G, O, name):
    """Each recorded CP2K task, replayed as a one-task list (grid_replay.c
    batched mode): GPU vs oracle on the full grid and vs the recorded values."""
    from cp2k_gb300.tasklist import single_task_list
    d = load_digests()[name]
    t = digest_task(d)
    inp = single_task_list(t)
    tl = G.GridTaskList(inp, precision=G.FP64)
    ot = O.OracleTaskList(inp)
    pab_c = (0.5 * t["rscale"] * t["pab"]).ravel()
    g_gpu = tl.collocate(t["func"], pab_c)[0]
    g_ora = ot.collocate(t["func"], pab_c)[0]
    assert rel_diff(g_gpu, g_ora) < TOL_GRID
    assert rel_diff(g_gpu[d["grid_idx"]], d["grid_val"]) < 1e-12
    assert abs(g_gpu.sum() - d["grid_sum"]) / max(1.0, abs(d["grid_sum"])) < 1e-10
    tau = t["func"] == 200
    pab_i = (0.5 * t["pab"]).ravel()
    hab, f, v = tl.integrate([g_ora], pab_i, compute_tau=tau, forces=True, virial=True)
    hab_o, f_o, v_o = ot.integrate([g_ora], pab_i, compute_tau=tau, forces=True, virial=True)
    assert rel_diff(hab, hab_o) < TOL_GRID
    assert rel_diff(f, f_o) < TOL_DERIV
    assert rel_diff(v, v_o) < TOL_DERIV
    # against the recorded values (which came from the recorded grid)
    assert rel_diff(hab.reshape(t["n2"], t["n1"]), d["hab"]) < 1e-11
    assert rel_diff(f, np.array(d["forces"])) < 1e-8
    assert rel_diff(v, np.array(d["virial"])) < 1e-8
    tl.close()
    ot.close()


@pytest.mark.parametrize("name", SAMPLE_TASKS)
def test_sample_task_double_float(G, O, name):
    """Each recorded CP2K task in the mixed mode with every task in the
    double-float class (threshold 0): the orthorhombic and the general
    double-float kernels, border masks included (general_subpatch*,
    general_overflow), within the mixed mode's stated bounds (1e-9 for grids
    and hab, 1e-7 for forces and virial)."""
    from cp2k_gb300.tasklist import single_task_list
    d = load_digests()[name]
    t = digest_task(d)
    inp = single_task_list(t)
    tl = G.GridTaskList(inp, precision=G.MIXED)
    tl.set_mixed_threshold(0.0)
    ot = O.OracleTaskList(inp)
    pab_c = (0.5 * t["rscale"] * t["pab"]).ravel()
    g_ora = ot.collocate(t["func"], pab_c)[0]
    assert rel_diff(tl.collocate(t["func"], pab_c)[0], g_ora) < 1e-9
    tau = t["func"] == 200
    pab_i = (0.5 * t["pab"]).ravel()
    hab, f, v = tl.integrate([g_ora], pab_i, compute_tau=tau, forces=True, virial=True)
    hab_o, f_o, v_o = ot.integrate([g_ora], pab_i, compute_tau=tau, forces=True, virial=True)
    assert rel_diff(hab, hab_o) < 1e-9
    assert rel_diff(f, f_o) < 1e-7
    assert rel_diff(v, v_o) < 1e-7
    tl.close()
    ot.close()


@pytest.mark.parametrize("name", SAMPLE_TASKS)
def test_sample_task_fp32(G, O, name):
    """Each recorded CP2K task in plain FP32 (orthorhombic and general FP32
    kernels, border masks included): max |d| / max |ref| <= 1e-5 for the
    grid and hab.  (Single tasks are looser than the workloads' 2e-6: the
    l2200 task, whose polynomial has only l = 2 terms in both factors,
    cancels to 3.2e-6.)"""
    from cp2k_gb300.tasklist import single_task_list
    d = load_digests()[name]
    t = digest_task(d)
    inp = single_task_list(t)
    tl = G.GridTaskList(inp, precision=G.FP32)
    ot = O.OracleTaskList(inp)
    pab_c = (0.5 * t["rscale"] * t["pab"]).ravel()
    g_ora = ot.collocate(t["func"], pab_c)[0]
    g = tl.collocate(t["func"], pab_c)[0]
    assert float(np.abs(g - g_ora).max()) <= 1e-5 * float(np.abs(g_ora).max())
    tau = t["func"] == 200
    pab_i = (0.5 * t["pab"]).ravel()
    hab, _, _ = tl.integrate([g_ora], pab_i, compute_tau=tau)
    hab_o, _, _ = ot.integrate([g_ora], pab_i, compute_tau=tau)
    assert float(np.abs(hab - hab_o).max()) <= 1e-5 * float(np.abs(hab_o).max())
    tl.close()
    ot.close()


# Reduced-size variants of the workloads (seed 5 at full size is in
# test_parity_fullsize.py).  The triclinic l<=4 case with compute_tau reaches
# contraction order 11 on |hab| ~ 2e3: two FP64 evaluation orders differ
# there by up to ~7e-12 relative (on the full-size workload CP2K's REF
# backend and the oracle themselves differ by 1.7e-12,
# tests/golden/fp64_spread.json), so its bound is 1e-11.
@pytest.mark.parametrize("name,scale,funcs,tol", [
    ("c1_64atoms", 0.3, (100, 200, 302, 412, 503, 602, 703, 801, 902, 906, 1003), TOL_GRID),
    ("c2_512atoms", 0.08, (100,), TOL_GRID),
    ("c3_256atoms_triclinic", 0.12, (100, 200), 1e-11),
])
def test_tasklist_fp64(G, O, name, scale, funcs, tol):
    from cp2k_gb300 import workload as W
    inp = W.config(name, scale=scale, seed=5)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    tl = G.GridTaskList(inp, precision=G.FP64)
    ot = O.OracleTaskList(inp)
    for func in funcs:
        g1 = tl.collocate(func, pab)
        g2 = ot.collocate(func, pab)
        e = max(rel_diff(a, b) for a, b in zip(g1, g2))
        assert e < tol, (func, e)
    for tau in (False, True):
        h1, f1, v1 = tl.integrate(V, pab, compute_tau=tau, forces=True, virial=True)
        h2, f2, v2 = ot.integrate(V, pab, compute_tau=tau, forces=True, virial=True)
        assert rel_diff(h1, h2) < tol, tau
        assert rel_diff(f1, f2) < TOL_DERIV
        assert rel_diff(v1, v2) < TOL_DERIV
        h3, _, _ = tl.integrate(V, compute_tau=tau)
        h4, _, _ = ot.integrate(V, compute_tau=tau)
        assert rel_diff(h3, h4) < tol
    tl.close()
    ot.close()


# Stated error bounds of the reduced-precision paths against the FP64 oracle,
# measured on seeded inputs (uniform [-1, 1] density-matrix blocks and
# potential), max |d| / max(1, |ref|) unless noted:
#   MIXED, default split (tasks with contribution bound <= 0.3 in FP32, the
#       rest in double-float):             rho, hab <= 1e-6, forces <= 1e-5
#   MIXED, threshold 0 (all double-float): rho, hab <= 1e-9, forces <= 1e-7
#   FP32 (plain FP32 per-point work):      max |d| / max |ref| <= 2e-6
@pytest.mark.parametrize("name,scale", [("c1_64atoms", 0.3), ("c2_512atoms", 0.08),
                                        ("c3_256atoms_triclinic", 0.12)])
def test_reduced_precision_bounds(G, O, name, scale):
    from cp2k_gb300 import workload as W
    inp = W.config(name, scale=scale, seed=9)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    ot = O.OracleTaskList(inp)
    g_ref = ot.collocate(100, pab)
    h_ref, f_ref, _ = ot.integrate(V, pab, forces=True)
    gmax = max(float(np.abs(g).max()) for g in g_ref)
    hmax = float(np.abs(h_ref).max())
    for prec, tau, tol_rel, tol_f, tol_max in ((G.MIXED, None, 1e-6, 1e-5, None),
                                                (G.MIXED, 0.0, 1e-9, 1e-7, None),
                                                (G.FP32, None, None, None, 2e-6)):
        tl = G.GridTaskList(inp, precision=prec)
        if tau is not None:
            tl.set_mixed_threshold(tau)
        g = tl.collocate(100, pab)
        h, f, _ = tl.integrate(V, pab, forces=True)
        if tol_rel is not None:
            assert max(rel_diff(a, b) for a, b in zip(g, g_ref)) < tol_rel
            assert rel_diff(h, h_ref) < tol_rel
            assert rel_diff(f, f_ref) < tol_f
        else:
            assert max(float(np.abs(a - b).max()) for a, b in zip(g, g_ref)) / gmax < tol_max
            assert float(np.abs(h - h_ref).max()) / hmax < tol_max
        tl.close()
    ot.close()


def test_cp2k_surface_and_empty_list(G):
    """grid_create_task_list & co. (the CP2K symbols) on an empty task list
    zero their outputs (src/grid/grid_task_list.c:185-189, 290-311)."""
    from cp2k_gb300 import workload as W
    inp = W.config("c1_64atoms", scale=0.1, seed=3)
    empty = type(inp)(**{**inp.__dict__, **{k: getattr(inp, k)[:0] for k in (
        "level_list", "iatom_list", "jatom_list", "iset_list", "jset_list", "ipgf_list",
        "jpgf_list", "border_mask_list", "block_num_list", "radius_list", "rab_list")}})
    tl = G.GridTaskList(empty, api="cp2k")
    g = tl.collocate(100, np.ones(inp.buffer_size))
    assert all(float(np.abs(x).max()) == 0.0 for x in g)
    h, f, v = tl.integrate([np.ones(n) for n in inp.grid_sizes()], np.ones(inp.buffer_size),
                           forces=True, virial=True)
    assert float(np.abs(h).max()) == 0.0 and float(np.abs(f).max()) == 0.0
    assert float(np.abs(v).max()) == 0.0
    tl.close()


def test_schedules_agree(G, O):
    """Reordering the work queues (size order, input order) leaves the FP64
    results within rounding.  (Re-creation through an existing handle is
    tested in test_parity_fullsize.py.)"""
    from cp2k_gb300 import workload as W
    inp = W.config("c1_64atoms", scale=0.2, seed=4)
    pab = W.density_blocks(inp)
    tl = G.GridTaskList(inp)
    outs = []
    for sched in (G.SCHEDULE_SIZE, G.SCHEDULE_INPUT, G.SCHEDULE_SIZE):
        tl.set_schedule(sched)
        outs.append(tl.collocate(100, pab))
    for o in outs[1:]:
        assert max(rel_diff(a, b) for a, b in zip(o, outs[0])) < 1e-13
    tl.close()


@pytest.mark.parametrize("case", ["ortho", "tricl"])
@pytest.mark.parametrize("api", ["backend", "cp2k"])
def test_ref_golden_fp64(G, case, api):
    """Against outputs of CP2K's own REF backend (committed fixtures): both the
    orthorhombic and the general (triclinic) path, rho and tau densities,
    hab with and without tau, forces and virial."""
    import golden_cases
    inp, pab, V, exp = golden_cases.load(case)
    tl = G.GridTaskList(inp, precision=G.FP64, api=api)
    for func in (100, 200):
        got = tl.collocate(func, pab)
        assert max(rel_diff(a, b) for a, b in zip(got, exp[f"rho{func}"])) < TOL_GRID
    for tau in (0, 1):
        h, f, v = tl.integrate(V, pab, compute_tau=bool(tau), forces=True, virial=True)
        assert rel_diff(h, exp[f"hab_tau{tau}"]) < TOL_GRID
        assert rel_diff(f, exp[f"forces_tau{tau}"]) < TOL_DERIV
        assert rel_diff(v, exp[f"virial_tau{tau}"]) < TOL_DERIV
    tl.close()


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_collocate_variants_agree(G, O, prec):
    """Row-walk and point-list collocate kernels give the same grids up to the
    order of the FP64 atomic additions (the same per-point arithmetic), and
    the point-list kernel matches the oracle in FP64."""
    from cp2k_gb300 import workload as W
    inp = W.config("c2_512atoms", scale=0.1, seed=31)
    pab = W.density_blocks(inp)
    tl = G.GridTaskList(inp, precision=prec)
    out = []
    for v in (0, 1):
        tl.set_collocate_variant(v)
        out.append(tl.collocate(100, pab))
    # FP64: atomic order only; mixed / FP32: also the order of the FP32 adds
    # into the low-word grid and of the FP32 row sums
    tol = TOL_GRID if prec == G.FP64 else 1e-10
    for a, b in zip(*out):
        assert rel_diff(a, b) < tol
    if prec == G.FP64:
        ot = O.OracleTaskList(inp)
        ref = ot.collocate(100, pab)
        assert max(rel_diff(a, b) for a, b in zip(out[1], ref)) < TOL_GRID
        ot.close()
    tl.close()


@pytest.mark.parametrize("prec,tau", [(1, 0.0), (1, None), (2, None)])
def test_general_collocate_variants_agree(G, O, prec, tau):
    """The general path's lane-per-i kernels (variant 0) and point-list
    kernels (variant 1) visit the same points: double-float grids agree to
    the order of the additions, FP32 grids to FP32 rounding (the point-list
    kernel evaluates the polynomial in Horner form); the point-list
    double-float grids match the oracle within the mixed mode's bound."""
    from cp2k_gb300 import workload as W
    inp = W.config("c3_256atoms_triclinic", scale=0.12, seed=33)
    pab = W.density_blocks(inp)
    tl = G.GridTaskList(inp, precision=prec)
    if tau is not None:
        tl.set_mixed_threshold(tau)
    out = []
    for v in (0, 1):
        tl.set_collocate_variant(v)
        out.append(tl.collocate(100, pab))
    if prec == G.FP32:
        gmax = max(float(np.abs(g).max()) for g in out[0])
        assert max(float(np.abs(a - b).max()) for a, b in zip(*out)) / gmax < 2e-6
    else:
        tol = 1e-10 if tau == 0.0 else 1e-6
        for a, b in zip(*out):
            assert rel_diff(a, b) < tol
    if tau == 0.0:
        ot = O.OracleTaskList(inp)
        ref = ot.collocate(100, pab)
        assert max(rel_diff(a, b) for a, b in zip(out[1], ref)) < 1e-9
        ot.close()
    tl.close()


@pytest.mark.parametrize("name,scale", [("c1_64atoms", 0.3), ("c3_256atoms_triclinic", 0.1)])
def test_mixed_all_functions_tau_virial(G, O, name, scale):
    """The mixed mode on every family of grid_func (derivative shifts of the
    density) and on integration with tau and virial, against the FP64 oracle
    within the mixed mode's stated bounds."""
    from cp2k_gb300 import workload as W
    inp = W.config(name, scale=scale, seed=23)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    ot = O.OracleTaskList(inp)
    tl = G.GridTaskList(inp, precision=G.MIXED)
    for func in (200, 301, 411, 501, 602, 703, 801, 902, 905, 1003):
        g = tl.collocate(func, pab)
        r = ot.collocate(func, pab)
        assert max(rel_diff(a, b) for a, b in zip(g, r)) < 1e-6, func
    h, f, v = tl.integrate(V, pab, compute_tau=True, forces=True, virial=True)
    ho, fo, vo = ot.integrate(V, pab, compute_tau=True, forces=True, virial=True)
    assert rel_diff(h, ho) < 1e-6
    assert rel_diff(f, fo) < 1e-5
    assert rel_diff(v, vo) < 1e-5
    tl.close()
    ot.close()


@pytest.mark.parametrize("lmax,random_sphi,funcs,tau", [
    (6, False, (100, 200), False),   # forces + virial: la = 8, lb = 7, lp = 15
    (5, False, (100, 200, 801), True),  # DXDX la = lb = 7; tau + virial la = 8, lb = 7
    (3, True, (100, 200, 801), True),
])
def test_high_l_and_contraction_fp64(G, O, lmax, random_sphi, funcs, tau):
    """Sets up to l = 6 and random orthonormal contraction matrices (sphi),
    against the oracle. The cases reach the largest shifted angular momenta
    whose per-task coefficient block (cab, alpha, cxyz) fits the 200 KB of
    shared memory of one CTA: la = 8 with lb = 7."""
    from cp2k_gb300 import workload as W
    inp = W.config("c1_64atoms", scale=0.12, seed=41, random_sphi=random_sphi,
                   elements=[(1.0, [lmax, 1])], zet=(0.3, 20.0))
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    tl = G.GridTaskList(inp, precision=G.FP64)
    ot = O.OracleTaskList(inp)
    for func in funcs:
        e = max(rel_diff(a, b) for a, b in zip(tl.collocate(func, pab), ot.collocate(func, pab)))
        assert e < 1e-11, (func, e)
    h1, f1, v1 = tl.integrate(V, pab, compute_tau=tau, forces=True, virial=True)
    h2, f2, v2 = ot.integrate(V, pab, compute_tau=tau, forces=True, virial=True)
    assert rel_diff(h1, h2) < 1e-11
    assert rel_diff(f1, f2) < TOL_DERIV
    assert rel_diff(v1, v2) < TOL_DERIV
    tl.close()
    ot.close()


def test_general_boxes_split_by_planes(G, O):
    """Large general-path boxes are split into plane ranges, each a work item
    of its own (integrate adds the ranges' partial coefficients); the split
    runs give the oracle's results, in FP64 and in the double-float class."""
    from cp2k_gb300 import workload as W
    inp = W.config("c3_256atoms_triclinic", scale=0.12, seed=13)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    ot = O.OracleTaskList(inp)
    g_ref = ot.collocate(100, pab)
    h_ref, f_ref, v_ref = ot.integrate(V, pab, forces=True, virial=True)
    for prec, tol, tol_d in ((G.FP64, 1e-11, TOL_DERIV), (G.MIXED, 1e-9, 1e-7)):
        tl = G.GridTaskList(inp, precision=prec)
        if prec == G.MIXED:
            tl.set_mixed_threshold(0.0)
        tl.set_launch_timing(True)
        g = tl.collocate(100, pab)
        info = [i for i in tl.launch_timings() if i["general"]]
        assert any(i["work_items"] > i["ntasks"] for i in info)
        assert max(rel_diff(a, b) for a, b in zip(g, g_ref)) < tol
        h, f, v = tl.integrate(V, pab, forces=True, virial=True)
        info = [i for i in tl.launch_timings() if i["general"]]
        assert any(i["work_items"] > i["ntasks"] for i in info)
        assert rel_diff(h, h_ref) < tol
        assert rel_diff(f, f_ref) < tol_d
        assert rel_diff(v, v_ref) < tol_d
        tl.close()
    ot.close()


@pytest.mark.parametrize("prec", [0, 1, 2])
@pytest.mark.parametrize("case", ["tricl", "ortho_l3"])
def test_transform_variants_agree(G, O, prec, case):
    """The staged (x, then y, then z) and the direct C_ab <-> C_xyz transforms
    of the coefficient and post kernels give the oracle's results: FP64 to
    the bounds of the FP64 tests, the double-float class (threshold 0) to
    1e-9 / 1e-7, FP32 to 1e-5 of the maximum (its stated accuracy; sets up to
    l = 3 cancel more than the workloads' l <= 2); collocation of rho and of the
    tau density, integration with tau, forces and virial."""
    from cp2k_gb300 import workload as W
    if case == "tricl":
        inp = W.config("c3_256atoms_triclinic", scale=0.1, seed=35)
    else:
        inp = W.config("c1_64atoms", scale=0.2, seed=36, elements=[(1.0, [3, 2])])
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    ot = O.OracleTaskList(inp)
    ref = {f: ot.collocate(f, pab) for f in (100, 200)}
    h_ref, f_ref, v_ref = ot.integrate(V, pab, compute_tau=True, forces=True, virial=True)
    ot.close()
    tl = G.GridTaskList(inp, precision=prec)
    if prec == G.MIXED:
        tl.set_mixed_threshold(0.0)
    tol = {G.FP64: (1e-11, TOL_DERIV), G.MIXED: (1e-9, 1e-7)}
    for variant in (0, 1):
        tl.set_transform_variant(variant)
        for f in (100, 200):
            g = tl.collocate(f, pab)
            if prec == G.FP32:
                gmax = max(float(np.abs(r).max()) for r in ref[f])
                assert max(float(np.abs(a - b).max()) for a, b in zip(g, ref[f])) / gmax < 1e-5
            else:
                assert max(rel_diff(a, b) for a, b in zip(g, ref[f])) < tol[prec][0], (variant, f)
        h, fo, vi = tl.integrate(V, pab, compute_tau=True, forces=True, virial=True)
        if prec == G.FP32:
            assert float(np.abs(h - h_ref).max()) / float(np.abs(h_ref).max()) < 1e-5
        else:
            assert rel_diff(h, h_ref) < tol[prec][0], variant
            assert rel_diff(fo, f_ref) < tol[prec][1], variant
            assert rel_diff(vi, v_ref) < tol[prec][1], variant
    tl.close()


@pytest.mark.parametrize("api,precision", [("cp2k", "fp64"), ("backend", "fp64"),
                                           ("cp2k", "mixed")])
def test_copy_chunks_agree(G, O, api, precision):
    """Host-buffer calls copy pab in and hab out in pieces that overlap the
    kernels (grid_gb300_set_copy_chunks), each piece with work queues of its
    own tasks; 1, 2 and 3 pieces give the oracle's results (FP64: to 1e-12;
    mixed, with its row split: rho and hab to 1e-6, forces and virial to 1e-5,
    relative to max(1, |ref|)), and hab entries past the task list's blocks
    come back zeroed."""
    from cp2k_gb300 import workload as W
    inp = W.config("c2_512atoms", scale=0.1, seed=37)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    ot = O.OracleTaskList(inp)
    g_ref = ot.collocate(100, pab)
    h_ref, f_ref, v_ref = ot.integrate(V, pab, forces=True, virial=True)
    ot.close()
    prec = G.FP64 if precision == "fp64" else G.MIXED
    tol_g, tol_d = (TOL_GRID, TOL_DERIV) if precision == "fp64" else (1e-6, 1e-5)
    tl = G.GridTaskList(inp, precision=prec, api=api)
    for chunks in (1, 2, 3):
        tl.set_copy_chunks(chunks)
        g = tl.collocate(100, pab)
        assert max(rel_diff(a, b) for a, b in zip(g, g_ref)) < tol_g, chunks
        _, hab_buf, _ = tl.host_buffers()
        hab_buf.host[:] = 7.0  # stale values must not survive
        h, f, v = tl.integrate(V, pab, forces=True, virial=True)
        assert rel_diff(h, h_ref) < tol_g, chunks
        assert rel_diff(f, f_ref) < tol_d
        assert rel_diff(v, v_ref) < tol_d
    tl.close()


@pytest.mark.parametrize("name,scale", [("c2_512atoms", 0.1), ("c1_64atoms", 0.3)])
def test_tensor_core_integrate(G, O, name, scale):
    """The FP32 class's orthorhombic integration on the tensor cores (TF32
    products, each operand split in two, three products) against the CUDA-core
    kernel and the oracle: mixed mode within its stated bounds (hab 1e-6,
    forces 1e-5, relative to max(1, |ref|)), plain FP32 within 1e-5 of the
    maximum, the two kernels within 2e-6 of each other."""
    from cp2k_gb300 import workload as W
    inp = W.config(name, scale=scale, seed=39)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    ot = O.OracleTaskList(inp)
    h_ref, f_ref, _ = ot.integrate(V, pab, forces=True)
    h_only_ref, _, _ = ot.integrate(V)
    ot.close()
    for prec in (G.MIXED, G.FP32):
        tl = G.GridTaskList(inp, precision=prec)
        res = {}
        for tc in (0, 1):
            tl.set_tensor_integrate(tc)
            res[tc] = (tl.integrate(V)[0],) + tl.integrate(V, pab, forces=True)[:2]
        hmax = float(np.abs(h_only_ref).max())
        assert float(np.abs(res[1][0] - res[0][0]).max()) / hmax < 2e-6
        if prec == G.MIXED:
            assert rel_diff(res[1][0], h_only_ref) < 1e-6
            assert rel_diff(res[1][1], h_ref) < 1e-6
            assert rel_diff(res[1][2], f_ref) < 1e-5
        else:
            assert float(np.abs(res[1][0] - h_only_ref).max()) / hmax < 1e-5
        tl.close()


def test_row_split(G, O):
    """Mixed mode with the outer rows of the double-float tasks in FP32 (the
    default) on the full 512-atom workload, against the oracle: densities of
    GRID_FUNC_AB and of a derivative function (DXDX, whose class test carries
    the derivative factor) within 1e-6 in the reference measure, the
    Tr(V rho) energy within 1e-8 Ha per atom, hab within 1e-6, forces, virial
    and tau-integrated hab within 1e-5 (relative to max(1, |ref|)); and the
    same bounds with every task whole."""
    from cp2k_gb300 import workload as W
    inp = W.config("c2_512atoms", seed=5)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    ot = O.OracleTaskList(inp)
    tl = G.GridTaskList(inp, precision=G.MIXED)
    split, fp32_points = tl.row_split_stats()
    assert split > 0.05 and fp32_points > tl.mixed_split()[1] + 0.1
    dvol = [abs(float(np.linalg.det(d))) for d in inp.dh]
    res = {}
    for on in (1, 0):
        tl.set_row_split(on)
        rho = {f: tl.collocate(f, pab) for f in (100, 801)}
        res[on] = (rho, tl.integrate(V, pab, forces=True, virial=True),
                   tl.integrate(V, pab, compute_tau=True, forces=True)[:2])
    for f in (100, 801):
        ref = ot.collocate(f, pab)
        for on in (1, 0):
            assert max(rel_diff(a, b) for a, b in zip(res[on][0][f], ref)) < 1e-6, (f, on)
            if f == 100:
                e = [sum(float((a * v).sum()) * dv for a, v, dv in zip(g, V, dvol))
                     for g in (res[on][0][f], ref)]
                assert abs(e[0] - e[1]) / inp.natoms < 1e-8, on
    h2, f2, v2 = ot.integrate(V, pab, forces=True, virial=True)
    ht2, ft2, _ = ot.integrate(V, pab, compute_tau=True, forces=True)
    for on in (1, 0):
        (h1, f1, v1), (ht1, ft1) = res[on][1], res[on][2]
        assert rel_diff(h1, h2) < 1e-6
        assert rel_diff(f1, f2) < 1e-5
        assert rel_diff(v1, v2) < 1e-5
        assert rel_diff(ht1, ht2) < 1e-5
        assert rel_diff(ft1, ft2) < 1e-5
    tl.close()
    ot.close()


# the tensor-core collocation keeps about 21 bits per product (TF32 high and
# low parts, three products): eight times the FP32 bound of the CUDA-core
# kernels where a task's polynomial cancels
TOL_TC_COLL = 8e-5


@pytest.mark.parametrize("name,scale", [("c2_512atoms", 0.1), ("c1_64atoms", 0.3)])
def test_tensor_core_collocate(G, O, name, scale):
    """The mixed mode's FP32-class orthorhombic collocation on the tensor
    cores (opt-in) against the CUDA-core kernels and the oracle: both
    within the mixed mode's bound (rho 1e-6 in the reference measure, shells
    of split tasks included), and within 2e-6 of each other; and with every
    task in the FP32 class (threshold 1e30) within TOL_TC_COLL of the largest
    density value."""
    from cp2k_gb300 import workload as W
    inp = W.config(name, scale=scale, seed=43)
    pab = W.density_blocks(inp)
    ot = O.OracleTaskList(inp)
    ref = ot.collocate(100, pab)
    ot.close()
    rmax = max(float(np.abs(r).max()) for r in ref)
    tl = G.GridTaskList(inp, precision=G.MIXED)
    res = {}
    for tc in (0, 1):
        tl.set_tensor_collocate(tc)
        res[tc] = tl.collocate(100, pab)
        assert max(rel_diff(a, b) for a, b in zip(res[tc], ref)) < 1e-6, tc
    assert max(float(np.abs(a - b).max()) for a, b in zip(res[1], res[0])) / rmax < 2e-6
    tl.set_mixed_threshold(1e30)
    tl.set_tensor_collocate(1)
    g = tl.collocate(100, pab)
    assert max(float(np.abs(a - b).max()) for a, b in zip(g, ref)) / rmax < TOL_TC_COLL
    tl.close()


@pytest.mark.parametrize("name", sorted(SAMPLE_TASKS))
def test_tensor_core_collocate_sample_tasks(G, O, name):
    """Every sample task collocated with the tensor-core kernel (mixed mode,
    threshold 1e30: every task in the FP32 class; the kernel takes the
    orthorhombic tasks with lp <= 6, the others run the CUDA-core kernels):
    max |d| / max |ref| <= TOL_TC_COLL against the oracle."""
    from cp2k_gb300.tasklist import single_task_list
    t = digest_task(load_digests()[name])
    inp = single_task_list(t)
    tl = G.GridTaskList(inp, precision=G.MIXED)
    tl.set_mixed_threshold(1e30)
    tl.set_tensor_collocate(True)
    ot = O.OracleTaskList(inp)
    pab_c = (0.5 * t["rscale"] * t["pab"]).ravel()
    g_ora = ot.collocate(t["func"], pab_c)[0]
    g = tl.collocate(t["func"], pab_c)[0]
    assert float(np.abs(g - g_ora).max()) <= TOL_TC_COLL * float(np.abs(g_ora).max())
    tl.close()
    ot.close()
