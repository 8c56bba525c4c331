"""The oracle (C restatement of CP2K's REF backend, oracle/grid_oracle.c)
pinned against the reference: its recorded single-task golden vectors
(src/grid/sample_tasks, via the committed digests and, when present, the
files themselves), outputs of CP2K's REF backend on synthetic task lists
(committed fixtures and, when built, the library itself), and the
collocate/integrate adjointness identity."""
import numpy as np
import pytest

import golden_cases
from sample_tasks import (SAMPLE_TASKS, digest_task, have_reference, load_digests,
                          load_sample, rel_diff)


@pytest.fixture(scope="module")
def O():
    from oracle import oracle
    oracle.lib()
    return oracle


def _check_task(O, t, grid_expect_full=None, digest=None):
    from cp2k_gb300.tasklist import single_task_list
    g = O.collocate_pgf_product(t)
    if grid_expect_full is not None:
        assert rel_diff(g, grid_expect_full) < 1e-12
    if digest is not None:
        assert rel_diff(g[digest["grid_idx"]], digest["grid_val"]) < 1e-12
        assert abs(g.sum() - digest["grid_sum"]) <= 1e-10 * max(1.0, abs(digest["grid_sum"]))
    tau = t["func"] == 200
    grid_in = grid_expect_full if grid_expect_full is not None else g
    hab, f, v = O.integrate_pgf_product(t, grid_in, tau)
    ref = digest if digest is not None else {"hab": t["hab"], "forces": [t["force_a"], t["force_b"]],
                                             "virial": t["virial"]}
    assert rel_diff(hab, ref["hab"]) < 1e-11
    # forces / virial: the reference unit test weighs these by 1e-4
    # (src/grid/grid_replay.c:445, 481, 495), i.e. 1e-8 relative
    assert rel_diff(f, np.array(ref["forces"])) < 1e-8
    assert rel_diff(v[0] + v[1], np.array(ref["virial"])) < 1e-8
    # batched replay through a one-task list (grid_replay.c:154-214, 306-327)
    inp = single_task_list(t)
    tl = O.OracleTaskList(inp)
    gb = tl.collocate(t["func"], (0.5 * t["rscale"] * t["pab"]).ravel())[0]
    assert rel_diff(gb, g) < 1e-13
    hb, fb, vb = tl.integrate([grid_in], (0.5 * t["pab"]).ravel(), compute_tau=tau, forces=True,
                              virial=True)
    assert rel_diff(hb.reshape(t["n2"], t["n1"]), hab) < 1e-13
    assert rel_diff(fb, f) < 1e-12
    tl.close()


@pytest.mark.parametrize("name", SAMPLE_TASKS)
def test_oracle_vs_sample_digests(O, name):
    d = load_digests()[name]
    _check_task(O, digest_task(d), digest=d)


@pytest.mark.skipif(not have_reference(), reason="CP2K sources not present")
@pytest.mark.parametrize("name", SAMPLE_TASKS)
def test_oracle_vs_sample_task_files(O, name):
    t = load_sample(name)
    _check_task(O, t, grid_expect_full=t["grid"])


@pytest.mark.parametrize("case", golden_cases.CASES)
def test_oracle_vs_ref_golden(O, case):
    inp, pab, V, exp = golden_cases.load(case)
    tl = O.OracleTaskList(inp)
    for func in (100, 200):
        got = tl.collocate(func, pab)
        assert max(rel_diff(a, b) for a, b in zip(got, exp[f"rho{func}"])) < 1e-12
    for tau in (0, 1):
        h, f, v = tl.integrate(V, pab, compute_tau=bool(tau), forces=True, virial=True)
        assert rel_diff(h, exp[f"hab_tau{tau}"]) < 1e-12
        assert rel_diff(f, exp[f"forces_tau{tau}"]) < 1e-8
        assert rel_diff(v, exp[f"virial_tau{tau}"]) < 1e-8
    tl.close()


def _ref_available():
    try:
        from oracle import refgrid
        return refgrid.available()
    except Exception:
        return False


@pytest.mark.skipif(not _ref_available(), reason="oracle/_ref not built (CP2K sources absent)")
@pytest.mark.parametrize("name,scale,funcs,random_sphi", [
    ("c1_64atoms", 0.2, (100, 200, 303, 421, 502, 601, 702, 803, 903, 904, 1001), False),
    ("c1_64atoms", 0.2, (100,), True),
    ("c3_256atoms_triclinic", 0.08, (100, 200), False),
])
def test_oracle_vs_reference_library(O, name, scale, funcs, random_sphi):
    from cp2k_gb300 import workload as W
    from oracle import refgrid as R
    inp = W.config(name, scale=scale, seed=13, random_sphi=random_sphi)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    ot, rt = O.OracleTaskList(inp), R.RefTaskList(inp)
    for func in funcs:
        e = max(rel_diff(a, b) for a, b in zip(ot.collocate(func, pab), rt.collocate(func, pab)))
        assert e < 5e-12, (func, e)
    for tau in (False, True):
        ho, fo, vo = ot.integrate(V, pab, compute_tau=tau, forces=True, virial=True)
        hr, fr, vr = rt.integrate(V, pab, compute_tau=tau, forces=True, virial=True)
        assert rel_diff(ho, hr) < 5e-12
        assert rel_diff(fo, fr) < 1e-8 and rel_diff(vo, vr) < 1e-8
    ot.close()
    rt.close()


def test_adjointness(O):
    """sum_levels <collocate(P), V> = sum_blocks P . H with H = integrate(V):
    collocate and integrate are adjoint (cab_to_grid / its reverse,
    src/grid/ref/grid_ref_collint.h:917-965); REF's off-diagonal factor 2 is in
    both (grid_ref_task_list.c:369, 625)."""
    from cp2k_gb300 import workload as W
    inp = W.config("c1_64atoms", scale=0.2, seed=17)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    tl = O.OracleTaskList(inp)
    rho = tl.collocate(100, pab)
    hab, _, _ = tl.integrate(V)
    lhs = sum(float(np.dot(r, v)) for r, v in zip(rho, V))
    # hab holds the integrals of each block once; collocate weighs off-diagonal
    # blocks twice -> weight the block entries accordingly
    w = np.ones(inp.buffer_size)
    atoms = {}
    for b, ia, ja in zip(inp.block_num_list - 1, inp.iatom_list, inp.jatom_list):
        atoms[int(b)] = (int(ia), int(ja))
    for b, (ia, ja) in atoms.items():
        if ia != ja:
            n = inp.basis_sets[inp.atom_kinds[ia - 1] - 1].nsgf * \
                inp.basis_sets[inp.atom_kinds[ja - 1] - 1].nsgf
            off = inp.block_offsets[b]
            w[off:off + n] = 2.0
    rhs = float(np.dot(pab * w, hab))
    assert abs(lhs - rhs) <= 1e-10 * max(1.0, abs(lhs))
    tl.close()


def _ref_integrate_pgf(t, grid, tau, derivatives):
    """CP2K's grid_ref_integrate_pgf_product (src/grid/ref/grid_ref_integrate.c:
    44-152) from the reference library built from its sources."""
    import ctypes as C

    from oracle import refgrid as R
    L = R.lib()  # loads the library and runs grid_library_init
    fn = L.grid_ref_integrate_pgf_product
    f64 = lambda a: np.ascontiguousarray(a, np.float64)
    i32 = lambda a: np.ascontiguousarray(a, np.int32)
    p = lambda a: a.ctypes.data_as(C.c_void_p) if a is not None else None
    fn.argtypes = ([C.c_bool, C.c_bool, C.c_int] + [C.c_int] * 4 + [C.c_double] * 2
                   + [C.c_void_p] * 8 + [C.c_double] + [C.c_int] * 4 + [C.c_void_p] * 8)
    hab = np.zeros((t["n2"], t["n1"]))
    f, v = np.zeros((2, 3)), np.zeros((2, 3, 3))
    hd = np.zeros((t["n2"], t["n1"], 3)) if derivatives else None
    ha = np.zeros((t["n2"], t["n1"], 3)) if derivatives else None
    ahd = np.zeros((t["n2"], t["n1"], 3, 3)) if derivatives else None
    arrs = [f64(t["dh"]), f64(t["dh_inv"]), f64(t["ra"]), f64(t["rab"]),
            i32(t["npts_global"]), i32(t["npts_local"]), i32(t["shift_local"]),
            i32(t["border_width"])]
    pab = f64(t["pab"])
    g = f64(grid)
    fn(bool(t["orthorhombic"]), bool(tau), int(t["border_mask"]), t["la_max"], t["la_min"],
       t["lb_max"], t["lb_min"], t["zeta"], t["zetb"], *[p(a) for a in arrs], t["radius"],
       t["o1"], t["o2"], t["n1"], t["n2"], p(g), p(hab), p(pab), p(f), p(v), p(hd), p(ha),
       p(ahd))
    return hab, f, v, hd, ha, ahd


@pytest.mark.parametrize("name", ["ortho_density_l0122", "ortho_density_l3333",
                                  "general_density", "general_subpatch16", "ortho_tau"])
def test_oracle_pgf_derivative_blocks_vs_reference_library(O, name):
    """The single-task integrate's optional outputs -- hdab, hadb, a_hdab
    (d hab / d a, d hab / d b, the virial of hab) and the separate virials of
    atoms a and b -- against CP2K's REF library on the recorded tasks."""
    from oracle import refgrid as R
    if not R.available():
        pytest.skip("CP2K's reference library is not built here")
    t = digest_task(load_digests()[name])
    grid = O.collocate_pgf_product(t)
    tau = t["func"] == 200
    got = O.integrate_pgf_product(t, grid, tau, derivatives=not tau)
    exp = _ref_integrate_pgf(t, grid, tau, derivatives=not tau)
    # hab at the reference's 1e-12; forces and virials at its 1e-8
    # (src/grid/grid_replay.c:445, 481, 495: weighed by 1e-4), which also
    # bounds the derivative blocks built from the same terms
    assert rel_diff(got[0], exp[0]) < 1e-12
    assert rel_diff(got[1], exp[1]) < 1e-8
    assert rel_diff(got[2], exp[2]) < 1e-8
    if not tau:
        for a, b in zip(got[3:], exp[3:]):
            assert rel_diff(a, b) < 1e-8
