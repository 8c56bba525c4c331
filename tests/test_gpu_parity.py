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


@pytest.mark.parametrize("name,scale,funcs", [
    ("c1_64atoms", 0.3, (100, 200, 302, 412, 503, 602, 703, 801, 902, 906, 1003)),
    ("c2_512atoms", 0.08, (100,)),
    ("c3_256atoms_triclinic", 0.12, (100, 200)),
])
def test_tasklist_fp64(G, O, name, scale, funcs):
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
        assert e < TOL_GRID * 5, (func, e)
    for tau in (False, True):
        h1, f1, v1 = tl.integrate(V, pab, compute_tau=tau, forces=True, virial=True)
        h2, f2, v2 = ot.integrate(V, pab, compute_tau=tau, forces=True, virial=True)
        assert rel_diff(h1, h2) < TOL_GRID * 5, tau
        assert rel_diff(f1, f2) < TOL_DERIV
        assert rel_diff(v1, v2) < TOL_DERIV
        h3, _, _ = tl.integrate(V, compute_tau=tau)
        h4, _, _ = ot.integrate(V, compute_tau=tau)
        assert rel_diff(h3, h4) < TOL_GRID * 5
    tl.close()
    ot.close()
