"""GPU parity at the full sizes of the 64-atom, 512-atom and triclinic
256-atom workloads: the CUDA backend, called through its C ABI, against the
oracle (the FP64 restatement of CP2K's REF backend) on the same seeded
inputs, element by element.

Bounds, in the reference's measure max |test - ref| / max(1, |ref|)
(src/grid/grid_task_list.c:249-262):

* FP64 path, grids and hab: 1e-12 (grid_task_list.c:353-370), except where
  CP2K's own REF backend and the oracle -- the same formulas in a different
  order of FP64 operations -- already differ by more on that input
  (tests/golden/fp64_spread.json, written by make_fp64_spread.py from CP2K's
  REF library).  There the bound is three times that spread.  This is the
  triclinic l <= 4 workload, whose densities reach 3.5e3 and whose hab
  entries reach 4e4 from sums that cancel to a few units.
* FP64 path, forces and virial: 1e-8 (grid_task_list.c:386-387, 409).
* mixed path (the default per-task FP32 / double-float split): rho <= 1e-6
  and Tr(V rho) energy error <= 1e-8 Ha per atom (the targets of the mixed
  mode), hab <= 1e-6, forces and virial <= 1e-5.
"""
import json
import os

import numpy as np
import pytest

from sample_tasks import rel_diff

pytestmark = pytest.mark.gpu

SPREAD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fp64_spread.json")
TOL_GRID, TOL_DERIV = 1e-12, 1e-8

CASES = {
    "c1_64atoms": (100, 200, 302, 412, 503, 602, 703, 801, 902, 906, 1003),
    "c2_512atoms": (100, 200),
    "c3_256atoms_triclinic": (100, 200),
}


def fp64_bound(name, key):
    with open(SPREAD) as fh:
        s = json.load(fh)[name][key]
    return max(TOL_GRID, 3.0 * s)


@pytest.fixture(scope="module")
def G():
    from cp2k_gb300 import grid
    grid.lib()
    return grid


@pytest.fixture(scope="module")
def O():
    from oracle import oracle
    return oracle


def energy(rho, V, inp):
    dvol = [abs(float(np.linalg.det(d))) for d in inp.dh]
    return sum(float((a * v).sum()) * dv for a, v, dv in zip(rho, V, dvol))


@pytest.mark.parametrize("name", sorted(CASES))
def test_fullsize_fp64(G, O, name):
    from cp2k_gb300 import workload as W
    inp = W.config(name, seed=5)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    tl = G.GridTaskList(inp, precision=G.FP64)
    ot = O.OracleTaskList(inp)
    for func in CASES[name]:
        e = max(rel_diff(a, b) for a, b in zip(tl.collocate(func, pab), ot.collocate(func, pab)))
        assert e < fp64_bound(name, f"rho{func}"), (func, e)
    for tau in (0, 1):
        h1, f1, v1 = tl.integrate(V, pab, compute_tau=bool(tau), forces=True, virial=True)
        h2, f2, v2 = ot.integrate(V, pab, compute_tau=bool(tau), forces=True, virial=True)
        assert rel_diff(h1, h2) < fp64_bound(name, f"hab_tau{tau}"), tau
        assert rel_diff(f1, f2) < TOL_DERIV
        assert rel_diff(v1, v2) < TOL_DERIV
        # hab alone (no density matrix passed): the same kernels without forces
        h3, _, _ = tl.integrate(V, compute_tau=bool(tau))
        assert rel_diff(h3, h2) < fp64_bound(name, f"hab_tau{tau}"), tau
    tl.close()
    ot.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_fullsize_mixed(G, O, name):
    from cp2k_gb300 import workload as W
    inp = W.config(name, seed=5)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    tl = G.GridTaskList(inp, precision=G.MIXED)
    ot = O.OracleTaskList(inp)
    r = ot.collocate(100, pab)
    g = tl.collocate(100, pab)
    assert max(rel_diff(a, b) for a, b in zip(g, r)) < 1e-6
    assert abs(energy(g, V, inp) - energy(r, V, inp)) / inp.natoms < 1e-8
    h1, f1, v1 = tl.integrate(V, pab, forces=True, virial=True)
    h2, f2, v2 = ot.integrate(V, pab, forces=True, virial=True)
    assert rel_diff(h1, h2) < 1e-6
    assert rel_diff(f1, f2) < 1e-5
    assert rel_diff(v1, v2) < 1e-5
    tl.close()
    ot.close()


@pytest.mark.parametrize("api", ["cp2k", "backend"])
def test_recreate_with_moved_geometry(G, O, api):
    """CP2K re-creates the task list through its existing handle whenever the
    geometry changes (src/grid/grid_task_list.c:42-63).  The list built for
    one geometry is re-created for another (other atom positions, another
    task count); results match the oracle on the new geometry, and the
    settings made on the handle (precision, mixed threshold) carry over."""
    from cp2k_gb300 import workload as W
    first = W.config("c1_64atoms", scale=0.3, seed=5)
    moved = W.config("c1_64atoms", scale=0.3, seed=6)
    assert moved.ntasks != first.ntasks
    tl = G.GridTaskList(first, precision=G.FP64, api=api)
    tl.collocate(100, W.density_blocks(first))
    for prec, tau, tol, tol_d in ((G.FP64, None, TOL_GRID, TOL_DERIV), (G.MIXED, 0.0, 1e-9, 1e-7)):
        tl.set_precision(prec)
        if tau is not None:
            tl.set_mixed_threshold(tau)
        tl.recreate(moved)
        assert G.lib().grid_gb300_get_precision(tl.impl) == prec
        if tau is not None:
            # threshold 0 kept: every task in the double-float class
            assert tl.mixed_split() == (0.0, 0.0)
        pab = W.density_blocks(moved)
        V = W.potential_grids(moved)
        ot = O.OracleTaskList(moved)
        e = max(rel_diff(a, b) for a, b in zip(tl.collocate(100, pab), ot.collocate(100, pab)))
        assert e < tol
        h1, f1, v1 = tl.integrate(V, pab, forces=True, virial=True)
        h2, f2, v2 = ot.integrate(V, pab, forces=True, virial=True)
        assert rel_diff(h1, h2) < tol
        assert rel_diff(f1, f2) < tol_d
        assert rel_diff(v1, v2) < tol_d
        ot.close()
        tl.recreate(first)  # and back, through the same handle
    tl.close()
