"""GPU: CP2K's single-task entry points grid_cpu_collocate_pgf_product and
grid_cpu_integrate_pgf_product (src/grid/grid_api.F:145, 318), run on the GPU
through the C ABI, against the oracle (the restatement of CP2K's REF backend,
src/grid/ref/grid_ref_collocate.c:19-49, grid_ref_integrate.c:44-152) and the
recorded values of the reference's 13 sample tasks.  Bounds as the
reference's unit test: 1e-12 for grids and hab, 1e-8 for forces, virials and
the derivative blocks (src/grid/grid_replay.c:445, 481, 495)."""
import numpy as np
import pytest

from sample_tasks import SAMPLE_TASKS, digest_task, load_digests, rel_diff

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", SAMPLE_TASKS)
def test_pgf_product_matches_oracle(name):
    from cp2k_gb300 import grid as G
    from oracle import oracle as O
    d = load_digests()[name]
    t = digest_task(d)
    g_ora = O.collocate_pgf_product(t)
    g = G.collocate_pgf_product(t)
    assert rel_diff(g, g_ora) < 1e-12
    assert rel_diff(g[d["grid_idx"]], d["grid_val"]) < 1e-12
    # values are added into the caller's grid
    g2 = G.collocate_pgf_product(t, g.copy())
    assert rel_diff(g2, 2 * g_ora) < 1e-12
    tau = t["func"] == 200
    got = G.integrate_pgf_product(t, g_ora, tau, derivatives=not tau)
    exp = O.integrate_pgf_product(t, g_ora, tau, derivatives=not tau)
    assert rel_diff(got[0], exp[0]) < 1e-12
    assert rel_diff(got[0], d["hab"]) < 1e-11
    assert rel_diff(got[1], exp[1]) < 1e-8
    assert rel_diff(got[2], exp[2]) < 1e-8
    assert rel_diff(got[1], np.array(d["forces"])) < 1e-8
    assert rel_diff(got[2][0] + got[2][1], np.array(d["virial"])) < 1e-8
    for a, b in zip(got[3:], exp[3:]):
        assert rel_diff(a, b) < 1e-8
    # hab only, no density matrix
    h, _, _ = G.integrate_pgf_product(t, g_ora, tau, forces=False, virial=False)
    assert rel_diff(h, exp[0]) < 1e-12
