"""The allocation-free entry point grid_gb300_collocate_pgf_product_static.

Callers that cannot allocate device memory while they run (a program that
gave the GPU's memory to its own fixed arena at start-up, drivers that forbid
cudaMalloc after initialisation because it can synchronise the device)
collocate single primitive pairs through it; its scratch is one static device
array shared by all calls.  Each recorded CP2K task is
collocated twice in a row through it (through the C ABI) and both results are
compared with the task-list entry point (grid_gb300_collocate_device_async on
a one-task list) at the FP64 tolerance of the other parity tests.  This file
is collected last so that a failure here cannot hide the other tests."""
import numpy as np
import pytest

from sample_tasks import SAMPLE_TASKS, digest_task, load_digests, rel_diff

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", SAMPLE_TASKS)
def test_static_scratch_matches_task_list(name):
    import torch
    from cp2k_gb300 import grid as G
    from cp2k_gb300.tasklist import single_task_list

    t = digest_task(load_digests()[name])
    inp = single_task_list(t)
    n = int(np.prod(t["npts_local"]))
    dev = torch.device("cuda", 0)
    # existing entry point: one-task list (block = 0.5 * rscale * pab, internal rscale 2)
    tl = G.GridTaskList(inp, precision=G.FP64)
    ref = torch.zeros(n, dtype=torch.float64, device=dev)
    pab_blocks = torch.tensor((0.5 * t["rscale"] * t["pab"]).ravel(), device=dev)
    tl.collocate_device(t["func"], pab_blocks, [ref])
    torch.cuda.synchronize()
    ref_h = ref.cpu().numpy()
    tl.close()
    pab = torch.tensor(np.ascontiguousarray(t["pab"]).ravel(), device=dev)
    for call in range(2):
        out = torch.zeros(n, dtype=torch.float64, device=dev)
        status = G.collocate_pgf_product_static(t, pab, out)
        assert status == 0, G.lib().grid_gb300_static_scratch_error()
        torch.cuda.synchronize()
        assert rel_diff(out.cpu().numpy(), ref_h) < 1e-12, call


def test_static_scratch_rejects_oversized_task():
    """A task whose sphere bounds would not fit the static array is refused on
    the host with a message; nothing is copied or launched."""
    import torch
    from cp2k_gb300 import grid as G

    t = dict(digest_task(load_digests()["ortho_density_l0000"]))
    h = 0.01
    t["dh"] = [[h, 0, 0], [0, h, 0], [0, 0, h]]
    t["dh_inv"] = [[1 / h, 0, 0], [0, 1 / h, 0], [0, 0, 1 / h]]
    t["radius"] = 20.0
    edge = 2 * int(np.ceil(t["radius"] / h)) + 2  # ~4000 points per cube edge
    assert 2.0 * edge * (2 + 2 * edge) > G.lib().grid_gb300_static_scratch_bytes()
    t["npts_global"] = t["npts_local"] = [edge, edge, edge]
    pab = torch.tensor(np.ascontiguousarray(t["pab"]).ravel(), device="cuda")
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert G.collocate_pgf_product_static(t, pab, out) != 0
    assert b"scratch" in G.lib().grid_gb300_static_scratch_error()
    # out of range angular momenta are refused the same way
    t2 = dict(digest_task(load_digests()["ortho_density_l0000"]))
    t2["la_max"] = 12
    assert G.collocate_pgf_product_static(t2, pab, out) != 0
    torch.cuda.synchronize()
    assert float(out.abs().max()) == 0.0


def test_static_scratch_rejects_box_beyond_shared_memory():
    """A general-path task (border mask set) whose index box fits the static
    array but not the grid kernel's shared memory is refused on the host with
    a message, and a task-list call made afterwards still runs and matches the
    oracle (no stale launch error is left behind)."""
    import torch
    from cp2k_gb300 import grid as G
    from cp2k_gb300.tasklist import single_task_list
    from oracle import oracle as O

    base = digest_task(load_digests()["ortho_density_l0000"])
    t = dict(base)
    h = 0.01
    t["dh"] = [[h, 0, 0], [0, h, 0], [0, 0, h]]
    t["dh_inv"] = [[1 / h, 0, 0], [0, 1 / h, 0], [0, 0, 1 / h]]
    t["radius"] = 200.0  # 40,000 points along j: per-warp tables > 200 KB
    t["border_mask"] = 1
    t["npts_global"] = t["npts_local"] = [64, 64, 64]
    pab = torch.tensor(np.ascontiguousarray(t["pab"]).ravel(), device="cuda")
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert G.collocate_pgf_product_static(t, pab, out) != 0
    assert b"shared memory" in G.lib().grid_gb300_static_scratch_error()
    torch.cuda.synchronize()
    assert float(out.abs().max()) == 0.0
    inp = single_task_list(base)
    tl = G.GridTaskList(inp, precision=G.FP64)
    ot = O.OracleTaskList(inp)
    pab_c = (0.5 * base["rscale"] * base["pab"]).ravel()
    assert rel_diff(tl.collocate(base["func"], pab_c)[0], ot.collocate(base["func"], pab_c)[0]) < 1e-12
    tl.close()
    ot.close()
