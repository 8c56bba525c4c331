"""CUDA-graph capture of one SCF step (grid_gb300_capture_step): a replay
gives the results of the plain call sequence, reads its inputs at replay
time, counts its kernels, and refuses to run after the task list changed."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _setup(precision):
    import torch
    from cp2k_gb300 import grid as G
    from cp2k_gb300 import workload as W
    inp = W.config("c1_64atoms", scale=0.3, seed=8)
    pab = torch.tensor(W.density_blocks(inp), device="cuda")
    V = [torch.tensor(v, device="cuda") for v in W.potential_grids(inp)]
    rho = [torch.empty(n, dtype=torch.float64, device="cuda") for n in inp.grid_sizes()]
    hab = torch.empty(inp.buffer_size, dtype=torch.float64, device="cuda")
    tl = G.GridTaskList(inp, precision=precision)
    return torch, G, W, inp, pab, V, rho, hab, tl


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_replay_matches_plain_calls(prec):
    torch, G, W, inp, pab, V, rho, hab, tl = _setup(prec)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        tl.collocate_device(100, pab, rho, stream=s)
        tl.integrate_device(V, hab, stream=s)
    s.synchronize()
    rho0 = [g.clone() for g in rho]
    hab0 = hab.clone()
    n0 = G.kernel_launches()
    with torch.cuda.stream(s):
        tl.collocate_device(100, pab, rho, stream=s)
        tl.integrate_device(V, hab, stream=s)
    s.synchronize()
    per_step = G.kernel_launches() - n0
    g = tl.capture_step(100, pab, rho, V, hab, stream=s)
    assert g.kernels == per_step
    for r in rho:
        r.zero_()
    hab.zero_()
    torch.cuda.synchronize()
    n1 = G.kernel_launches()
    g.launch(stream=s)
    g.wait(stream=s)
    assert G.kernel_launches() - n1 == per_step
    tol = 1e-13
    for a, b in zip(rho, rho0):
        assert float((a - b).abs().max()) <= tol * max(1.0, float(b.abs().max()))
    assert float((hab - hab0).abs().max()) <= tol * max(1.0, float(hab0.abs().max()))
    # new inputs in the same buffers: the replay reads them
    pab.mul_(-0.5)
    g.launch(stream=s)
    g.wait(stream=s)
    for a, b in zip(rho, rho0):
        assert float((a + 0.5 * b).abs().max()) <= tol * max(1.0, float(b.abs().max()))
    g.free()
    tl.close()


def test_replay_after_change_fails_loudly():
    code = (
        "import torch\n"
        "from cp2k_gb300 import grid as G, workload as W\n"
        "inp = W.config('c1_64atoms', scale=0.2, seed=8)\n"
        "pab = torch.tensor(W.density_blocks(inp), device='cuda')\n"
        "V = [torch.tensor(v, device='cuda') for v in W.potential_grids(inp)]\n"
        "rho = [torch.empty(n, dtype=torch.float64, device='cuda') for n in inp.grid_sizes()]\n"
        "hab = torch.empty(inp.buffer_size, dtype=torch.float64, device='cuda')\n"
        "tl = G.GridTaskList(inp, precision=G.MIXED)\n"
        "s = torch.cuda.Stream()\n"
        "g = tl.capture_step(100, pab, rho, V, hab, stream=s)\n"
        "g.launch(stream=s); g.wait(stream=s)\n"
        "print('REPLAYED', flush=True)\n"
        "tl.set_precision(G.FP64)\n"
        "g.launch(stream=s)\n"
        "print('RELAUNCHED', flush=True)\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=300)
    assert "REPLAYED" in r.stdout and "RELAUNCHED" not in r.stdout
    assert r.returncode != 0 and "capture again" in r.stderr


def test_autotune_keeps_results():
    torch, G, W, inp, pab, V, rho, hab, tl = _setup(1)
    tl.collocate_device(100, pab, rho)
    tl.integrate_device(V, hab)
    torch.cuda.synchronize()
    rho0 = [g.clone() for g in rho]
    hab0 = hab.clone()
    ms = tl.autotune(100, pab, rho, V, hab)
    assert ms > 0 and tl.tuned_split() in (26, 34, 42, 66)
    tl.set_launch_timing(True)
    tl.collocate_device(100, pab, rho)
    info = tl.launch_timings()
    tl.integrate_device(V, hab)
    torch.cuda.synchronize()
    assert all(1 <= i["warps_per_block"] <= 4 for i in info)
    for a, b in zip(rho, rho0):
        assert float((a - b).abs().max()) <= 1e-13 * max(1.0, float(b.abs().max()))
    assert float((hab - hab0).abs().max()) <= 1e-13 * max(1.0, float(hab0.abs().max()))
    tl.close()
