"""GPU checks of the learned task-cost model: the CUDA loss/gradient, Adam
and inference kernels against the float64 oracle (oracle/mlp_oracle.py),
training on per-task timings the grid kernels record, and the schedule the
trained model produces against the analytic size schedule (same results,
measured time of both reported)."""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def CM():
    from cp2k_gb300 import costmodel
    from cp2k_gb300 import grid
    grid.lib()
    return costmodel


def _rand(n, seed):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.25, M.NPARAMS).astype(np.float32)
    x = rng.normal(0, 1, (n, M.NIN)).astype(np.float32)
    t = rng.normal(0, 1, n).astype(np.float32)
    return p, x, t


@pytest.mark.parametrize("n", [1, 31, 32, 1000, 4097])
def test_loss_grad_vs_oracle(CM, n):
    import torch
    p, x, t = _rand(n, n)
    m = CM.CostModel(params=p)
    loss, grad = m.loss_grad(torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda"))
    lo, go = M.loss_grad(p.astype(np.float64), x, t)
    assert abs(float(loss.item()) - lo) <= 1e-5 * max(1.0, abs(lo))
    g = grad.cpu().numpy().astype(np.float64)
    # FP32 accumulation over the samples: relative to the largest component
    assert np.max(np.abs(g - go)) <= 2e-5 * np.max(np.abs(go))
    # deterministic: the same call gives the same bits
    _, grad2 = m.loss_grad(torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda"))
    assert torch.equal(grad, grad2)


def test_adam_vs_oracle(CM):
    import torch
    from cp2k_gb300 import grid as G
    p, x, t = _rand(300, 7)
    m = CM.CostModel(params=p)
    xd, td = torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda")
    mo, vo, po = np.zeros(M.NPARAMS), np.zeros(M.NPARAMS), p.astype(np.float64)
    md, vd = torch.zeros_like(m.params), torch.zeros_like(m.params)
    L = G.lib()
    for step in range(1, 4):
        _, grad = m.loss_grad(xd, td)
        _, go = M.loss_grad(po, x, t)
        po, mo, vo = M.adam(po, go, mo, vo, step, 1e-2)
        L.grid_gb300_cost_model_adam(CM._ptr(m.params), CM._ptr(grad), CM._ptr(md), CM._ptr(vd),
                                     step, 1e-2, 0.9, 0.999, 1e-8, None)
    torch.cuda.synchronize()
    assert np.max(np.abs(m.params.cpu().numpy() - po)) < 1e-4


@pytest.mark.parametrize("n", [1, 127, 128, 5000])
def test_predict_vs_oracle(CM, n):
    p, x, _ = _rand(n, 11)
    x = x * 3 + 1
    norm = np.concatenate([x.mean(0), x.std(0) + 0.5]).astype(np.float32)
    m = CM.CostModel(params=p, norm=norm)
    y = m.predict(x)
    yo = M.predict(p.astype(np.float64), x, norm)
    assert np.max(np.abs(y - yo)) <= 1e-4 * max(1.0, np.max(np.abs(yo)))


def test_training_fits_a_smooth_target(CM):
    rng = np.random.default_rng(5)
    X = rng.uniform(-2, 2, (20000, 6)).astype(np.float32)
    T = (np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2] + 0.1 * X[:, 3] ** 2).astype(np.float32)
    m = CM.CostModel(seed=1)
    hist = m.train(X[:16000], T[:16000], epochs=40, batch=1024, X_val=X[16000:], T_val=T[16000:])
    assert hist[-1][2] < 0.05 * float(np.var(T))


def test_schedule_from_recorded_timings(CM):
    """Per-task cycles recorded by the grid kernels train the model; the
    model-ordered queues give the same grids and hab as the size order."""
    import torch
    from cp2k_gb300 import grid as G
    from cp2k_gb300 import workload as W
    inp = W.config("c2_512atoms", scale=0.12, seed=21)
    pab = torch.tensor(W.density_blocks(inp), device="cuda")
    V = [torch.tensor(v, device="cuda") for v in W.potential_grids(inp)]
    grids = [torch.empty(n, dtype=torch.float64, device="cuda") for n in inp.grid_sizes()]
    hab = torch.empty(inp.buffer_size, dtype=torch.float64, device="cuda")
    tl = G.GridTaskList(inp, precision=G.MIXED)
    X, T, ok = CM.collect_timings(tl, pab, V, grids, hab, steps=2)
    assert ok.sum() > 0.5 * inp.ntasks and np.all(np.isfinite(T))
    f = tl.task_features()
    assert np.all(f[:, 0] >= 0) and np.all(f[:, 2] > 0)
    rng = np.random.default_rng(0)
    perm = rng.permutation(len(T))
    ntr = int(0.8 * len(T))
    m = CM.CostModel(seed=2)
    hist = m.train(X[perm[:ntr]], T[perm[:ntr]], epochs=15, batch=1024,
                   X_val=X[perm[ntr:]], T_val=T[perm[ntr:]])
    assert hist[-1][2] < 0.5 * float(np.var(T))
    tl.collocate_device(100, pab, grids)
    tl.integrate_device(V, hab)
    torch.cuda.synchronize()
    rho_size = [g.clone() for g in grids]
    hab_size = hab.clone()
    m.apply(tl)
    tl.collocate_device(100, pab, grids)
    tl.integrate_device(V, hab)
    torch.cuda.synchronize()
    for a, b in zip(grids, rho_size):
        assert float((a - b).abs().max()) <= 1e-12 * max(1.0, float(b.abs().max()))
    assert float((hab - hab_size).abs().max()) <= 1e-12 * max(1.0, float(hab_size.abs().max()))
    tl.close()


def test_model_beats_size_cost_prediction(CM):
    """The learned model's gain over the analytic size cost: on held-out
    tasks it predicts log(task time) with a lower mean squared error than
    the size cost's best affine fit in log space (fitted on the same
    training tasks), and ranks the tasks at least as well."""
    import torch
    from cp2k_gb300 import grid as G
    from cp2k_gb300 import workload as W
    from cp2k_gb300.costmodel_eval import size_cost, spearman
    inp = W.config("c2_512atoms", scale=0.25, seed=23)
    pab = torch.tensor(W.density_blocks(inp), device="cuda")
    V = [torch.tensor(v, device="cuda") for v in W.potential_grids(inp)]
    grids = [torch.empty(n, dtype=torch.float64, device="cuda") for n in inp.grid_sizes()]
    hab = torch.empty(inp.buffer_size, dtype=torch.float64, device="cuda")
    tl = G.GridTaskList(inp, precision=G.MIXED)
    tl.collocate_device(100, pab, grids)
    tl.integrate_device(V, hab)
    X, T, ok = CM.collect_timings(tl, pab, V, grids, hab, steps=2)
    pts, lp = tl.sizes()
    S = np.log(size_cost(pts, lp)[ok])
    rng = np.random.default_rng(1)
    perm = rng.permutation(len(T))
    ntr = int(0.8 * len(T))
    tr, va = perm[:ntr], perm[ntr:]
    m = CM.CostModel(seed=3)
    m.train(X[tr], T[tr], epochs=30, batch=1024)
    pred = m.predict(X[va])
    mse_model = float(np.mean((pred - T[va]) ** 2))
    A = np.vstack([S[tr], np.ones(ntr)]).T
    coef = np.linalg.lstsq(A, T[tr], rcond=None)[0]
    mse_size = float(np.mean((coef[0] * S[va] + coef[1] - T[va]) ** 2))
    assert mse_model < mse_size, (mse_model, mse_size)
    assert spearman(pred, T[va]) >= spearman(S[va], T[va]) - 0.01
    tl.close()


def test_launch_timings_cover_all_tasks(CM):
    import torch
    from cp2k_gb300 import grid as G
    from cp2k_gb300 import workload as W
    inp = W.config("c1_64atoms", scale=0.3, seed=4)
    pab = torch.tensor(W.density_blocks(inp), device="cuda")
    grids = [torch.empty(n, dtype=torch.float64, device="cuda") for n in inp.grid_sizes()]
    tl = G.GridTaskList(inp, precision=G.MIXED)
    tl.set_launch_timing(True)
    tl.collocate_device(100, pab, grids)
    info = tl.launch_timings()
    pts, _ = tl.sizes()
    # every task once, or (row split) its two parts, whose points add up
    assert sum(i["ntasks"] for i in info) >= int((pts > 0).sum())
    assert sum(i["points"] for i in info) == int(pts.sum())
    assert all(i["ms"] > 0 and i["blocks"] > 0 and i["warps_per_block"] >= 1 for i in info)
    tl.close()
