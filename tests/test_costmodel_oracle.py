"""CPU checks of the float64 restatement of the task-cost MLP (the oracle
the GPU cost-model kernels are tested against): its analytic gradient
against central finite differences, and Adam's first step."""
import numpy as np

from oracle import mlp_oracle as M


def _setup(n=37, seed=3):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.3, M.NPARAMS)
    x = rng.normal(0, 1, (n, M.NIN))
    t = rng.normal(0, 1, n)
    return p, x, t


def test_gradient_matches_finite_differences():
    p, x, t = _setup()
    _, g = M.loss_grad(p, x, t)
    rng = np.random.default_rng(0)
    # a sample of every block of the layout, plus both biases of the output
    idx = np.concatenate([rng.choice(np.arange(a, b), 12, replace=False) for a, b in (
        (M.O_W1, M.O_B1), (M.O_B1, M.O_W2), (M.O_W2, M.O_B2), (M.O_B2, M.O_W3),
        (M.O_W3, M.O_B3))] + [[M.O_B3]])
    fd = M.finite_difference_grad(p, x, t, idx)
    assert np.max(np.abs(fd - g[idx])) <= 1e-7 * max(1.0, np.max(np.abs(g[idx])))


def test_adam_first_step_is_signed_lr():
    p, x, t = _setup()
    _, g = M.loss_grad(p, x, t)
    p1, m, v = M.adam(p, g, np.zeros_like(p), np.zeros_like(p), 1, 1e-3, eps=0.0)
    nz = g != 0
    assert np.allclose((p - p1)[nz], 1e-3 * np.sign(g[nz]))


def test_predict_normalisation():
    p, x, _ = _setup()
    norm = np.concatenate([x.mean(0), x.std(0)])
    y1 = M.predict(p, x, norm)
    y2 = M.forward(p, (x - x.mean(0)) / x.std(0))[0]
    assert np.allclose(y1, y2)
