"""TEST INFRASTRUCTURE ONLY: float64 numpy restatement of the task-cost MLP
(6 -> 64 -> 64 -> 1, SiLU, mean-squared-error loss, Adam) that the CUDA
kernels in cp2k_gb300/csrc/mlp_kernels.cu implement in FP32.  Used by the
tests to check the device loss, gradient, optimiser step and predictions.
The model is this project's own (CP2K has no learned scheduler), so there is
no reference implementation to pin against; the gradient here is itself
checked by central finite differences in the tests.

Parameter layout (flat): W1[64][6] b1[64] W2[64][64] b2[64] w3[64] b3."""
import numpy as np

NIN, NH = 6, 64
O_W1 = 0
O_B1 = O_W1 + NH * NIN
O_W2 = O_B1 + NH
O_B2 = O_W2 + NH * NH
O_W3 = O_B2 + NH
O_B3 = O_W3 + NH
NPARAMS = O_B3 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[O_W1:O_B1].reshape(NH, NIN), p[O_B1:O_W2], p[O_W2:O_B2].reshape(NH, NH),
            p[O_B2:O_W3], p[O_W3:O_B3], p[O_B3])


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def forward(p, x):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ W1.T + b1
    h1 = z1 * _sig(z1)
    z2 = h1 @ W2.T + b2
    h2 = z2 * _sig(z2)
    y = h2 @ w3 + b3
    return y, (x, z1, h1, z2, h2)


def predict(p, x, norm=None):
    x = np.asarray(x, dtype=np.float64)
    if norm is not None:
        norm = np.asarray(norm, dtype=np.float64)
        x = (x - norm[:NIN]) / norm[NIN:]
    return forward(p, x)[0]


def loss_grad(p, x, t):
    """Mean squared error and its gradient with respect to the flat
    parameters (chain rule through the two SiLU layers)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    y, (x, z1, h1, z2, h2) = forward(p, x)
    n = len(y)
    r = y - np.asarray(t, dtype=np.float64)
    loss = float((r * r).sum() / n)
    g = 2.0 * r / n
    ds = lambda z: _sig(z) * (1.0 + z * (1.0 - _sig(z)))
    dw3 = h2.T @ g
    db3 = g.sum()
    dz2 = np.outer(g, w3) * ds(z2)
    dW2 = dz2.T @ h1
    db2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * ds(z1)
    dW1 = dz1.T @ x
    db1 = dz1.sum(0)
    grad = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dw3, [db3]])
    return loss, grad


def adam(p, grad, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def finite_difference_grad(p, x, t, idx, h=1e-6):
    p = np.asarray(p, dtype=np.float64)
    out = []
    for i in idx:
        a, b = p.copy(), p.copy()
        a[i] += h
        b[i] -= h
        out.append((loss_grad(a, x, t)[0] - loss_grad(b, x, t)[0]) / (2 * h))
    return np.array(out)
