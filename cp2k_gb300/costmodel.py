"""Learned task-cost model of the persistent grid kernels.

The persistent collocate/integrate kernels take tasks from cost-ordered work
queues (longest first), so the last warps to finish determine the tail of
each launch.  The default order uses an analytic size (points x (lp+1)); this
module trains a 6 -> 64 -> 64 -> 1 MLP (SiLU, FP32) on per-task timings that
the kernels themselves record (clock64 cycles per task) and hands its
predictions to the task list for GRID_GB300_SCHEDULE_MODEL.

Training, gradients, the Adam update and inference all run in the library's
hand-written CUDA kernels (cp2k_gb300/csrc/mlp_kernels.cu) through its C
ABI; torch only provides device memory and streams.

Features per task (grid_gb300_task_features): la_max, lb_max, zeta_a+zeta_b,
cube radius in grid points, level grid spacing (bohr), cell skew.  Target:
log(collocate cycles + integrate cycles) of the task in one SCF step."""
import ctypes as C
import io

import numpy as np

from . import grid as G

NIN = 6
FEATURES = ("la_max", "lb_max", "zeta_sum", "cube_radius_points", "level_spacing_bohr",
            "cell_skew")


def nparams() -> int:
    return int(G.lib().grid_gb300_cost_model_nparams())


def init_params(seed: int = 0) -> np.ndarray:
    """Uniform fan-in initialisation (variance 2/fan_in: suits SiLU)."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((NIN, 64), (64, 64), (64, 1)):
        lim = np.sqrt(6.0 / fan_in)
        w = rng.uniform(-lim, lim, size=(fan_out, fan_in))
        parts += [w.ravel(), np.zeros(fan_out)]
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == nparams()
    return p


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _stream(torch, stream):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class CostModel:
    """Parameters and feature normalisation on the device, training and
    inference through the library's CUDA kernels."""

    def __init__(self, params=None, norm=None, seed: int = 0, device="cuda"):
        import torch
        self.torch = torch
        self.device = torch.device(device)
        p = init_params(seed) if params is None else np.asarray(params, np.float32)
        self.params = torch.tensor(p, dtype=torch.float32, device=self.device)
        n = np.concatenate([np.zeros(NIN), np.ones(NIN)]) if norm is None else norm
        self.norm = torch.tensor(np.asarray(n, np.float32), device=self.device)
        self.history = []

    # ------------------------------------------------------------- training
    def fit_norm(self, X: np.ndarray):
        """Standardise each feature by its mean and spread (constant
        features, e.g. the skew of an orthorhombic cell, keep scale 1)."""
        X = np.asarray(X, np.float64)
        mean = X.mean(0)
        std = X.std(0)
        std[std < 1e-6] = 1.0
        self.norm = self.torch.tensor(np.concatenate([mean, std]).astype(np.float32),
                                      device=self.device)

    def standardise(self, X: np.ndarray) -> np.ndarray:
        n = self.norm.cpu().numpy().astype(np.float64)
        return ((np.asarray(X, np.float64) - n[:NIN]) / n[NIN:]).astype(np.float32)

    def loss_grad(self, Xs, T, stream=None):
        """Loss and gradient on device tensors Xs [n][6] (standardised) and
        T [n]; returns (loss tensor [1], grad tensor [nparams])."""
        torch = self.torch
        n = int(Xs.shape[0])
        work = torch.empty(int(G.lib().grid_gb300_cost_model_work_floats(n)),
                           dtype=torch.float32, device=self.device)
        loss = torch.empty(1, dtype=torch.float32, device=self.device)
        grad = torch.empty_like(self.params)
        G.lib().grid_gb300_cost_model_loss_grad(_ptr(self.params), _ptr(Xs), _ptr(T), n,
                                                _ptr(loss), _ptr(grad), _ptr(work),
                                                _stream(torch, stream))
        return loss, grad

    def train(self, X: np.ndarray, T: np.ndarray, epochs: int = 60, batch: int = 2048,
              lr: float = 3e-3, lr_final: float = 3e-4, seed: int = 0, X_val=None, T_val=None,
              fit_norm: bool = True):
        """Minibatch Adam on the device.  X raw features [n][6], T targets
        (log time).  Learning rate decays geometrically from lr to lr_final.
        Returns the history of (epoch, train loss, validation loss)."""
        torch = self.torch
        if fit_norm:
            self.fit_norm(X)
        Xd = torch.tensor(self.standardise(X), device=self.device)
        Td = torch.tensor(np.asarray(T, np.float32), device=self.device)
        Xv = Tv = None
        if X_val is not None:
            Xv = torch.tensor(self.standardise(X_val), device=self.device)
            Tv = torch.tensor(np.asarray(T_val, np.float32), device=self.device)
        n = Xd.shape[0]
        m = torch.zeros_like(self.params)
        v = torch.zeros_like(self.params)
        gen = torch.Generator(device="cpu")
        gen.manual_seed(seed)
        nb = max(1, n // batch)
        total = epochs * nb
        step = 0
        L = G.lib()
        stream = torch.cuda.current_stream()
        work = torch.empty(int(L.grid_gb300_cost_model_work_floats(batch)), dtype=torch.float32,
                           device=self.device)
        loss = torch.empty(1, dtype=torch.float32, device=self.device)
        grad = torch.empty_like(self.params)
        for ep in range(epochs):
            perm = torch.randperm(n, generator=gen).to(self.device)
            tl = 0.0
            for b in range(nb):
                idx = perm[b * batch:(b + 1) * batch]
                xb = Xd.index_select(0, idx).contiguous()
                tb = Td.index_select(0, idx).contiguous()
                step += 1
                rate = lr * (lr_final / lr) ** ((step - 1) / max(total - 1, 1))
                L.grid_gb300_cost_model_loss_grad(_ptr(self.params), _ptr(xb), _ptr(tb),
                                                  int(xb.shape[0]), _ptr(loss), _ptr(grad),
                                                  _ptr(work), _stream(torch, stream))
                L.grid_gb300_cost_model_adam(_ptr(self.params), _ptr(grad), _ptr(m), _ptr(v),
                                             step, rate, 0.9, 0.999, 1e-8,
                                             _stream(torch, stream))
                tl += float(loss.item()) if b == nb - 1 else 0.0
            vl = None
            if Xv is not None:
                vl = float(self.loss_grad(Xv, Tv)[0].item())
            self.history.append((ep, tl, vl))
        return self.history

    # ------------------------------------------------------------ inference
    def predict(self, X: np.ndarray, stream=None) -> np.ndarray:
        """Predicted log time for raw features X [n][6]."""
        torch = self.torch
        Xd = torch.tensor(np.ascontiguousarray(X, np.float32), device=self.device)
        y = torch.empty(Xd.shape[0], dtype=torch.float32, device=self.device)
        G.lib().grid_gb300_cost_model_predict(_ptr(self.params), _ptr(Xd), int(Xd.shape[0]),
                                              _ptr(self.norm), _ptr(y), _stream(torch, stream))
        return y.cpu().numpy()

    def apply(self, tl: "G.GridTaskList", stream=None):
        """Predict every task of the list on the device and schedule by it."""
        G.lib().grid_gb300_apply_cost_model(tl.impl, _ptr(self.params), _ptr(self.norm),
                                            _stream(self.torch, stream))
        tl.set_schedule(G.SCHEDULE_MODEL)

    # ------------------------------------------------------------ storage
    def to_bytes(self) -> bytes:
        b = io.BytesIO()
        np.savez(b, params=self.params.cpu().numpy(), norm=self.norm.cpu().numpy())
        return b.getvalue()

    @classmethod
    def from_bytes(cls, data: bytes, device="cuda"):
        z = np.load(io.BytesIO(data))
        return cls(params=z["params"], norm=z["norm"], device=device)


def collect_timings(tl: "G.GridTaskList", pab_dev, V_dev, grids_dev, hab_dev, steps: int = 1,
                    func: int = 100, stream=None):
    """Runs `steps` SCF steps (collocate + integrate) with per-task timing and
    returns (features [n][6], log cycles [n]) for the tasks that ran, the
    cycles summed over both calls and averaged over the steps."""
    import torch
    tl.set_task_timing(True)
    cyc = np.zeros(tl.inp.ntasks, np.float64)
    for _ in range(steps):
        tl.collocate_device(func, pab_dev, grids_dev, stream=stream)
        torch.cuda.synchronize()
        cyc += tl.task_cycles()
        tl.integrate_device(V_dev, hab_dev, stream=stream)
        torch.cuda.synchronize()
        cyc += tl.task_cycles()
    tl.set_task_timing(False)
    f = tl.task_features()
    ok = cyc > 0
    return f[ok], np.log(cyc[ok] / steps).astype(np.float32), ok
