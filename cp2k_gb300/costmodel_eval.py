"""Train the task-cost model on recorded per-task timings of the 512-, 1024-
and 2048-atom workloads and compare its schedule with the analytic size
schedule:

    python -m cp2k_gb300.costmodel_eval --samples 200000 \\
        --save cp2k_gb300/costmodel_gb300.npz --json out.json

1. For each workload the mixed-precision SCF step (collocate GRID_FUNC_AB +
   integrate hab) runs with per-task cycle recording; features and
   log(cycles) of every task are kept.
2. `--samples` tasks drawn at random (seeded) from all three workloads form
   the data set, split 80/20 into training and validation.
3. The MLP is trained on the device (library kernels, Adam).
4. Prediction quality on the validation tasks: mean squared error of log
   time and rank correlation with the measured times, next to the same
   figures for the analytic size cost (best affine fit in log space).
5. Each workload's SCF step is timed with the size schedule and with the
   model schedule (CUDA events, L2 flushed between steps), and the results of
   both are compared."""
import argparse
import json
import time

import numpy as np

WORKLOADS = ("c2_512atoms", "c4_1024atoms", "c4_2048atoms")


def _rank(a):
    r = np.empty(len(a))
    r[np.argsort(a, kind="stable")] = np.arange(len(a))
    return r


def spearman(a, b) -> float:
    return float(np.corrcoef(_rank(a), _rank(b))[0, 1])


def size_cost(pts, lp):
    return pts.astype(np.float64) * (lp + 1) + 64.0 * (lp + 1) * (lp + 2)


class Workload:
    def __init__(self, name, torch, G, W, seed=1):
        self.name = name
        self.inp = W.config(name, seed=seed)
        self.pab = torch.tensor(W.density_blocks(self.inp), device="cuda")
        self.V = [torch.tensor(v, device="cuda") for v in W.potential_grids(self.inp)]
        self.grids = [torch.empty(n, dtype=torch.float64, device="cuda")
                      for n in self.inp.grid_sizes()]
        self.hab = torch.empty(self.inp.buffer_size, dtype=torch.float64, device="cuda")
        self.tl = G.GridTaskList(self.inp, precision=G.MIXED)

    def step_ms(self, torch, flush, steps=5):
        s = torch.cuda.current_stream()
        out = []
        for _ in range(steps + 1):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            self.tl.collocate_device(100, self.pab, self.grids, stream=s)
            self.tl.integrate_device(self.V, self.hab, stream=s)
            e1.record(s)
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1))
        return float(np.median(out[1:]))


def main():
    import torch

    from . import costmodel as CM
    from . import grid as G
    from . import workload as W

    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=200000)
    ap.add_argument("--steps", type=int, default=2, help="timing passes per workload")
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--workloads", default=",".join(WORKLOADS))
    ap.add_argument("--save", default=None, help="write the trained model (npz) here")
    ap.add_argument("--json", default=None, help="write the evaluation (JSON) here")
    args = ap.parse_args()

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    wl = []
    Xs, Ts, Ss, tags = [], [], [], []
    for i, name in enumerate(args.workloads.split(",")):
        w = Workload(name, torch, G, W)
        w.tl.collocate_device(100, w.pab, w.grids)  # warm-up
        w.tl.integrate_device(w.V, w.hab)
        X, T, ok = CM.collect_timings(w.tl, w.pab, w.V, w.grids, w.hab, steps=args.steps)
        pts, lp = w.tl.sizes()
        Xs.append(X)
        Ts.append(T)
        Ss.append(np.log(size_cost(pts, lp)[ok]))
        tags.append(np.full(len(T), i))
        wl.append(w)
        print(f"{name}: {w.inp.ntasks} tasks, {len(T)} timed", flush=True)
    X = np.concatenate(Xs)
    T = np.concatenate(Ts)
    S = np.concatenate(Ss)
    rng = np.random.default_rng(args.seed)
    pick = rng.choice(len(T), size=min(args.samples, len(T)), replace=False)
    ntr = int(0.8 * len(pick))
    tr, va = pick[:ntr], pick[ntr:]

    model = CM.CostModel(seed=args.seed)
    t0 = time.time()
    hist = model.train(X[tr], T[tr], epochs=args.epochs, X_val=X[va], T_val=T[va],
                       seed=args.seed)
    train_s = time.time() - t0
    pred = model.predict(X[va])
    mse_model = float(np.mean((pred - T[va]) ** 2))
    # the size cost's best affine fit in log space (fitted on the training set)
    A = np.vstack([S[tr], np.ones(ntr)]).T
    coef = np.linalg.lstsq(A, T[tr], rcond=None)[0]
    mse_size = float(np.mean((coef[0] * S[va] + coef[1] - T[va]) ** 2))
    res = {
        "samples": int(len(pick)), "train": int(ntr), "validation": int(len(va)),
        "epochs": args.epochs, "train_seconds": train_s,
        "target_variance": float(np.var(T[va])),
        "val_mse_log_time": {"model": mse_model, "size_cost_affine": mse_size},
        "val_spearman": {"model": spearman(pred, T[va]), "size_cost": spearman(S[va], T[va])},
        "loss_history": [[e, a, b] for e, a, b in hist[:: max(1, len(hist) // 12)]],
        "schedules": {},
    }
    for w in wl:
        w.tl.set_schedule(G.SCHEDULE_SIZE)
        ms_size = w.step_ms(torch, flush)
        rho = [g.clone() for g in w.grids]
        hab = w.hab.clone()
        model.apply(w.tl)
        ms_model = w.step_ms(torch, flush)
        drho = max(float((a - b).abs().max()) / max(1.0, float(b.abs().max()))
                   for a, b in zip(w.grids, rho))
        dhab = float((w.hab - hab).abs().max()) / max(1.0, float(hab.abs().max()))
        res["schedules"][w.name] = {"ntasks": w.inp.ntasks, "size_ms": ms_size,
                                    "model_ms": ms_model, "gain": ms_size / ms_model - 1.0,
                                    "rho_max_rel_diff": drho, "hab_max_rel_diff": dhab}
        print(w.name, res["schedules"][w.name], flush=True)
        w.tl.close()
    print(json.dumps(res), flush=True)
    if args.json:
        with open(args.json, "w") as f:
            json.dump(res, f, indent=1)
    if args.save:
        with open(args.save, "wb") as f:
            f.write(model.to_bytes())


if __name__ == "__main__":
    main()
