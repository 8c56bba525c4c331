"""Run collocate + integrate steps on a synthetic configuration (device
resident), e.g. as the workload of a profiler:

    python -m cp2k_gb300.run_case --config c2_512atoms --scale 0.5 \\
        --precision mixed --steps 2

Prints the per-phase kernel times of every step."""
import argparse

import torch

from . import grid as G
from . import workload as W


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2_512atoms", choices=sorted(W.CONFIGS))
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed", "fp32"])
    ap.add_argument("--threshold", type=float, default=None,
                    help="mixed path: contribution bound below which tasks run in FP32")
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--forces", action="store_true")
    args = ap.parse_args()
    inp = W.config(args.config, scale=args.scale)
    pab = torch.tensor(W.density_blocks(inp), device="cuda")
    V = [torch.tensor(v, device="cuda") for v in W.potential_grids(inp)]
    grids = [torch.empty(n, dtype=torch.float64, device="cuda") for n in inp.grid_sizes()]
    hab = torch.empty(inp.buffer_size, dtype=torch.float64, device="cuda")
    f = torch.empty((inp.natoms, 3), dtype=torch.float64, device="cuda") if args.forces else None
    tl = G.GridTaskList(inp, precision={"mixed": G.MIXED, "fp64": G.FP64,
                                        "fp32": G.FP32}[args.precision])
    if args.threshold is not None:
        tl.set_mixed_threshold(args.threshold)
    s = torch.cuda.current_stream()
    for step in range(args.steps):
        tl.collocate_device(100, pab, grids, stream=s)
        tc = tl.timings()
        tl.integrate_device(V, hab, pab_dev=pab if f is not None else None, forces_dev=f,
                            stream=s)
        ti = tl.timings()
        print(f"step {step}: ntasks {inp.ntasks} collocate {tc} integrate {ti}", flush=True)
    torch.cuda.synchronize()
    tl.close()


if __name__ == "__main__":
    main()
