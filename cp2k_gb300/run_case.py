"""Run collocate + integrate steps on a synthetic configuration (device
resident), e.g. as the workload of a profiler:

    python -m cp2k_gb300.run_case --config c2_512atoms --scale 0.5 \\
        --precision mixed --steps 2

Prints the per-phase kernel times of every step.  --taskgen instead runs the
device task-list generator (and the block packing) on the configuration's
geometry.  With --compare the step is
also run in FP64 on the same inputs, and one JSON line reports the median
step times (CUDA events) of both and the errors of the chosen precision
against FP64: max relative rho (reference measure), Tr(V rho) energy per
atom, hab, forces and virial."""
import argparse
import json

import numpy as np
import torch

from . import grid as G
from . import workload as W

PRECISIONS = {"mixed": G.MIXED, "fp64": G.FP64, "fp32": G.FP32}


def _step(tl, pab, V, grids, hab, f, vir, s):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    tl.collocate_device(100, pab, grids, stream=s)
    tl.integrate_device(V, hab, pab_dev=pab if (f is not None or vir is not None) else None,
                        forces_dev=f, virial_dev=vir, stream=s)
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def _taskgen(inp, steps):
    import time
    gen = G.TaskGenerator(inp)
    ms = []
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        gen.run(inp.atom_positions)
        ms.append((time.perf_counter() - t0) * 1e3)
    a = gen.host_arrays()
    equal = all(np.array_equal(np.asarray(getattr(inp, k)).reshape(v.shape), v)
                for k, v in a.items())
    # pab blocks from a block store holding them in task-list order
    boff = torch.tensor(np.ascontiguousarray(inp.block_offsets, np.int32), device="cuda")
    sizes = np.diff(np.append(inp.block_offsets.astype(np.int64), inp.buffer_size))
    src = torch.tensor(W.density_blocks(inp), device="cuda")
    dst = torch.empty_like(src)
    G.pack_blocks(boff.to(torch.int64), boff, torch.tensor(sizes.astype(np.int32), device="cuda"),
                  src, dst)
    torch.cuda.synchronize()
    print(json.dumps({"ntasks": gen.ntasks, "nblocks": gen.nblocks, "run_ms": ms,
                      "arrays_equal_host_generator": bool(equal),
                      "pack_equal": bool(torch.equal(src, dst))}), flush=True)
    gen.free()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2_512atoms", choices=sorted(W.CONFIGS))
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--precision", default="mixed", choices=sorted(PRECISIONS))
    ap.add_argument("--threshold", type=float, default=None,
                    help="mixed path: contribution bound below which tasks run in FP32")
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--no-row-split", action="store_true",
                    help="mixed mode: keep every double-float task whole")
    ap.add_argument("--forces", action="store_true")
    ap.add_argument("--virial", action="store_true")
    ap.add_argument("--transform", type=int, default=-1, choices=[-1, 0, 1],
                    help="C_ab <-> C_xyz transform: 0 direct, 1 staged, -1 staged forward")
    ap.add_argument("--compare", action="store_true",
                    help="also run FP64 and print times and errors as one JSON line")
    ap.add_argument("--taskgen", action="store_true",
                    help="generate the task list on the device --steps times (and pack the "
                         "pab blocks once), check it against the host generator, print times")
    args = ap.parse_args()
    inp = W.config(args.config, scale=args.scale)
    if args.taskgen:
        _taskgen(inp, args.steps)
        return
    pab = torch.tensor(W.density_blocks(inp), device="cuda")
    V = [torch.tensor(v, device="cuda") for v in W.potential_grids(inp)]
    grids = [torch.empty(n, dtype=torch.float64, device="cuda") for n in inp.grid_sizes()]
    hab = torch.empty(inp.buffer_size, dtype=torch.float64, device="cuda")
    f = torch.empty((inp.natoms, 3), dtype=torch.float64, device="cuda") if args.forces else None
    vir = torch.empty((3, 3), dtype=torch.float64, device="cuda") if args.virial else None
    tl = G.GridTaskList(inp, precision=PRECISIONS[args.precision])
    if args.threshold is not None:
        tl.set_mixed_threshold(args.threshold)
    tl.set_transform_variant(args.transform)
    tl.set_row_split(not args.no_row_split)
    s = torch.cuda.current_stream()
    if not args.compare:
        for step in range(args.steps):
            tl.collocate_device(100, pab, grids, stream=s)
            tc = tl.timings()
            tl.integrate_device(V, hab, pab_dev=pab if (f is not None or vir is not None) else None,
                                forces_dev=f, virial_dev=vir, stream=s)
            ti = tl.timings()
            print(f"step {step}: ntasks {inp.ntasks} collocate {tc} integrate {ti}", flush=True)
        torch.cuda.synchronize()
        tl.close()
        return

    res = {"config": args.config, "scale": args.scale, "ntasks": inp.ntasks,
           "precision": args.precision, "forces": args.forces, "virial": args.virial,
           "transform": args.transform}
    out = {}
    for name, prec in (("fp64", G.FP64), (args.precision, PRECISIONS[args.precision])):
        tl.set_precision(prec)
        _step(tl, pab, V, grids, hab, f, vir, s)  # warm-up
        ms = [_step(tl, pab, V, grids, hab, f, vir, s) for _ in range(max(1, args.steps))]
        out[name] = ([g.clone() for g in grids], hab.clone(),
                     f.clone() if f is not None else None, vir.clone() if vir is not None else None)
        res[f"{name}_ms"] = float(np.median(ms))
    rho64, hab64, f64, v64 = out["fp64"]
    rho, habx, fx, vx = out[args.precision]
    dvol = [abs(float(np.linalg.det(d))) for d in inp.dh]
    energy = lambda r: sum(float((g * v).sum()) * dv for g, v, dv in zip(r, V, dvol))
    rel = lambda a, b: float((a - b).abs().max()) / max(1.0, float(b.abs().max()))
    res["speedup"] = res["fp64_ms"] / res[f"{args.precision}_ms"]
    res["errors"] = {
        "rho_max_rel_ref_measure": max(
            float(((a - b).abs() / b.abs().clamp(min=1.0)).max()) for a, b in zip(rho, rho64)),
        "energy_ha_per_atom": abs(energy(rho) - energy(rho64)) / inp.natoms,
        "hab_max_rel": rel(habx, hab64),
    }
    if f is not None:
        res["errors"]["forces_max_rel"] = rel(fx, f64)
    if vir is not None:
        res["errors"]["virial_max_rel"] = rel(vx, v64)
    if args.precision == "mixed":
        res["fp32_share_tasks"], res["fp32_share_points"] = tl.mixed_split()
        res["row_split_tasks"], res["fp32_share_points_row_split"] = tl.row_split_stats()
    print(json.dumps(res), flush=True)
    tl.close()


if __name__ == "__main__":
    main()
