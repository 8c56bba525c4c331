"""Benchmark: collocate + integrate per SCF step on one GB300, mixed vs FP64.

Workload: the 512-atom water-like box (24.8 A cubic, O:H 1:2, O 3 sets up to
l=2 and H 2 sets up to l=1, two primitives per set, exponents log-uniform in
[0.04, 40] bohr^-2, 5 grid levels 216^3 .. 54^3, ~3.8e5 tasks), seeded
synthetic data.  One step = grid_collocate_task_list(GRID_FUNC_AB) +
grid_integrate_task_list (hab only), as one SCF iteration does.

  value      mixed-precision ms per step, device-resident buffers, CUDA events
             on the launching stream, L2 flushed between steps;
  e2e        the same step through the CP2K C ABI with host offload buffers
             (H2D pab + V grids, D2H rho grids + hab inside the timed region);
  fp64_*     the plain FP64 path timed the same way;
  errors     mixed / FP64 / FP32 against the oracle's FP64 results on the
             same inputs (and mixed against the FP64 path);
  roofline   the dominant grid kernel of the mixed step (largest total time
             from per-launch CUDA events; the tensor-core FP32-class
             integrate) against the measured HBM roof, and its algorithmic
             flops against the CUDA-core FMA roof (roofline_fp32);
             roofline_fp64 the same for the FP64 step;
  mixed_no_row_split / mixed_model_schedule / mixed_one_queue_stream
             the mixed step with one feature switched back (diagnostics);
  hartree_step_on_device  collocate -> plane waves -> Hartree potential ->
             level grids -> integrate, every buffer on the device;
  task_generation  the geometry's task list generated on the device against
             the host generator (time, equality), the task list created from
             it, and the pab blocks packed from / added back to a block store
             on the device (GB/s against the measured HBM roof);
  cpu_baseline  whole SCF steps of the oracle (FP64 C restatement of CP2K's
             REF backend) on all host cores;
  triclinic_256atoms_forces_virial, c5_6144atoms_forces
             the other workloads' mixed and FP64 steps with forces (and
             virial), errors against the oracle, the oracle's step time and
             the task-list creation time (--no-secondary skips them).

--impl reference times whole SCF steps of the reference's CPU implementation
of the path (the oracle port, all host threads) on the same workload and
prints the same metric.  Under torchrun every rank runs an independent replica
(the path has no data exchange on one GPU); rank 0 prints the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "collocate+integrate ms per SCF step, mixed vs FP64, 1 GB300, stated error"
WORKLOAD = "c2_512atoms"
CONFIG = {
    "workload": "512-atom water-like box, 24.8 A cubic, 5 levels 216^3..54^3, "
                "O 3 sets l<=2 / H 2 sets l<=1, 2 primitives per set, zeta in [0.04, 40]",
    "step": "collocate(GRID_FUNC_AB) + integrate(hab)",
    "seed": 1,
    "l2": "flushed (256 MiB write) between timed steps; pab buffer 468 MB > L2",
}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# --------------------------------------------------------------------------
# CPU baseline: whole SCF steps of the oracle
# --------------------------------------------------------------------------
def oracle_steps(inp, pab, V, nsteps: int, warmup: int = 0, forces: bool = False,
                 virial: bool = False):
    """Times whole SCF steps (collocate GRID_FUNC_AB + integrate) of the oracle
    -- the FP64 C restatement of CP2K's REF backend -- on all host threads.
    Task-list creation is outside the timed region, as it is for the GPU.
    Returns (ms per step list, rho, hab, forces, virial) of the last step."""
    from oracle import oracle as O

    ot = O.OracleTaskList(inp)
    times, out = [], None
    for i in range(warmup + nsteps):
        t0 = time.perf_counter()
        rho = ot.collocate(100, pab)
        hab, f, v = ot.integrate(V, pab if (forces or virial) else None, forces=forces,
                                 virial=virial)
        dt = (time.perf_counter() - t0) * 1e3
        if i >= warmup:
            times.append(dt)
        out = (rho, hab, f, v)
    ot.close()
    return times, out


def host_threads() -> int:
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def reference_arm(args, world, rank):
    if rank != 0:
        return
    from cp2k_gb300 import build
    from cp2k_gb300 import workload as W

    build.build_workload()
    inp = W.config(WORKLOAD)
    pab = W.density_blocks(inp)
    V = W.potential_grids(inp)
    times, _ = oracle_steps(inp, pab, V, args.steps, args.warmup)
    v = float(np.mean(times))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "ms",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": v, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": CONFIG,
        "cpu_baseline": {"value": v, "unit": "ms", "cores": host_threads(), "kind": "port",
                         "sample": f"{args.steps} whole SCF steps of the workload ({inp.ntasks} "
                                   f"tasks each), mean; oracle = C restatement of CP2K's REF "
                                   f"backend (CP2K's own CPU backend cannot be built on the GPU "
                                   f"host: its sources are not there)"},
        "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def measure_peak(torch, dtype, n):
    """cuBLAS GEMM throughput (TFLOP/s) in `dtype` with TF32 off: the CUDA-core
    FP32 FMA peak (float32) or the FP64 peak (float64) of this GPU."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(n, n, device="cuda", dtype=dtype)
    b = torch.randn(n, n, device="cuda", dtype=dtype)
    for _ in range(2):
        torch.mm(a, b)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(3):
        e0.record()
        torch.mm(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b
    return best


# DRAM bytes per SCF step (dram__bytes_read.sum + dram__bytes_write.sum over
# the kernel's launches of one step) of the dominant kernels of the 512-atom
# mixed and FP64 steps, from one ncu capture of this workload at the default
# launch split; the bench cannot run ncu itself, and divides by its own
# launches per step.  Keys: kernel label as in "roofline.kernel".
NCU_TRAFFIC_PER_STEP = {
    "integrate_ortho_tc<4>": (2.628 + 0.021 + 26.141 + 0.091 + 167.054 + 42.108
                              + 112.559 + 15.697) * 1e6,
    "collocate_ortho<float,4>": (3.369 + 0.040 + 33.993 + 8.245 + 263.428 + 1072.301
                                 + 145.123 + 406.260) * 1e6,
    "integrate_ortho<double,4>": ((35.777 + 0.760) + (594.138 + 123.159)) * 1e6,
}


def _kernel_label(info):
    prec = {0: "double", 1: "dfloat", 2: "float"}[info["precision"]]
    kind = "general" if info["general"] else "ortho"
    phase = "collocate" if info["phase"] == 0 else "integrate"
    if (info["phase"] == 1 and prec == "float" and not info["general"]
            and info["lp_bucket"] <= 6):
        # FP32-class orthorhombic integration runs on the tensor cores (default)
        return f"integrate_ortho_tc<{info['lp_bucket']}>"
    return f"{phase}_{kind}<{prec},{info['lp_bucket']}>"


def load_cost_model(torch):
    """The trained task-cost model shipped with the package (trained on this
    GPU type by cp2k_gb300.costmodel_eval), or None."""
    from cp2k_gb300 import costmodel as CM
    path = os.path.join(ROOT, "cp2k_gb300", "costmodel_gb300.npz")
    if not os.path.exists(path):
        return None, None
    with open(path, "rb") as fh:
        return CM.CostModel.from_bytes(fh.read()), os.path.relpath(path, ROOT)


def kernel_times(torch, tl, G, prec, sched, step, flush, nsteps=3):
    """Per grid-kernel launch CUDA events (recorded on the launching stream)
    over `nsteps` steps: label -> {ms: [...], points, flops, launches, phase}
    and the total visited points per phase."""
    tl.set_precision(prec)
    tl.set_schedule(sched)
    tl.set_launch_timing(True)
    per, phase_points = {}, [0.0, 0.0]
    for _ in range(nsteps):
        flush.zero_()
        torch.cuda.synchronize()
        infos = step()
        for i in infos:
            k = per.setdefault(_kernel_label(i), {"ms": [], "points": 0.0, "flops": 0.0,
                                                  "launches": 0, "phase": i["phase"]})
            k["ms"].append(i["ms"])
            k["points"] += i["points"]
            k["flops"] += i["flops"]
            k["launches"] += 1
            phase_points[i["phase"]] += i["points"]
    tl.set_launch_timing(False)
    return per, phase_points


def roofline_objects(per, phase_points, field_points, peaks, peak_kind, fp_peak, fp_kind, arith):
    """The dominant kernel (largest total time) against the HBM roof and
    against the CUDA-core FMA roof of its arithmetic.

    Algorithmic HBM bytes of a step: every grid point written once by the
    collocate phase (8 B FP64 grid, plus 4 B of FP32 low words in the mixed
    mode) or read once by the integrate phase (8 B: FP64 or hi/lo float
    pairs); a launch is charged the share of its phase's visited points that
    it visits.  Algorithmic flops of a launch: 2 (lp + 1) per visited point
    (the separable inner-loop minimum)."""
    dom = max(per, key=lambda k: sum(per[k]["ms"]))
    d = per[dom]
    avg_ms = float(np.mean(d["ms"]))
    if d["phase"] == 0:
        # FP64 grid RMW; the double-float class adds its FP32 low words
        bpp = 12.0 if (arith == "mixed" and "<dfloat" in dom) else 8.0
    else:
        # FP32 kernels of the mixed mode read the dense high words (4 B)
        bpp = 4.0 if (arith == "mixed" and ("<float" in dom or "_tc<" in dom)) else 8.0
    # the kernel's share of the phase's visited points (all its launches of
    # a step), spread over its launches per step
    share = d["points"] / max(phase_points[d["phase"]], 1.0)
    alg_bytes = bpp * field_points * share / (d["launches"] / 3.0)
    alg_flops = d["flops"] / d["launches"]
    gbs = alg_bytes / (avg_ms * 1e-3) / 1e9
    tf = alg_flops / (avg_ms * 1e-3) / 1e12
    per_step = NCU_TRAFFIC_PER_STEP.get(dom)
    traffic = per_step / (d["launches"] / 3.0) if per_step else None
    hbm = {"bound": "hbm", "achieved": gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
           "frac": gbs / peaks.get("hbm_gbs", 1.0), "traffic": traffic, "kernel": dom,
           "launch_ms": avg_ms, "launches_per_step": d["launches"] / 3.0,
           "algorithmic_bytes_per_launch": alg_bytes, "peak_kind": peak_kind,
           "binding": False}
    fma = {"bound": "fp32_fma" if arith != "fp64" else "fp64_fma", "achieved": tf,
           "peak": fp_peak, "unit": "TFLOP/s", "frac": tf / fp_peak, "peak_kind": fp_kind,
           "kernel": dom, "launch_ms": avg_ms, "flops_per_launch": alg_flops, "binding": True}
    share_k = {k: sum(v["ms"]) / sum(sum(x["ms"]) for x in per.values())
               for k, v in sorted(per.items(), key=lambda kv: -sum(kv[1]["ms"]))}
    return hbm, fma, share_k


def field_energy(rho, V, inp):
    dvol = [abs(float(np.linalg.det(d_))) for d_ in inp.dh]
    return sum(float((np.asarray(g) * np.asarray(v)).sum()) * dv for g, v, dv in zip(rho, V, dvol))


def errors_vs(rho, hab, rho_ref, hab_ref, V, inp, f=None, f_ref=None, vir=None, vir_ref=None):
    """The reference's measure max |d| / max(1, |ref|) for rho, hab, forces,
    virial; max |d| / max |rho|; Tr(V rho) energy error per atom (Ha)."""
    rel = lambda a, b: float(np.max(np.abs(np.asarray(a) - np.asarray(b))
                                    / np.maximum(1.0, np.abs(np.asarray(b)))))
    out = {
        "rho_max_rel_ref_measure": max(rel(a, b) for a, b in zip(rho, rho_ref)),
        "rho_max_abs_over_max_rho": max(float(np.abs(np.asarray(a) - np.asarray(b)).max())
                                        for a, b in zip(rho, rho_ref))
        / max(float(np.abs(np.asarray(b)).max()) for b in rho_ref),
        "energy_ha_per_atom": abs(field_energy(rho, V, inp) - field_energy(rho_ref, V, inp))
        / inp.natoms,
        "hab_max_rel": rel(hab, hab_ref),
    }
    if f is not None:
        out["forces_max_rel"] = rel(f, f_ref)
    if vir is not None:
        out["virial_max_rel"] = rel(vir, vir_ref)
    return out


def hartree_step(torch, G, tl, inp, pab, grids, hab, stream, flush, nsteps):
    """One Hartree step kept on the device, mixed mode: collocate ->
    density_rs2pw -> periodic Poisson solve -> potential_pw2rs -> integrate
    (CUDA events on the stream, L2 flushed before each step), with the share
    of the plane-wave part."""
    npts = [tuple(int(x) for x in n) for n in inp.npts_local]
    dh = np.asarray(inp.dh[0], np.float64).reshape(3, 3)
    pw = G.PwTransfer(npts)
    n0 = int(np.prod(npts[0]))
    dev = grids[0].device
    g = torch.empty(2 * n0, dtype=torch.float64, device=dev)
    tl.set_precision(G.MIXED)
    times, pw_times = [], []
    for i in range(nsteps + 1):
        flush.zero_()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            e[0].record(stream)
            tl.collocate_device(100, pab, grids, stream=stream)
            e[1].record(stream)
            pw.density_rs2pw(grids, None, g, stream=stream)
            pw.poisson(dh, g, g, stream=stream)
            pw.potential_g2rs(g, grids, stream=stream)
            e[2].record(stream)
            tl.integrate_device(grids, hab, stream=stream)
            e[3].record(stream)
        torch.cuda.synchronize()
        if i:
            times.append(e[0].elapsed_time(e[3]))
            pw_times.append(e[1].elapsed_time(e[2]))
    pw.close()
    return {"ms_per_step": float(np.mean(times)), "plane_wave_ms": float(np.mean(pw_times)),
            "steps": "collocate, density_rs2pw, Poisson (Hartree) in G space, "
                     "potential_g2rs, integrate; all buffers on the device"}


def geometry_change(torch, G, inp, gen, V, grids, stream, nsteps=3):
    """A change of geometry as an MD step makes it, mixed mode: the atoms
    moved (0.05 bohr rms), the task list generated on the device, re-created
    through its handle from the device arrays (grid_gb300_taskgen_create_
    task_list), then the first collocate + integrate (which build the work
    queues) and a second one.  Returns per-geometry means."""
    dev = grids[0].device
    cap = int(inp.buffer_size * 1.05) + 1024
    pab = torch.zeros(cap, dtype=torch.float64, device=dev)
    hab = torch.empty(cap, dtype=torch.float64, device=dev)
    rng = np.random.default_rng(5)
    pos = inp.atom_positions.copy()
    tl, rows = None, []
    for _ in range(nsteps + 1):
        pos = pos + rng.normal(scale=0.05, size=pos.shape)
        t0 = time.perf_counter()
        gen.run(pos)
        t1 = time.perf_counter()
        if gen.buffer_size > cap:
            continue
        tl = G.GridTaskList.from_generator(gen, precision=G.MIXED, existing=tl)
        steps = []
        for _k in range(2):
            torch.cuda.synchronize()
            a = time.perf_counter()
            with torch.cuda.stream(stream):
                tl.collocate_device(100, pab, grids, stream=stream)
                tl.integrate_device(V, hab, stream=stream)
            torch.cuda.synchronize()
            steps.append((time.perf_counter() - a) * 1e3)
        rows.append(((t1 - t0) * 1e3, tl.create_s * 1e3, steps[0], steps[1]))
    if tl is not None:
        tl.close()
    del pab, hab
    rows = np.array(rows[1:] if len(rows) > 1 else rows)  # the first builds the list's streams
    gen_ms, create_ms, first_ms, step_ms = (float(x) for x in rows.mean(axis=0))
    return {"geometries": int(len(rows)), "generate_ms": gen_ms, "create_task_list_ms": create_ms,
            "first_step_ms": first_ms, "step_ms": step_ms,
            "overhead_ms": gen_ms + create_ms + first_ms - step_ms,
            "timing": "wall clock; create is the C call alone; the first step builds the "
                      "work queues on the host"}


def task_generation(torch, G, inp, host_s, pab=None, flush=None, peaks=None, reps=5,
                    geom=None):
    """The workload's task list generated on the device (grid_gb300_taskgen_run:
    the screening, radii, levels and block offsets of CP2K's
    generate_qs_task_list) against the host generator's arrays, the task list
    created from it; with `pab`, the density-matrix blocks gathered on the
    device from a block store into the pab buffer (rs_pack_buffer) and added
    back (rs_unpack_buffer), against the HBM roof."""
    gen = G.TaskGenerator(inp)
    gen.run(inp.atom_positions)
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        gen.run(inp.atom_positions)
        ts.append((time.perf_counter() - t0) * 1e3)
    arrays = gen.host_arrays()
    equal = all(np.array_equal(np.asarray(getattr(inp, k)).reshape(v.shape), v)
                for k, v in arrays.items())
    t0 = time.perf_counter()
    tl2 = G.GridTaskList.from_generator(gen, precision=None, schedule=None)
    create_s = time.perf_counter() - t0
    tl2.close()
    geo = geometry_change(torch, G, inp, gen, *geom) if geom is not None else None
    gen.free()
    res = {"ntasks": inp.ntasks, "device_ms": float(np.median(ts)),
           "host_generator_s": host_s, "arrays_equal_host_generator": bool(equal),
           "create_task_list_from_device_arrays_s": create_s,
           "timing": "wall clock of the whole call (positions upload, 5 kernels, 2 reads of "
                     "the totals), median of %d" % reps}
    if geo is not None:
        res["geometry_change"] = geo
    if pab is None:
        return res
    # a block store: the task list's blocks at shuffled places in one arena
    dev = pab.device
    blk = inp.block_num_list - 1
    first = np.unique(blk, return_index=True)[1]
    nsgf = np.array([inp.basis_sets[k - 1].nsgf for k in inp.atom_kinds])
    sizes = (nsgf[inp.iatom_list[first] - 1] * nsgf[inp.jatom_list[first] - 1]).astype(np.int32)
    perm = np.random.default_rng(0).permutation(len(sizes))
    store_off = np.zeros(len(sizes), np.int64)
    store_off[perm] = np.concatenate([[0], np.cumsum(sizes[perm].astype(np.int64))[:-1]])
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device=dev)
    d_store_off, d_sizes = t(store_off), t(sizes)
    d_boff = t(np.ascontiguousarray(inp.block_offsets, np.int32))
    store = torch.zeros(int(sizes.astype(np.int64).sum()), dtype=torch.float64, device=dev)
    G.unpack_blocks(d_boff, d_store_off, d_sizes, pab, store)
    out = torch.empty_like(pab)
    moved = 8.0 * float(sizes.astype(np.int64).sum())
    for name, fn, nbytes in (
            ("pack", lambda: G.pack_blocks(d_store_off, d_boff, d_sizes, store, out), 2 * moved),
            ("unpack", lambda: G.unpack_blocks(d_boff, d_store_off, d_sizes, pab, store),
             3 * moved)):
        fn()
        times = []
        for _ in range(reps):
            flush.zero_()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            torch.cuda.synchronize()
            e[0].record()
            fn()
            e[1].record()
            torch.cuda.synchronize()
            times.append(e[0].elapsed_time(e[1]))
        ms = float(np.median(times))
        gbs = nbytes / ms * 1e-6
        res[name] = {"ms": ms, "bytes": nbytes, "gbs": gbs,
                     "frac_of_measured_hbm": gbs / peaks.get("hbm_gbs", 1.0)}
    res["pack"]["equal"] = bool(torch.equal(out, pab))
    del store, out
    torch.cuda.empty_cache()
    return res


def secondary_case(torch, G, W, name, forces, virial, nsteps, cpu_steps, flush):
    """Mixed and FP64 step times (device-resident, default launch shapes, size
    schedule) of another workload, with forces / virial as its configuration
    asks, errors against the oracle's FP64 results, the oracle's own step
    time on the host cores, and the task-list creation time."""
    dev = torch.device("cuda", torch.cuda.current_device())
    t0 = time.perf_counter()
    inp = W.config(name)
    host_gen_s = time.perf_counter() - t0
    pab_h = W.density_blocks(inp)
    V_h = W.potential_grids(inp)
    gen_s = time.perf_counter() - t0
    pab = torch.tensor(pab_h, device=dev)
    V = [torch.tensor(v, device=dev) for v in V_h]
    grids = [torch.empty(n, dtype=torch.float64, device=dev) for n in inp.grid_sizes()]
    hab = torch.empty(inp.buffer_size, dtype=torch.float64, device=dev)
    f = torch.empty((inp.natoms, 3), dtype=torch.float64, device=dev) if forces else None
    vir = torch.empty((3, 3), dtype=torch.float64, device=dev) if virial else None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tl = G.GridTaskList(inp, api="cp2k")
    torch.cuda.synchronize()
    create_s = time.perf_counter() - t0
    stream = torch.cuda.Stream(device=dev)
    res, outs = {"ntasks": inp.ntasks, "forces": forces, "virial": virial,
                 "task_list_create_s": create_s, "workload_generate_s": gen_s}, {}
    for prec, key in ((G.MIXED, "mixed"), (G.FP64, "fp64")):
        tl.set_precision(prec)
        times = []
        for i in range(1 + nsteps):
            flush.zero_()
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                e[0].record(stream)
                tl.collocate_device(100, pab, grids, stream=stream)
                tl.integrate_device(V, hab, pab_dev=pab if (forces or virial) else None,
                                    forces_dev=f, virial_dev=vir, stream=stream)
                e[1].record(stream)
            torch.cuda.synchronize()
            if i:
                times.append(e[0].elapsed_time(e[1]))
        res[f"{key}_ms_per_step"] = float(np.mean(times))
        outs[key] = ([g.cpu().numpy() for g in grids], hab.cpu().numpy(),
                     f.cpu().numpy() if f is not None else None,
                     vir.cpu().numpy() if vir is not None else None)
    res["speedup_vs_fp64"] = res["fp64_ms_per_step"] / res["mixed_ms_per_step"]
    res["task_generation"] = task_generation(torch, G, inp, host_gen_s)
    tl.close()
    del pab, V, grids, hab, f, vir
    torch.cuda.empty_cache()
    ctimes, ref = oracle_steps(inp, pab_h, V_h, cpu_steps, 0, forces=forces, virial=virial)
    res["cpu_baseline"] = {"value": float(np.mean(ctimes)), "unit": "ms", "cores": host_threads(),
                           "kind": "port", "sample": f"{cpu_steps} whole SCF step(s)"}
    for key in ("mixed", "fp64"):
        rho, h, ff, vv = outs[key]
        res[f"errors_{key}_vs_oracle"] = errors_vs(rho, h, ref[0], ref[1], V_h, inp, ff, ref[2],
                                                   vv, ref[3])
    return res


def gpu_arm(args, world, rank, local):
    import torch

    from cp2k_gb300 import grid as G
    from cp2k_gb300 import workload as W

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    t0 = time.perf_counter()
    inp = W.config(WORKLOAD)
    host_gen_s = time.perf_counter() - t0
    pab_h = W.density_blocks(inp)
    V_h = W.potential_grids(inp)
    pab = torch.tensor(pab_h, device=dev)
    V = [torch.tensor(v, device=dev) for v in V_h]
    grids = [torch.empty(n, dtype=torch.float64, device=dev) for n in inp.grid_sizes()]
    hab = torch.empty(inp.buffer_size, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tl = G.GridTaskList(inp, api="cp2k")
    torch.cuda.synchronize()
    create_s = time.perf_counter() - t0
    stream = torch.cuda.Stream(device=dev)
    model, model_path = load_cost_model(torch)
    if model is not None:
        with torch.cuda.stream(stream):
            model.apply(tl, stream=stream)
    # the size schedule is the default; the learned model's order is timed
    # beside it as a diagnostic (it gains within the run-to-run noise)
    sched_mixed = G.SCHEDULE_SIZE
    # autotuned size split and launch shapes, per precision, on this workload
    tuned = {}
    for prec, sched in ((G.MIXED, sched_mixed), (G.FP64, G.SCHEDULE_SIZE),
                        (G.FP32, sched_mixed)):
        tl.set_precision(prec)
        tl.set_schedule(sched)
        with torch.cuda.stream(stream):
            tuned[prec] = (tl.autotune(100, pab, grids, V, hab, stream=stream), tl.tuned_split())
        torch.cuda.synchronize()

    launched = [0, 0]  # kernel counter at the first timed step, launches in timed steps

    def one_step():
        with torch.cuda.stream(stream):
            tl.collocate_device(100, pab, grids, stream=stream)
        infos = tl.launch_timings()
        with torch.cuda.stream(stream):
            tl.integrate_device(V, hab, stream=stream)
        return infos + tl.launch_timings()

    def run_steps(prec, sched, nsteps, warm=1):
        # a precision or schedule switch may rebuild work queues on the host:
        # `warm` untimed steps run first so that no timed step pays for it
        tl.set_precision(prec)
        tl.set_schedule(sched)
        times = []
        for i in range(warm + nsteps):
            if i == warm:
                launched[0] = G.kernel_launches()
            flush.zero_()
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                e[0].record(stream)
                tl.collocate_device(100, pab, grids, stream=stream)
                tl.integrate_device(V, hab, stream=stream)
                e[1].record(stream)
            torch.cuda.synchronize()
            if i >= warm:
                times.append(e[0].elapsed_time(e[1]))
        launched[1] = G.kernel_launches() - launched[0]
        return times

    # warm-up all paths, then the timed regions
    run_steps(G.MIXED, sched_mixed, args.warmup)
    if model is not None:
        run_steps(G.MIXED, G.SCHEDULE_MODEL, max(1, min(args.warmup, 2)))
    run_steps(G.FP64, G.SCHEDULE_SIZE, max(1, min(args.warmup, 2)))
    run_steps(G.FP32, sched_mixed, max(1, min(args.warmup, 2)))
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        torch.cuda.nvtx.range_push("timed_mixed")  # lets a profiler select this region
        t_mixed = run_steps(G.MIXED, sched_mixed, args.steps)
        torch.cuda.nvtx.range_pop()
    launches = launched[1]
    torch.cuda.synchronize()
    barrier(world)
    rho_mixed = [g.cpu().numpy() for g in grids]
    hab_mixed = hab.cpu().numpy()
    # the same step replayed as one CUDA graph
    graph = tl.capture_step(100, pab, grids, V, hab, stream=stream)
    t_graph = []
    for _ in range(max(1, min(args.steps, 5))):
        flush.zero_()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            e[0].record(stream)
            graph.launch(stream=stream)
            e[1].record(stream)
        graph.wait(stream=stream)
        t_graph.append(e[0].elapsed_time(e[1]))
    graph_kernels = graph.kernels
    graph.free()
    t_model = (run_steps(G.MIXED, G.SCHEDULE_MODEL, max(1, min(args.steps, 5)))
               if model is not None else None)
    # the queue launches of each phase on one stream (no tail overlap)
    tl.set_queue_streams(1)
    t_one_stream = run_steps(G.MIXED, sched_mixed, max(1, min(args.steps, 5)))
    tl.set_queue_streams(2)
    # every double-float task whole (no FP32 outer rows)
    tl.set_row_split(False)
    run_steps(G.MIXED, sched_mixed, 1)
    t_no_row_split = run_steps(G.MIXED, sched_mixed, max(1, min(args.steps, 5)))
    tl.set_row_split(True)
    row_split_share = tl.row_split_stats() + (tl.mixed_split()[1],)
    t_fp64 = run_steps(G.FP64, G.SCHEDULE_SIZE, max(1, min(args.steps, 3)))
    rho64 = [g.cpu().numpy() for g in grids]
    hab64 = hab.cpu().numpy()
    t_fp32 = run_steps(G.FP32, sched_mixed, max(1, min(args.steps, 5)))
    rho32 = [g.cpu().numpy() for g in grids]
    hab32 = hab.cpu().numpy()
    hartree = hartree_step(torch, G, tl, inp, pab, grids, hab, stream, flush,
                           max(1, min(args.steps, 5)))
    taskgen = task_generation(torch, G, inp, host_gen_s, pab, flush, _peaks()[0],
                              geom=(V, grids, stream))

    ms_mixed = max_over_ranks(float(np.mean(t_mixed)), world)
    ms_model = max_over_ranks(float(np.mean(t_model)), world) if t_model else None
    ms_fp64 = max_over_ranks(float(np.mean(t_fp64)), world)
    ms_fp32 = max_over_ranks(float(np.mean(t_fp32)), world)

    # per-launch CUDA events of mixed and FP64 steps (outside the timed region)
    peaks, peak_kind = _peaks()
    fp32_peak = measure_peak(torch, torch.float32, 8192)
    fp64_peak = measure_peak(torch, torch.float64, 4096)
    field_points = float(sum(inp.grid_sizes()))
    per_m, pp_m = kernel_times(torch, tl, G, G.MIXED, sched_mixed, one_step, flush)
    roof_hbm, roof_fp32, share_mixed = roofline_objects(
        per_m, pp_m, field_points, peaks, peak_kind, fp32_peak,
        "measured cuBLAS SGEMM (TF32 off) on this GPU", "mixed")
    per_d, pp_d = kernel_times(torch, tl, G, G.FP64, G.SCHEDULE_SIZE, one_step, flush)
    roof_hbm64, roof_fp64, share_fp64 = roofline_objects(
        per_d, pp_d, field_points, peaks, peak_kind, fp64_peak,
        "measured cuBLAS DGEMM on this GPU", "fp64")

    # e2e through the CP2K C ABI with host offload buffers: inputs are placed
    # in the pinned host buffers once (as CP2K fills them); each timed step
    # copies pab and V host->device, computes, and copies rho and hab back.
    tl.set_precision(G.MIXED)
    tl.set_schedule(sched_mixed)
    tl.collocate(100, pab_h, copy_out=False)
    tl.integrate(V_h, copy_out=False)
    torch.cuda.synchronize()
    e2e = []
    import gc
    gc.collect()
    gc.disable()  # no collector pauses of this harness inside the timed calls
    tl.collocate(100, copy_out=False)  # one more untimed step after the collection
    tl.integrate(copy_out=False)
    try:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            tl.collocate(100, copy_out=False)
            tl.integrate(copy_out=False)
            e2e.append((time.perf_counter() - t0) * 1e3)
    finally:
        gc.enable()
    e2e_ms = max_over_ranks(float(np.mean(e2e)), world)
    # the same with the copies in one piece each (no overlap with the kernels)
    tl.set_copy_chunks(1)
    e2e1 = []
    for _ in range(max(3, min(args.steps, 5))):
        t0 = time.perf_counter()
        tl.collocate(100, copy_out=False)
        tl.integrate(copy_out=False)
        e2e1.append((time.perf_counter() - t0) * 1e3)
    tl.set_copy_chunks(3)
    e2e_one_piece = max_over_ranks(float(np.mean(e2e1[1:])), world)
    h2d = 8 * inp.buffer_size + 8 * int(field_points)  # pab + V grids
    d2h = 8 * int(field_points) + 8 * inp.buffer_size  # rho grids + hab
    tl.close()
    del pab, V, grids, hab
    torch.cuda.empty_cache()

    line = None
    if rank == 0:
        # the oracle: whole FP64 SCF steps on the host cores (CPU baseline),
        # and the FP64 reference results the errors are measured against
        cpu, err_oracle = None, {}
        if world == 1 and not args.no_cpu_baseline:
            ctimes, ref = oracle_steps(inp, pab_h, V_h, 3, 0)
            cpu = {"value": float(np.mean(ctimes)), "unit": "ms", "cores": host_threads(),
                   "kind": "port",
                   "sample": f"3 whole SCF steps of the workload ({inp.ntasks} tasks each), mean"}
            err_oracle = {
                "mixed": errors_vs(rho_mixed, hab_mixed, ref[0], ref[1], V_h, inp),
                "fp64": errors_vs(rho64, hab64, ref[0], ref[1], V_h, inp),
                "fp32": errors_vs(rho32, hab32, ref[0], ref[1], V_h, inp),
            }
        line = {
            "metric": METRIC, "value": ms_mixed, "unit": "ms", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_mixed,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 pairs (double-float) bulk / f64 accumulate", "data": "synthetic",
            "config": {**CONFIG, "ntasks": inp.ntasks, "parallelism": f"replicas x{world}",
                       "schedule": "size (longest first)"},
            "fp64_ms_per_step": ms_fp64, "speedup_vs_fp64": ms_fp64 / ms_mixed,
            "mixed_model_schedule_ms_per_step": ms_model,
            "cost_model": {"params": model_path, "use": "diagnostic; the size schedule is the default"},
            "mixed_one_queue_stream_ms_per_step": max_over_ranks(float(np.mean(t_one_stream)),
                                                                 world),
            "mixed_no_row_split_ms_per_step": max_over_ranks(float(np.mean(t_no_row_split)),
                                                             world),
            "hartree_step_on_device": hartree,
            "task_generation": taskgen,
            "row_split": {"tasks_split": row_split_share[0],
                          "fp32_share_of_points": row_split_share[1],
                          "fp32_class_share_of_points": row_split_share[2]},
            "mixed_cuda_graph_ms_per_step": max_over_ranks(float(np.mean(t_graph)), world),
            "cuda_graph_kernels": int(graph_kernels),
            "autotune": {{0: "fp64", 1: "mixed", 2: "fp32"}[p]: {"grid_ms": v[0], "size_split": v[1]}
                         for p, v in tuned.items()},
            "cost_model_gain": (ms_mixed / ms_model - 1.0) if ms_model else None,
            "fp32_ms_per_step": ms_fp32, "fp32_speedup_vs_fp64": ms_fp64 / ms_fp32,
            "errors_mixed_vs_oracle": err_oracle.get("mixed"),
            "errors_fp64_vs_oracle": err_oracle.get("fp64"),
            "errors_fp32_vs_oracle": err_oracle.get("fp32"),
            "errors_mixed_vs_fp64": errors_vs(rho_mixed, hab_mixed, rho64, hab64, V_h, inp),
            "targets": {"speedup_vs_fp64": 3.0, "rho_max_rel": 1e-6, "energy_ha_per_atom": 1e-8,
                        "fp64_rel": 1e-12},
            "kernel_share_mixed": share_mixed,
            "kernel_share_fp64": share_fp64,
            "roofline": roof_hbm,
            "roofline_fp32": roof_fp32,
            "roofline_fp64": roof_fp64,
            "roofline_fp64_hbm": roof_hbm64,
            "task_list_create_s": create_s,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "e2e_copies_in_one_piece_ms": e2e_one_piece,
            "e2e_steps_ms": [round(x, 3) for x in e2e],
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
        }
    # secondary workloads (reported beside the headline, not part of it)
    if rank == 0 and world == 1 and not args.no_secondary:
        line["triclinic_256atoms_forces_virial"] = secondary_case(
            torch, G, W, "c3_256atoms_triclinic", True, True, 5, 2, flush)
        line["c5_6144atoms_forces"] = secondary_case(
            torch, G, W, "c5_6144atoms", True, False, 3, 1, flush)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the triclinic and 6144-atom lines")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        reference_arm(args, world, rank)
    else:
        gpu_arm(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
