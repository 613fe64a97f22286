#!/usr/bin/env python
"""SIMP iterations per second of the GPU inner loop (one JSON line).

A step is one SIMP iteration (filter, SIMP law, K_ff assembly, AMG setup,
AMG-PCG per load case, sensitivities, filter pull-back, OC update) on the
seeded synthetic Hex8 cantilever of 192 x 96 x 96 cells (1,769,472 elements,
5,419,584 free DOFs), resident in GPU memory.  `value` is device-timed (CUDA
events on the library's stream); `e2e` repeats the step through the public
API with the design copied from pinned host memory and back every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl own|reference]
                  [--config NAME] [--precision fp64|mixed]
                  [--warm zero|previous|projection|learned]

`--warm learned` trains the displacement surrogate before the timed region
(2,000 pairs from plain FP64 SIMP runs of seeded variants) and starts every
PCG solve from the energy-optimal combination of the previous displacements
and its prediction.

`--impl reference` times the CPU restatement of the reference's algorithm (the
reference itself needs Eigen, which is absent) on the host cores, on the full
workload: W warm-up SIMP iterations (the first builds the hierarchy), then K
timed iterations, each a complete SIMP iteration of the full grid.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from sparlab_gb300 import problems as P  # noqa: E402

# PCG initial guess per load case (simp_problem_desc.warm_start)
WARM = {"zero": 0, "previous": 1, "projection": 2, "learned": 3}

METRIC = "SIMP iter/s at Hex8 1.77M elts, compliance err<=1e-6: plain vs learned+mixed"

WORKLOADS = {
    "hex8_192x96x96": (P.hex8_192x96x96, (96, 48, 48)),
    "hex8_96x48x48": (P.hex8_96x48x48, (48, 24, 24)),
    "q4_600x200": (P.q4_cantilever_600x200, None),
    "q4_120x40": (P.q4_cantilever_120x40, None),
}
# 64 independent instances (48 Q4, 16 Hex8, seed 4): a step is one SIMP
# iteration of every instance; the metric is instance-iterations per second
BATCHED = "batched_64"
BATCHED_METRIC = "instance SIMP iter/s, 64 independent Q4/Hex8 instances (seed 4)"


# Undamped free vibration of the solid Hex8 96 x 48 x 48 cantilever (unit
# cells, E = 1, nu = 0.3, density 1): a step is one complete modal analysis
# (6 lowest modes, consistent mass, subspace iteration over its own AMG-PCG
# hierarchy); the metric is modal analyses per second
MODAL = "modal_hex8_96x48x48"
MODAL_METRIC = "modal analyses/s (6 lowest modes, Hex8 96x48x48 solid cantilever)"
MODAL_MODES = 6


def modal_spec(nx=96, ny=48, nz=48):
    spec = P.hex8_cantilever(nx, ny, nz, 0.2, f"modal_hex8_{nx}x{ny}x{nz}")
    spec.rtol = 1e-10
    return spec


def modal_cpu_baseline(steps=1):
    """Oracle modal analysis of the same cantilever with every axis divided
    by four (1/64 of the cells), scaled by the cell ratio."""
    import oracle
    from oracle import modal as OM
    spec = modal_spec(24, 12, 12)
    ratio = 64.0
    times, its = [], 0
    for _ in range(steps):
        pr = oracle.Problem(spec)
        t0 = time.perf_counter()
        r = OM.solve_modal(pr, spec, num_modes=MODAL_MODES, density=spec.density, rtol=spec.rtol)
        times.append(time.perf_counter() - t0)
        its = r.iterations
    t = min(times)
    return {"value": 1.0 / (t * ratio), "unit": "analyses/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{spec.name}: 24x12x12 cells (1/64 of the workload's), {its} subspace iterations, "
                      f"min of {steps} analyses ({t:.2f} s each), scaled by the cell ratio 64"}


# Linear buckling of a solid Hex8 column (the reference's Euler column,
# tests/test_buckling.cpp:41-68, refined): 384 x 24 x 24 cubic cells, length 1,
# square section 0.0625, steel, root clamped, unit axial compression on the
# free end.  A step is one analysis (static solve, geometric stiffness, the 4
# smallest positive load factors by subspace iteration).
BUCKLING = "buckling_hex8_column_384x24x24"
BUCKLING_METRIC = "buckling analyses/s (4 load factors, Hex8 column 384x24x24)"
BUCKLING_MODES = 4


def buckling_spec(nx=384, ny=24, nz=24):
    spec = P.column(3, nx, ny, nz, length=1.0, height=0.0625, width=0.0625)
    spec.rtol = 1e-10
    return spec


def buckling_cpu_baseline():
    """Oracle buckling analysis (AMG-PCG solves) of the column with every
    axis divided by four (96 x 6 x 6), scaled by the cell ratio 64."""
    import oracle
    from oracle import buckling as OB
    spec = buckling_spec(96, 6, 6)
    pr = oracle.Problem(spec)
    t0 = time.perf_counter()
    r = OB.analyse_buckling(pr, spec, num_modes=BUCKLING_MODES, linear="amg_cg", rtol=spec.rtol)
    t = time.perf_counter() - t0
    return {"value": 1.0 / (t * 64.0), "unit": "analyses/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{spec.name}: 96x6x6 cells (1/64 of the workload's), {r.iterations} subspace "
                      f"iterations, one analysis ({t:.2f} s), scaled by the cell ratio 64"}


def workload_config(spec):
    """The static description of a workload, printed identically by both
    arms (run-specific figures go to the line's "run" object)."""
    return {"workload": spec.name, "elements": spec.num_elements, "free_dofs": int(len(spec.free_dofs())),
            "load_cases": int(spec.loads.shape[0]), "volume_fraction": spec.volume_fraction,
            "filter_radius": spec.filter_radius, "rtol": spec.rtol}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for name, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_baseline(spec):
    """The oracle (the reference's algorithms, OpenMP on every host core where
    the reference uses it) on the full workload: the first SIMP iteration
    builds the hierarchy, the second is timed.  Also returns the oracle's
    first two iterations (compliance, CG iterations) for the parity check."""
    import oracle
    pr = oracle.Problem(spec)
    x = np.full(pr.ne, spec.volume_fraction if spec.initial_density < 0 else spec.initial_density)
    first = []
    ev = pr.evaluate(x)
    first.append((float(ev["compliance"]), int(ev["linear_iterations"])))
    x, _ = pr.oc_update(x, ev["dc_dx"], ev["dv_dx"])
    t0 = time.perf_counter()
    ev = pr.evaluate(x)
    x, _ = pr.oc_update(x, ev["dc_dx"], ev["dv_dx"])
    t = time.perf_counter() - t0
    first.append((float(ev["compliance"]), int(ev["linear_iterations"])))
    base = {"value": 1.0 / t, "unit": "iter/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{spec.name} at full size: its second SIMP iteration ({t:.2f} s, "
                      f"{first[1][1]} CG iterations; the first builds the hierarchy); the timed GPU steps "
                      f"are later iterations, which need more CG iterations"}
    return base, first


def batched_cpu_baseline(specs, every=8):
    """Oracle on every `every`-th instance (one setup iteration, one timed
    iteration each), scaled to the whole batch."""
    import oracle
    total = 0.0
    sample = specs[::every]
    for spec in sample:
        pr = oracle.Problem(spec)
        x = np.full(pr.ne, spec.volume_fraction)
        ev = pr.evaluate(x)
        x, _ = pr.oc_update(x, ev["dc_dx"], ev["dv_dx"])
        t0 = time.perf_counter()
        ev = pr.evaluate(x)
        pr.oc_update(x, ev["dc_dx"], ev["dv_dx"])
        total += time.perf_counter() - t0
    scale = len(specs) / len(sample)
    return {"value": len(specs) / (total * scale), "unit": "instance-iter/s", "cores": os.cpu_count(),
            "kind": "port", "sample": f"{len(sample)} of the {len(specs)} instances (every {every}th), "
                                      f"one timed SIMP iteration each after a setup iteration "
                                      f"({total:.2f} s), scaled by {scale:.0f}"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.config == BUCKLING:
        base = buckling_cpu_baseline()
        v = base["value"]
        print(json.dumps({
            "impl": "reference", "metric": BUCKLING_METRIC, "value": v, "unit": "analyses/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic cantilever (no dataset)",
            "config": {"workload": BUCKLING, "modes": BUCKLING_MODES, "host_threads": os.cpu_count()},
            "cpu_baseline": base,
            "e2e": {"value": v, "unit": "analyses/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }), flush=True)
        return
    if args.config == MODAL:
        base = modal_cpu_baseline()
        v = base["value"]
        print(json.dumps({
            "impl": "reference", "metric": MODAL_METRIC, "value": v, "unit": "analyses/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic cantilever (no dataset)",
            "config": {"workload": MODAL, "modes": MODAL_MODES, "host_threads": os.cpu_count()},
            "cpu_baseline": base,
            "e2e": {"value": v, "unit": "analyses/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }), flush=True)
        return
    if args.config == BATCHED:
        specs = P.batched_instances(seed=4)
        base = batched_cpu_baseline(specs)
        v = base["value"]
        print(json.dumps({
            "impl": "reference", "metric": BATCHED_METRIC, "value": v, "unit": "instance-iter/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": len(specs) / v * 1e3, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic seeded instances (no dataset)",
            "config": {"workload": BATCHED, "instances": len(specs), "precision": "fp64",
                       "host_threads": os.cpu_count()},
            "cpu_baseline": base,
            "e2e": {"value": v, "unit": "instance-iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }), flush=True)
        return
    import oracle
    spec = WORKLOADS[args.config][0]()
    pr = oracle.Problem(spec)
    x = np.full(pr.ne, spec.volume_fraction if spec.initial_density < 0 else spec.initial_density)
    warm_s = time.perf_counter()
    for _ in range(max(1, args.warmup)):     # the first iteration builds the hierarchy
        ev = pr.evaluate(x)
        x, _ = pr.oc_update(x, ev["dc_dx"], ev["dv_dx"])
    warm_s = time.perf_counter() - warm_s
    times, comp, its = [], [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ev = pr.evaluate(x)
        x, _ = pr.oc_update(x, ev["dc_dx"], ev["dv_dx"])
        times.append(time.perf_counter() - t0)
        comp.append(float(ev["compliance"]))
        its.append(int(ev["linear_iterations"]))
    per = sum(times) / len(times)
    value = 1.0 / per
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic seeded cantilever (no dataset)",
        "config": workload_config(spec),
        "run": {"implementation": "the oracle: a C++ restatement of the reference's algorithms (the reference "
                                  "needs Eigen, absent here); OpenMP where the reference uses it",
                "host_threads": os.cpu_count(), "warmup_seconds": round(warm_s, 2),
                "step_seconds": [round(t, 3) for t in times],
                "cg_iterations_per_step": its, "compliance_per_step": comp},
        "cpu_baseline": {"value": value, "unit": "iter/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"the full {spec.name} workload: {args.steps} SIMP iterations timed after "
                                   f"{max(1, args.warmup)} warm-up iterations (the first builds the hierarchy)"},
        "e2e": {"value": value, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def whole_job_rate(ms_local, steps, world, device=None):
    """The slowest replica bounds the job: the max over ranks of the timed
    milliseconds, and the whole-job rate world * steps / that time."""
    ms = float(ms_local)
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * steps / (ms * 1e-3)


def run_own_buckling(args):
    """Buckling analyses of the solid cantilever; replicas under torchrun."""
    import torch
    import torch.distributed as dist
    from sparlab_gb300 import _lib
    from sparlab_gb300.topopt import GpuSimpProblem

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    spec = buckling_spec()
    prob = GpuSimpProblem(spec, precision=args.precision, device=local)
    lib = _lib.load()
    for _ in range(args.warmup):
        prob.buckling(num_modes=BUCKLING_MODES, mode_shapes=False)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    barrier()
    launches0 = lib.simp_kernel_launches()
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    recs = [prob.buckling(num_modes=BUCKLING_MODES, mode_shapes=False) for _ in range(args.steps)]
    e1.record()
    barrier()
    clocks = sampler.stop()
    launches = lib.simp_kernel_launches() - launches0
    ms, value = whole_job_rate(e0.elapsed_time(e1), args.steps, world, dev)
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    for _ in range(args.steps):
        prob.buckling(num_modes=BUCKLING_MODES, mode_shapes=True)
    f1.record()
    barrier()
    e2e_ms, e2e_value = whole_job_rate(f0.elapsed_time(f1), args.steps, world, dev)
    if rank != 0:
        return
    line = {
        "metric": BUCKLING_METRIC, "value": value, "unit": "analyses/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic cantilever (no dataset)",
        "config": {"workload": BUCKLING, "elements": spec.num_elements, "free_dofs": prob.nfree,
                   "modes": BUCKLING_MODES, "precision": args.precision,
                   "subspace_size": recs[-1].subspace_size,
                   "subspace_iterations": [r.iterations for r in recs],
                   "pcg_iterations": [r.linear_iterations for r in recs],
                   "load_factors": [float(f) for f in recs[-1].load_factors],
                   "l2": "working set (K_ff and K_G 1.4 GB) larger than L2"},
        "roofline": None,
        "cpu_baseline": buckling_cpu_baseline() if world == 1 else None,
        "e2e": {"value": e2e_value, "unit": "analyses/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 8 * BUCKLING_MODES * prob.ndof},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_own_modal(args):
    """Modal analyses of the solid cantilever; replicas under torchrun."""
    import torch
    import torch.distributed as dist
    from sparlab_gb300 import _lib
    from sparlab_gb300.topopt import GpuSimpProblem

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    spec = modal_spec()
    prob = GpuSimpProblem(spec, precision=args.precision, device=local)
    lib = _lib.load()
    for _ in range(args.warmup):
        r = prob.modal(num_modes=MODAL_MODES, mode_shapes=False)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    barrier()
    launches0 = lib.simp_kernel_launches()
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    recs = [prob.modal(num_modes=MODAL_MODES, mode_shapes=False) for _ in range(args.steps)]
    e1.record()
    barrier()
    clocks = sampler.stop()
    launches = lib.simp_kernel_launches() - launches0
    ms, value = whole_job_rate(e0.elapsed_time(e1), args.steps, world, dev)
    # e2e: the same analysis through the public API with the mode shapes
    # copied back to the host every step
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    for _ in range(args.steps):
        r = prob.modal(num_modes=MODAL_MODES, mode_shapes=True)
    f1.record()
    barrier()
    e2e_ms, e2e_value = whole_job_rate(f0.elapsed_time(f1), args.steps, world, dev)
    if rank != 0:
        return
    line = {
        "metric": MODAL_METRIC, "value": value, "unit": "analyses/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic cantilever (no dataset)",
        "config": {"workload": MODAL, "elements": spec.num_elements, "free_dofs": prob.nfree,
                   "modes": MODAL_MODES, "mass": "consistent", "precision": args.precision,
                   "subspace_size": recs[-1].subspace_size,
                   "subspace_iterations": [r.iterations for r in recs],
                   "pcg_iterations": [r.linear_iterations for r in recs],
                   "frequencies_hz": [float(f) for f in recs[-1].frequencies_hz],
                   "l2": "working set (K_ff and M_ff 1.3 GB) larger than L2"},
        "roofline": None,
        "cpu_baseline": modal_cpu_baseline() if world == 1 else None,
        "e2e": {"value": e2e_value, "unit": "analyses/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 8 * MODAL_MODES * prob.ndof},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_own_batched(args):
    """64 independent instances: each rank takes instances rank, rank + N, ...
    (no collective on the data path) and drives its share from host threads,
    one CUDA stream per instance."""
    import torch
    import torch.distributed as dist
    from sparlab_gb300 import _lib
    from sparlab_gb300.topopt import GpuSimpProblem, run_batched

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    specs = P.batched_instances(seed=4)
    mine = specs[rank::world]
    probs = [GpuSimpProblem(s, precision=args.precision, device=local) for s in mine]
    lib = _lib.load()
    schedule = {}
    run_batched(probs, args.warmup, tune=True, report=schedule)   # warm-up iterations pick the host workers
    workers = schedule.get("workers")

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    barrier()
    launches0 = lib.simp_kernel_launches()
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    recs = run_batched(probs, args.steps, workers=workers)
    e1.record()
    barrier()
    clocks = sampler.stop()
    launches = lib.simp_kernel_launches() - launches0
    ms, _ = whole_job_rate(e0.elapsed_time(e1), args.steps, world, dev)
    value = len(specs) * args.steps / (ms * 1e-3)

    # e2e: every instance's design from pinned host memory and back, each step
    hosts = []
    for p in probs:
        h = torch.empty(p.ne, dtype=torch.float64, pin_memory=True).numpy()
        h[:] = p.design()
        hosts.append(h)
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    for _ in range(args.steps):
        for p, h in zip(probs, hosts):
            p.set_design(h)
        run_batched(probs, 1, workers=workers)
        for p, h in zip(probs, hosts):
            p.design(out=h)
    f1.record()
    barrier()
    e2e_ms, _ = whole_job_rate(f0.elapsed_time(f1), args.steps, world, dev)
    h2d = sum(8 * p.ne for p in probs)

    big = max(probs, key=lambda p: p.nnz)
    kms, alg_bytes = big.time_operator(20)
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (kms * 1e-3) / 1e9
    if rank != 0:
        return
    line = {
        "metric": BATCHED_METRIC, "value": value, "unit": "instance-iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic seeded instances (no dataset)",
        "config": {"workload": BATCHED, "instances": len(specs), "precision": args.precision,
                   "instances_per_rank": len(mine), "host_threads": os.cpu_count(),
                   "elements_total": sum(s.num_elements for s in specs),
                   "cg_iterations_per_step": [sum(r[k].linear_iterations for r in recs)
                                              for k in range(args.steps)],
                   "schedule": schedule,
                   "autotune": {k: v[0] for k, v in _lib.autotune_report().items()},
                   "l2": "no flush: a step touches every instance's operators once"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "level-0 CG operator of the largest instance (%s)" % big.spec.name,
                     "bytes_per_launch": alg_bytes, "ms_per_launch": kms,
                     "peak_kind": f"{peak_kind} hbm_gbs (burst copy)"},
        "cpu_baseline": batched_cpu_baseline(specs) if world == 1 else None,
        "e2e": {"value": len(specs) * args.steps / (e2e_ms * 1e-3), "unit": "instance-iter/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def train_surrogate(args, device):
    """The learned start's network, trained before the timed region on
    (density, displacement) pairs that the plain FP64 solver produces along
    20-iteration SIMP runs of 100 seeded Hex8 cantilever variants (seeds
    100-149 on 48 x 24 x 24, 150-199 on 96 x 48 x 48): 2,000 pairs."""
    from sparlab_gb300.surrogate import Surrogate, generate_samples, training_variants
    sur = Surrogate(seed=7, device=device)
    t0 = time.perf_counter()
    generate_samples(sur, training_variants(range(100, 200)), iterations=20, precision="fp64")
    t1 = time.perf_counter()
    losses = sur.train(epochs=args.train_epochs, learning_rate=2e-3, batch=4, seed=11)
    t2 = time.perf_counter()
    info = {"pairs": sur.num_samples, "generation_seconds": round(t1 - t0, 1),
            "training_seconds": round(t2 - t1, 1), "epochs": args.train_epochs,
            "epoch_losses": [round(v, 6) for v in losses], "parameters": sur.num_params}
    return sur, info


def run_own(args):
    import torch
    import torch.distributed as dist
    from sparlab_gb300 import _lib
    from sparlab_gb300.topopt import GpuSimpProblem

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    spec = WORKLOADS[args.config][0]()
    learned = args.warm == "learned" and spec.dim == 3
    spec.warm_start = WARM["learned" if learned else ("previous" if args.warm == "learned" else args.warm)]
    together = "graph" if args.graph_loads else not args.sequential_loads
    lib = _lib.load()
    sur, sur_info = (train_surrogate(args, local) if learned else (None, None))

    tc = {} if args.tensor_cores is None else {"tensor_cores": args.tensor_cores}

    def make(precision, with_surrogate=True):
        p = GpuSimpProblem(spec, precision=precision, device=local, block_pcg=together, **tc)
        if with_surrogate and sur is not None:
            p.set_surrogate(sur)
        return p

    prob = make(args.precision)
    # warm-up: the first iteration builds the hierarchy
    t_setup = time.perf_counter()
    warm_recs = [prob.iterate() for _ in range(args.warmup)]
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t_setup

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    barrier()
    launches0 = lib.simp_kernel_launches()
    learned0 = prob.learned_seconds()
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    recs = [prob.iterate() for _ in range(args.steps)]
    e1.record()
    barrier()
    clocks = sampler.stop()
    launches = lib.simp_kernel_launches() - launches0
    learned_s = prob.learned_seconds() - learned0
    ms, value = whole_job_rate(e0.elapsed_time(e1), args.steps, world, dev)
    per_step = ms / args.steps

    # e2e: a fresh instance over the same iterations (the same warm-up, then
    # the timed steps), with the design copied in from pinned host memory and
    # the design and compliance read back every step
    e2e_prob = make(args.precision)
    for _ in range(args.warmup):
        e2e_prob.iterate()
    x_host = torch.empty(prob.ne, dtype=torch.float64, pin_memory=True).numpy()
    x_host[:] = e2e_prob.design()
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    for _ in range(args.steps):
        e2e_prob.set_design(x_host)
        r = e2e_prob.iterate()
        e2e_prob.design(out=x_host)
        _ = r.compliance
    f1.record()
    barrier()
    e2e_prob.close()
    e2e_ms, e2e_value = whole_job_rate(f0.elapsed_time(f1), args.steps, world, dev)

    # dominant kernel: the level-0 operator of the CG (both modes), timed
    # alone with CUDA events on the library's stream
    kms, alg_bytes = prob.time_operator(20)
    nnz = prob.nnz
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (kms * 1e-3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "spmv_traffic.json")
    if os.path.exists(prof):
        with open(prof) as f:
            d = json.load(f)
        if d.get("workload") == spec.name:
            traffic = d.get("traffic_bytes_per_launch")

    def timed_run(precision, with_surrogate):
        p = make(precision, with_surrogate)
        first = [p.iterate() for _ in range(args.warmup)]
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record()
        rr = [p.iterate() for _ in range(args.steps)]
        g1.record()
        torch.cuda.synchronize()
        t = g0.elapsed_time(g1)
        p.close()
        return first, rr, t

    # the plain FP64 loop (the reference's warm start) on the same iterations,
    # for the metric's plain-vs-learned+mixed ratio and the compliance bar;
    # with the learned start also the mixed loop without it
    plain = mixed_only = mixed_projected = None
    plain_first = None
    if args.precision == "mixed" and not args.no_plain and world == 1:
        if learned:
            spec.warm_start = WARM["previous"]
            _, mrec, mms = timed_run("mixed", False)
            mixed_only = {"value": args.steps / (mms * 1e-3), "unit": "iter/s", "ms_per_step": mms / args.steps,
                          "cg_iterations_per_step": [r.linear_iterations for r in mrec],
                          "max_rel_compliance_diff": max(abs(a.compliance / b.compliance - 1)
                                                         for a, b in zip(recs, mrec))}
            # the learned start without the network: the energy-optimal start
            # over the displacement history alone (what the prediction adds)
            spec.warm_start = WARM["projection"]
            _, jrec, jms = timed_run("mixed", False)
            mixed_projected = {"value": args.steps / (jms * 1e-3), "unit": "iter/s",
                               "ms_per_step": jms / args.steps,
                               "cg_iterations_per_step": [r.linear_iterations for r in jrec],
                               "max_rel_compliance_diff": max(abs(a.compliance / b.compliance - 1)
                                                              for a, b in zip(recs, jrec))}
        spec.warm_start = WARM["previous"]
        plain_first, prec, pms = timed_run("fp64", False)
        plain = {"value": args.steps / (pms * 1e-3), "unit": "iter/s", "ms_per_step": pms / args.steps,
                 "warm_start": "previous",
                 "cg_iterations_per_step": [r.linear_iterations for r in prec],
                 "compliance_per_step": [r.compliance for r in prec],
                 "max_rel_compliance_diff": max(abs(a.compliance / b.compliance - 1)
                                                for a, b in zip(recs, prec))}

    if rank != 0:
        return
    st = prob.amg_stats()
    cpu, oracle_check = None, None
    if world == 1:
        cpu, first = cpu_baseline(spec)
        if plain_first is not None and len(plain_first) >= 2:
            oracle_check = {
                "iterations": [1, 2],
                "oracle_compliance": [c for c, _ in first],
                "gpu_fp64_compliance": [r.compliance for r in plain_first[:2]],
                "max_rel_compliance_diff": max(abs(r.compliance / c - 1) for r, (c, _) in zip(plain_first, first)),
                "oracle_cg_iterations": [i for _, i in first],
                "gpu_fp64_cg_iterations": [r.linear_iterations for r in plain_first[:2]]}
    line = {
        "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic seeded cantilever (no dataset)",
        "config": workload_config(spec),
        "run": {"precision": args.precision,
                "warm_start": "learned" if learned else spec_warm_name(spec.warm_start),
                "nnz_kff": prob.nnz, "replicas": world,
                "level0_tensor_cores": int(prob.options.tensor_cores),
                "load_case_solves": ("one graph, fused multi-RHS CG operator" if together == "graph" else
                                     "concurrent" if together else "sequential"),
                "l2": ("working set (K_ff %.2f GB) larger than the 129 MB L2" % (nnz * 12 / 1e9)
                       if nnz * 12 > 129e6 else
                       "working set (K_ff %.3f GB) fits in the 129 MB L2; not flushed between steps"
                       % (nnz * 12 / 1e9)),
                "amg_levels": st["num_levels"],
                "operator_complexity": round(st["operator_complexity"], 6),
                "cg_iterations_per_step": [r.linear_iterations for r in recs],
                "cg_iterations_warmup": [r.linear_iterations for r in warm_recs],
                "oc_bisections_per_step": [r.bisections for r in recs],
                "compliance_per_step": [r.compliance for r in recs],
                "warmup_seconds_incl_setup": round(t_setup, 3),
                "surrogate_seconds_in_timed_steps": round(learned_s, 4) if learned else None,
                "surrogate": sur_info,
                "mixed_previous_start": mixed_only,
                "mixed_projected_start_without_network": mixed_projected,
                "autotune": {k: {"chosen": v[0], "ms": [round(t, 4) for t in v[1]]}
                             for k, v in _lib.autotune_report().items()},
                "plain_fp64": plain,
                "oracle_check": oracle_check},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": (f"k_rows_apply<4,{spec.dim},0,double> (level-0 K_ff operator of the CG, "
                                "FP64 values; FP64-pipe bound on GB300)" if args.precision == "fp64" else
                                f"k_rows_apply_df<4,{spec.dim},0> (level-0 K_ff operator of the CG, "
                                "double-float values and arithmetic on the FP32 pipes)"),
                     "bytes_per_launch": alg_bytes, "ms_per_launch": kms,
                     "peak_kind": f"{peak_kind} hbm_gbs (burst copy)"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "iter/s",
                "h2d_bytes_per_step": 8 * prob.ne, "d2h_bytes_per_step": 8 * prob.ne + 8},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def spec_warm_name(w):
    return {v: k for k, v in WARM.items()}.get(w, str(w))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="own", choices=["own", "reference"])
    ap.add_argument("--config", default="hex8_192x96x96", choices=sorted(WORKLOADS) + [BATCHED, MODAL, BUCKLING])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 comparison run that follows a mixed-precision run")
    ap.add_argument("--warm", default="learned", choices=sorted(WARM),
                    help="PCG initial guess: zero, the previous displacement (the reference's "
                         "warm start), the energy-optimal combination of the last three, or that "
                         "combination with the displacement surrogate's prediction (learned; 3-D "
                         "workloads: the network is trained before the timed region)")
    ap.add_argument("--train-epochs", type=int, default=4,
                    help="training epochs of the surrogate over its 2,000 pairs (learned start)")
    ap.add_argument("--tensor-cores", type=int, default=None, choices=[0, 1],
                    help="matrix-free level 0 on the tensor cores (1) or on FP32 FMAs (0); "
                         "default: the library's default")
    ap.add_argument("--graph-loads", action="store_true",
                    help="advance a multi-load workload's load cases together in one CUDA graph, "
                         "their CG products as one multi-RHS launch over the shared K_ff")
    ap.add_argument("--sequential-loads", action="store_true",
                    help="solve a multi-load workload's load cases one after another instead of "
                         "concurrently (one workspace and stream per load case)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.config == BATCHED:
        run_own_batched(args)
    elif args.config == MODAL:
        run_own_modal(args)
    elif args.config == BUCKLING:
        run_own_buckling(args)
    else:
        run_own(args)


if __name__ == "__main__":
    main()
