"""Benchmark: fluid_mc residual + Jacobian assembly, elements/s, mixed form vs FP64 form.

Workload (one GPU): 1.0M Delaunay tetrahedra of a jittered 54^3 lattice in the unit
box, 3 components (melt + H2O + CO2), 7 dofs per node, 28x28 element blocks
(the 3D FP64 assembly configuration and its mixed-precision form).  Synthetic,
seeded inputs; the CSR values (0.9 GB) are larger than L2 and are rewritten
every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value    : mixed-form elements/s with inputs resident in HBM (device pointers),
           CUDA events on the launching stream around K assemblies
e2e      : the same call through the C ABI with pinned HOST buffers: per step the
           H2D copy of I and P and the D2H copy of A and b are inside the timed region
roofline : interior kernel (mixed form), algorithmic bytes per element x elements
           / its CUDA-event duration, against the measured HBM copy bandwidth
cpu_baseline / --impl reference : the CPU oracle (a restatement of the reference's
           assembly, OpenMP over element colours) on the host cores

Multi-GPU: every rank assembles its own replica (one process per GPU, no data-path
collective); value = all ranks' elements / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

METRIC = "residual+Jacobian elements/s, mixed vs FP64 on 1 GB300 at <=1e-6 rel err; HBM %"
BYTES_PER_ELEM_TET = 4 * 4 + 8 * 3 * 4 + 2 * 8 * 4 * 7 + 16 * (4 * 7) ** 2 + 16 * 4 * 7  # 13,552
LATTICE_N = 54


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                line = out.stdout.strip().splitlines()
                if line:
                    self.samples.append([x.strip() for x in line[0].split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for i, n in enumerate(names):
                if len(s) > 5 + i and s[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def build_workload(seed: int = 0, lattice: int = LATTICE_N):
    gm = importlib.import_module("gales-multi-fluid_gb300")
    syn = importlib.import_module("gales-multi-fluid_gb300.synthetic")
    mesh = syn.box_tet_delaunay(lattice, seed=seed + 1)
    mat = syn.material_for(3, seed)
    setup = syn.setup_for(3, 3)
    I, P = syn.state_for(mesh, 3, seed)
    return gm, mesh, mat, setup, I, P, 1e-3


def workload_config(mesh, lattice=LATTICE_N):
    return {"workload": f"3D FP64/mixed assembly, {mesh.n_elements} Delaunay tets of a jittered "
                        f"{lattice}^3 lattice, 3 components (melt, H2O, CO2), 7 dofs, 28x28 blocks",
            "n_elements": int(mesh.n_elements), "n_nodes": int(mesh.n_nodes), "dofs_per_node": 7,
            "l2": "CSR values (0.9 GB) > L2, rewritten every step", "seed": 0}


def cpu_oracle_rate(mesh, mat, setup, I, P, dt, row_ptr, col, colour, n_colours, budget_s=20.0):
    """Elements/s of the CPU oracle on the host cores over a bounded element sample."""
    import oracle
    nthreads = os.cpu_count() or 1
    gm = importlib.import_module("gales-multi-fluid_gb300")
    # bounded sample: the first n elements in element order (their own sub-mesh)
    n_try = min(mesh.n_elements, 20000)
    sub = gm.Mesh(mesh.coords, mesh.conn[:n_try], mesh.node_flag, mesh.el_on_boundary[:n_try],
                  mesh.bd_sides[mesh.bd_sides[:, 0] < n_try], name="sample")
    nd = 7
    nrp, ncol, rp, cl = oracle.pattern(sub, nd)
    sc, snc = oracle.colouring(sub)
    t0 = time.perf_counter()
    oracle.assemble(sub, mat, setup, I, P, dt, rp, cl, nthreads=nthreads, colour=sc, n_colours=snc)
    t1 = time.perf_counter()
    rate = n_try / (t1 - t0)
    n = int(min(mesh.n_elements, max(n_try, rate * budget_s)))
    if n > n_try:
        sub = gm.Mesh(mesh.coords, mesh.conn[:n], mesh.node_flag, mesh.el_on_boundary[:n],
                      mesh.bd_sides[mesh.bd_sides[:, 0] < n], name="sample")
        nrp, ncol, rp, cl = oracle.pattern(sub, nd)
        sc, snc = oracle.colouring(sub)
        t0 = time.perf_counter()
        oracle.assemble(sub, mat, setup, I, P, dt, rp, cl, nthreads=nthreads, colour=sc, n_colours=snc)
        t1 = time.perf_counter()
        rate = n / (t1 - t0)
    return rate, nthreads, n


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    gm, mesh, mat, setup, I, P, dt = build_workload()
    vals = []
    for i in range(args.warmup + args.steps):
        rate, cores, n = cpu_oracle_rate(mesh, mat, setup, I, P, dt, None, None, None, 0,
                                         budget_s=max(2.0, 60.0 / max(1, args.warmup + args.steps)))
        if i >= args.warmup:
            vals.append(rate)
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "elements/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(mesh),
            "cpu_baseline": {"value": v, "unit": "elements/s", "cores": cores, "kind": "port",
                             "sample": f"first {n} elements of the workload per step (full interior+boundary "
                                       f"assembly of that sub-mesh, FP64)"},
            "e2e": {"value": v, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--lattice", type=int, default=LATTICE_N, help="lattice points per side (54 -> 1.0M tets)")
    ap.add_argument("--only", default="both", choices=["both", "mixed", "fp64"],
                    help="profiling aid: run only one form (no e2e, no CPU leg)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    b = importlib.import_module("gales-multi-fluid_gb300.build")
    b.build()
    gm, mesh, mat, setup, I, P, dt = build_workload(lattice=args.lattice)
    fa = gm.FluidAssembly(mesh, mat, setup, device=local)
    lp = fa.linear_system(device=dev)
    nnz = int(lp.row_ptr[-1])
    Id = torch.from_numpy(I).to(dev)
    Pd = torch.from_numpy(P).to(dev)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream

    def step(form):
        fa.execute(Id, Pd, dt, lp, form=form, stream=sh)

    if args.only != "both":
        form = gm.FORM_MIXED if args.only == "mixed" else gm.FORM_FP64
        for _ in range(args.warmup + args.steps):
            step(form)
        torch.cuda.synchronize(dev)
        if rank == 0:
            print(json.dumps({"profile_run": args.only, "n_elements": mesh.n_elements,
                              "interior_kernel_ms": fa.phase_ms(1)}), flush=True)
        return
    # accuracy of the mixed form against the FP64 form on this workload
    step(gm.FORM_FP64)
    with torch.cuda.stream(stream):
        v64, b64 = lp.vals.clone(), lp.rhs.clone()
    torch.cuda.synchronize(dev)
    step(gm.FORM_MIXED)
    err_A = float(torch.linalg.norm(lp.vals - v64) / torch.linalg.norm(v64))
    err_b = float(torch.linalg.norm(lp.rhs - b64) / torch.linalg.norm(b64))
    del v64, b64

    def timed(form, k, warm, sampler=None):
        for _ in range(warm):
            step(form)
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        kern = []
        launches0 = fa.launch_count()
        e0.record(stream)
        for _ in range(k):
            step(form)
            kern.append(fa.phase_ms(1))
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / k
        if dist:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms, statistics.median(kern), fa.launch_count() - launches0

    ms64, k64, _ = timed(gm.FORM_FP64, args.fp64_steps, 1)
    with ClockSampler(local) as clk:
        ms_mx, k_mx, launches = timed(gm.FORM_MIXED, args.steps, args.warmup)
    clocks = clk.summary()

    # e2e: host pinned buffers through the C ABI, copies inside the timed region
    Ih = torch.from_numpy(I).pin_memory()
    Ph = torch.from_numpy(P).pin_memory()
    lph = gm.LinearSystem(lp.row_ptr, lp.col, torch.zeros(nnz, dtype=torch.float64).pin_memory(),
                          torch.zeros(fa.n_rows, dtype=torch.float64).pin_memory())
    for _ in range(args.warmup):
        fa.execute(Ih, Ph, dt, lph, form=gm.FORM_MIXED, stream=sh)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fa.execute(Ih, Ph, dt, lph, form=gm.FORM_MIXED, stream=sh)
    torch.cuda.synchronize(dev)
    e2e_s = (time.perf_counter() - t0) / args.steps
    if dist:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())

    ne = mesh.n_elements
    value = world * ne / (ms_mx * 1e-3)
    pk = peaks()
    hbm = pk.get("hbm_gbs")
    achieved = BYTES_PER_ELEM_TET * ne / (k_mx * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mx, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 element integrals + f64 EOS/tau/accumulation (mixed)",
        "data": "synthetic", "config": workload_config(mesh, args.lattice),
        "fp64": {"value": world * ne / (ms64 * 1e-3), "unit": "elements/s", "ms_per_step": ms64,
                 "interior_kernel_ms": k64},
        "mixed_over_fp64": ms64 / ms_mx,
        "mixed_rel_err_vs_fp64": {"matrix": err_A, "rhs": err_b},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if hbm else None, "traffic": None,
                     "kernel": "interior_kernel (mixed form)", "kernel_ms": k_mx,
                     "bytes_per_element": BYTES_PER_ELEM_TET, "peak_source": "measured (MEASURED_PEAKS.json)"},
        "e2e": {"value": world * ne / e2e_s, "unit": "elements/s",
                "h2d_bytes_per_step": 2 * fa.n_rows * 8, "d2h_bytes_per_step": (nnz + fa.n_rows) * 8},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu:
        rate, cores, n = cpu_oracle_rate(mesh, mat, setup, I, P, dt, None, None, None, 0)
        line["cpu_baseline"] = {"value": rate, "unit": "elements/s", "cores": cores, "kind": "port",
                                "sample": f"first {n} elements of the workload (their sub-mesh), FP64, "
                                          f"OpenMP over element colours"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
