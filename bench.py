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
hex      : 3,993,600 trilinear hexahedra, 4 components, 8 dofs: 10 mixed assemblies
           replayed from one CUDA graph, FP64 beside them, the mixed form's error, the
           roofline and the top-face gas-flux VJP
newton   : Newton iterations of a time step on the tet mesh, on the GPU, FP64 tangent
           against the mixed tangent (diagonal tau to 1e-8; shipped tau with n_max_it 3)

Multi-GPU: every rank assembles its own replica (one process per GPU, no data-path
collective); value = all ranks' elements / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import gc
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
# DRAM bytes per element of the mixed tet interior pass (point and matrix kernels; the
# point kernel's clear of A and b included):
# dram__bytes_read.sum + dram__bytes_write.sum from ncu on the 163,618-tet mesh of the
# 30^3 lattice, whose CSR bytes per element (1,002) match the 1.0M-tet mesh's (982);
# scaled by the element count (profiles/dram_traffic_tet4_lattice30_assembly.md).
TRAFFIC_BYTES_PER_ELEM_TET = 10502
LATTICE_N = 54


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


# Per-element instruction counts of the mixed tet pass (3 components), from ncu on the
# 163,618-tet mesh of the 30^3 lattice (profiles/point_matrix_kernels_mixed_tet4_lattice30.md):
# FP64 thread instructions per quadrature point of the point kernel and warp
# instructions per element of the matrix kernel.
POINT_FP64_PER_POINT = {"dfma": 193.5, "dmul_dadd": 197.2}
MATRIX_WARP_INST_PER_ELEM = 2758
NQ_TET = 4


def pipe_rates():
    """The device's FP64/FP32 arithmetic rates (pipe_rates probe built with the library)."""
    exe = ROOT / "gales-multi-fluid_gb300" / "pipe_rates"
    try:
        out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
        return json.loads(out.stdout.strip().splitlines()[-1])
    except Exception as e:  # reported, never fatal
        return {"error": f"{type(e).__name__}: {e}"}


def compute_roofline(n_el, point_ms, matrix_ms):
    """Compute side of the interior pass: the point kernel against the FP64 rate (its FP64
    instructions per point at the measured DFMA / DMUL rates), the matrix kernel against
    the issue rate (4 warp instructions per SM per clock)."""
    pr = pipe_rates()
    out = {"pipe_rates": pr, "point_kernel_ms": point_ms, "matrix_kernel_ms": matrix_ms}
    if "error" in pr or not (point_ms and matrix_ms and point_ms > 0 and matrix_ms > 0):
        return out
    sms, hz = pr["sm_count"], pr["clock_mhz"] * 1e6
    fp64_cycles = n_el * NQ_TET * (POINT_FP64_PER_POINT["dfma"] / pr["dfma_per_clk_sm"] +
                                   POINT_FP64_PER_POINT["dmul_dadd"] / pr["dmul_per_clk_sm"])
    t_fp64 = fp64_cycles / sms / hz * 1e3
    t_issue = n_el * MATRIX_WARP_INST_PER_ELEM / (4.0 * sms) / hz * 1e3
    out["point_kernel"] = {"bound": "fp64 (the FMA pipe, shared with FP32 on this GPU)",
                           "ms_at_peak": t_fp64, "frac": t_fp64 / point_ms,
                           "fp64_per_point": POINT_FP64_PER_POINT}
    out["matrix_kernel"] = {"bound": "instruction issue (4 warp instructions per SM per clock)",
                            "ms_at_peak": t_issue, "frac": t_issue / matrix_ms,
                            "warp_inst_per_element": MATRIX_WARP_INST_PER_ELEM}
    return out


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


def max_over_ranks(x: float, dist, device) -> float:
    """The slowest rank's value (replicas: one independent assembly per GPU)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: int, ms_max: float, world: int) -> float:
    """Units of all ranks per second of the slowest rank (weak scaling)."""
    return world * units_per_rank / (ms_max * 1e-3)


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


BYTES_PER_ELEM_HEX = 4 * 8 + 8 * 3 * 8 + 2 * 8 * 8 * 8 + 16 * (8 * 8) ** 2 + 16 * 8 * 8  # 67,808
# DRAM bytes per element of the mixed hex interior pass, from ncu on the 64,000-hex mesh
# of a 40^3 grid in one chunk with a separate clear kernel, like the chunks of the
# 160x160x156 assembly (point records far larger than L2); CSR bytes per element 14,172,
# 1.9% above that mesh's 13,911; scaled by the element count
# (profiles/dram_traffic_hex8_40cube_assembly.md, capture B).
TRAFFIC_BYTES_PER_ELEM_HEX = 64817


def top_gas_flux_lambda(mesh, mat, I, nd):
    """lambda = dJ/dI of J = sum over top-face nodes of A_n rho (1 - Y_melt) v_z: the
    gas mass flux through the top face (nodal quadrature, lumped quad areas), with rho
    the mixture density (fluid_properties.hpp:199-227) at the node.  Complex-step
    derivative per dof; nodes are independent, so one pass per dof covers them all."""
    coords = mesh.coords
    top = np.nonzero(np.abs(coords[:, 2] - coords[:, 2].max()) < 1e-12)[0]
    # lumped areas of the top quads (sides 0 of the boundary elements with a top side)
    bd = mesh.bd_sides[mesh.bd_sides[:, 1] == 0]
    quad = mesh.conn[bd[:, 0]][:, [4, 5, 6, 7]]
    x, y = coords[quad, 0], coords[quad, 1]
    area = 0.5 * np.abs((x * np.roll(y, -1, axis=1) - np.roll(x, -1, axis=1) * y).sum(axis=1))
    A = np.zeros(len(coords))
    np.add.at(A, quad.ravel(), np.repeat(area / 4.0, 4))
    S = I.reshape(-1, nd)[top]
    chems = mat.chemicals

    def J(Sc):
        p, vz, T = Sc[:, 0], Sc[:, 3], Sc[:, 4]
        Ys = [Sc[:, 5 + i] for i in range(len(chems) - 1)]
        Ys.append(1.0 - sum(Ys))
        irho = 0.0
        for c, q in enumerate(chems):
            r = q.rho if q.kind == 0 else p / (q.R * T)
            irho = irho + Ys[c] / r
        return A[top] * (1.0 / irho) * (1.0 - Ys[0]) * vz

    lam = np.zeros((len(coords), nd))
    h = 1e-30
    for j in range(nd):
        Sc = S.astype(np.complex128)
        Sc[:, j] += 1j * h * max(1.0, float(np.abs(S[:, j]).max()))
        lam[top, j] = J(Sc).imag / (h * max(1.0, float(np.abs(S[:, j]).max())))
    return lam.ravel(), float(J(S.astype(np.complex128)).real.sum())


def hex_block(args, torch, dev, with_clocks=False):
    """Large hex workload: 160x160x156 trilinear hexahedra (3,993,600) with 10% node
    jitter, 4 components, 8 dofs, 64x64 blocks; 10 mixed assemblies captured in one
    CUDA graph, FP64 beside it, the mixed form's error against the FP64 form, and the
    VJP of the top-face gas mass flux."""
    gm = importlib.import_module("gales-multi-fluid_gb300")
    syn = importlib.import_module("gales-multi-fluid_gb300.synthetic")
    nx, ny, nz = args.hex_dims
    t0 = time.perf_counter()
    mesh = syn.box_hex(nx, ny, nz, jitter=0.1, seed=4)
    mat = syn.material_for(4, 0)
    setup = syn.setup_for(3, 4)
    I, P = syn.state_for(mesh, 4, 0)
    t_mesh = time.perf_counter() - t0
    t0 = time.perf_counter()
    fa = gm.FluidAssembly(mesh, mat, setup, device=dev.index or 0)
    t_create = time.perf_counter() - t0
    if args.hex_chunk:
        fa.set_chunk(args.hex_chunk)
    lp = fa.device_system(dev)
    nnz = lp.vals.numel()
    Id, Pd = torch.tensor(I, device=dev), torch.tensor(P, device=dev)
    dt = 1e-3
    s = torch.cuda.Stream(device=dev)
    sh = s.cuda_stream
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def sync_timed(form, k, warm):
        for _ in range(warm):
            fa.execute(Id, Pd, dt, lp, form=form, stream=sh)
        torch.cuda.synchronize(dev)
        a, b = ev(), ev()
        a.record(s)
        for _ in range(k):
            fa.execute(Id, Pd, dt, lp, form=form, stream=sh)
        b.record(s)
        torch.cuda.synchronize(dev)
        return a.elapsed_time(b) / k, fa.phase_ms(1)

    ms64, k64 = sync_timed(gm.FORM_FP64, max(1, args.fp64_steps - 1), 1)
    # error of the mixed form against the FP64 values this step left (norms in slices,
    # so the difference never needs a second full copy)
    with torch.cuda.stream(s):
        v64, b64 = lp.vals.clone(), lp.rhs.clone()
    ms_sync, k_mx = sync_timed(gm.FORM_MIXED, 2, 1)
    sl = 1 << 28
    dA = nA = 0.0
    for i in range(0, nnz, sl):
        d = lp.vals[i:i + sl] - v64[i:i + sl]
        dA += float(torch.dot(d, d))
        nA += float(torch.dot(v64[i:i + sl], v64[i:i + sl]))
        del d
    err = {"matrix": (dA / nA) ** 0.5, "rhs": float(torch.linalg.norm(lp.rhs - b64) / torch.linalg.norm(b64)),
           "reference": "the GPU FP64 form of this run"}
    del v64, b64
    # 10 Newton-iteration assemblies in one CUDA graph
    n_in_graph = 10
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s, capture_error_mode="thread_local"):
        for _ in range(n_in_graph):
            fa.enqueue(Id, Pd, dt, lp, form=gm.FORM_MIXED, stream=sh)
    for _ in range(max(1, args.warmup // 3)):
        g.replay()
    torch.cuda.synchronize(dev)
    reps = max(1, args.steps // 5)
    clk = ClockSampler(dev.index or 0) if with_clocks else None
    if clk:
        clk.__enter__()
    a, b = ev(), ev()
    a.record(s)
    with torch.cuda.stream(s):
        for _ in range(reps):
            g.replay()
    b.record(s)
    torch.cuda.synchronize(dev)
    if clk:
        clk.__exit__()
    fa.sync(stream=sh)
    ms_graph = a.elapsed_time(b) / (reps * n_in_graph)
    del g
    # objective VJP: lambda = dJ/dI of the top-face gas mass flux, gradient w.r.t. theta
    lam, Jval = top_gas_flux_lambda(mesh, mat, I, fa.nd)
    lamd = torch.tensor(lam, device=dev)
    gst = torch.zeros_like(Id)
    th = torch.zeros(3 * 4, dtype=torch.float64, device=dev)
    fa.vjp(Id, Pd, dt, lamd, gm.VJP_EXACT, gst, th, stream=sh)
    torch.cuda.synchronize(dev)
    vjp_ms = fa.device_ms()
    ne = mesh.n_elements
    hbm = peaks().get("hbm_gbs")
    ach = BYTES_PER_ELEM_HEX * ne / (k_mx * 1e-3) / 1e9
    out = {
        "workload": f"3D hex assembly, {ne} trilinear hexahedra ({nx}x{ny}x{nz}, 10% jitter), 4 components, "
                    f"8 dofs, 64x64 blocks, 10 mixed assemblies per CUDA graph",
        "n_elements": int(ne), "n_nodes": int(mesh.n_nodes), "nnz": int(nnz), "csr_values_gb": nnz * 8 / 1e9,
        "value": ne / (ms_graph * 1e-3), "unit": "elements/s", "ms_per_assembly": ms_graph,
        "graph_replays": reps, "assemblies_timed": reps * n_in_graph, "mixed_stream_ms": ms_sync,
        "fp64": {"value": ne / (ms64 * 1e-3), "unit": "elements/s", "ms_per_step": ms64, "interior_kernel_ms": k64},
        "mixed_over_fp64": ms64 / ms_graph,
        "mixed_rel_err_vs_fp64": err,
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                     "frac": ach / hbm if hbm else None, "traffic": TRAFFIC_BYTES_PER_ELEM_HEX * ne,
                     "traffic_source": "ncu DRAM bytes per element of the interior pass on 64,000 hexes x elements",
                     "kernel": "interior pass (point_kernel + matrix_kernel, mixed form)",
                     "kernel_ms": k_mx, "bytes_per_element": BYTES_PER_ELEM_HEX,
                     "peak_source": "measured (MEASURED_PEAKS.json)"},
        "objective_vjp": {"J": Jval, "ms": vjp_ms,
                          "dJdmu_via_lambda": [float(th[3 * c + 1]) for c in range(4)],
                          "note": "lambda = dJ/dU seeded VJP (the transpose solve is outside the path)"},
        "host_setup_s": {"mesh": t_mesh, "create": t_create},
        "device_memory_gb": torch.cuda.max_memory_allocated(dev) / 1e9,
    }
    if clk:
        out["clocks"] = clk.summary()
    fa.close()
    return out


def run_hex(args):
    """--workload hex: the hex workload as the line's headline."""
    import torch
    dev = torch.device("cuda", 0)
    importlib.import_module("gales-multi-fluid_gb300.build").build()
    h = hex_block(args, torch, dev, with_clocks=True)
    line = {"metric": METRIC, "value": h["value"], "unit": "elements/s", "n_gpus": 1,
            "steps": h["assemblies_timed"], "warmup": args.warmup, "ms_per_step": h["ms_per_assembly"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 element integrals + f64 EOS/tau/accumulation (mixed)", "data": "synthetic",
            "config": {"workload": h["workload"], "n_elements": h["n_elements"], "n_nodes": h["n_nodes"],
                       "dofs_per_node": 8, "nnz": h["nnz"], "csr_values_gb": h["csr_values_gb"],
                       "l2": "CSR values > L2", "seed": 0},
            "roofline": h["roofline"], "clocks": h.get("clocks"), "hex": h}
    print(json.dumps(line), flush=True)


def adaptive_dt_block(gm, fa, mesh, mat, setup, I, dt, torch, dev, with_cpu):
    """Adaptive time step (f_mc + set_dt) on the benchmark mesh: device state, per-call
    wall time including the 8-byte read-back of the minimum; the oracle on the first
    50,000 elements (one thread) beside it."""
    Id = torch.tensor(I, device=dev)
    d_el = torch.zeros(mesh.n_elements, dtype=torch.float64, device=dev)
    for _ in range(3):
        dt_new = fa.adaptive_dt(Id, dt, 0.5, 1e-6, 1.0, dt_el=d_el)
    torch.cuda.synchronize(dev)
    k = 10
    t0 = time.perf_counter()
    for _ in range(k):
        dt_new = fa.adaptive_dt(Id, dt, 0.5, 1e-6, 1.0, dt_el=d_el)
    ms = (time.perf_counter() - t0) / k * 1e3
    out = {"workload": "f_mc over the benchmark mesh, CFL 0.5, device state", "ms": ms,
           "elements_per_s": mesh.n_elements / (ms * 1e-3), "dt_new": dt_new}
    if with_cpu:
        import oracle
        n = min(mesh.n_elements, 50000)
        sub = gm.Mesh(mesh.coords, mesh.conn[:n], mesh.node_flag, mesh.el_on_boundary[:n],
                      mesh.bd_sides[mesh.bd_sides[:, 0] < n], name="sample")
        t0 = time.perf_counter()
        oracle.adaptive_dt(sub, mat, setup, I, dt, 0.5)
        out["cpu_oracle_elements_per_s"] = n / (time.perf_counter() - t0)
        out["cpu_oracle_cores"] = 1
    return out


def newton_block(gm, syn, mesh, mat, torch, dev):
    """Newton iterations of one time step (main.cpp:216-245) on the benchmark mesh,
    entirely on the GPU (newton.time_step_device: assembly, ||b|| on the device, the
    residual check of residual_check.hpp:42-80, flexible GMRES + ILU(1) with an FP32
    factor, corrector and dof trimmer), from the near-rest state (hydrostatic p, I = P).
    The FP64 tangent against the mixed tangent (residual in FP64):
      tau_2014: the reference's diagonal tau (dc_2006 on, sharpness 2), to the reference's
                criterion ||b|| <= 1e-8 ||b_0||, at most 8 iterations;
      tau_2019: the shipped non-diagonal tau with the shipped n_max_it = 3.  It enters the
                tangent frozen and its dependence on the state is not differentiated;
                the oracle's own loop (CPU assembly + exact solves) stalls the same way."""
    newton = importlib.import_module("gales-multi-fluid_gb300.newton")
    I0, _ = syn.state_near_rest(mesh, 3, 0)
    Id = torch.tensor(I0, device=dev)
    out = {"workload": f"{mesh.n_elements} tets, near-rest state, dt 1e-3, FGMRES(200)+ILU(1) FP32 factor, 1e-9"}
    for name, tau, max_it in (("tau_2014", gm.TAU_2014, 8), ("tau_2019_shipped", gm.TAU_2019, 3)):
        try:
            fa = gm.FluidAssembly(mesh, mat, syn.setup_for(3, 3, tau=tau), device=dev.index or 0)
            sol = fa.linear_solver(gm.SolverParams(precond=gm.PRECOND_ILU_FP32))
            lp = fa.device_system(dev)
            blk = {}
            for form, label, rform in ((gm.FORM_FP64, "fp64", None), (gm.FORM_MIXED, "mixed_tangent", gm.FORM_FP64)):
                torch.cuda.synchronize(dev)
                t0 = time.perf_counter()
                r = newton.time_step_device(fa, sol, Id, 1e-3, form, max_it=max_it, residual_form=rform, lp=lp)
                torch.cuda.synchronize(dev)
                blk[label] = {"converged": r["converged"], "iterations": r["iterations"],
                              "history": r["history"], "linear_iterations": r["linear_iterations"],
                              "s": time.perf_counter() - t0}
            blk["same_iterations"] = blk["fp64"]["iterations"] == blk["mixed_tangent"]["iterations"]
            out[name] = blk
            sol.close()
            fa.close()
        except Exception as e:  # reported, never fatal to the assembly line
            out[name] = {"error": f"{type(e).__name__}: {e}"}
    return out


def linear_solve_block(gm, fa, lp, torch, dev, tstream, with_cpu=True):
    """The linear solve after the assembly (belos_linear_solver::execute with the shipped
    setup.txt settings: flexible GMRES(200), 5 restarts, ILU(1), 1e-9) on the mixed-form
    system the timed steps left in device memory, with the factor in FP64 (the
    reference's arithmetic) and in FP32: wall time of the call (factorisation included),
    its factorisation alone and one preconditioner application; and the CPU oracle's
    solve beside the library's on a bounded sample."""
    out = {"what": "FGMRES(200) + ILU(1), rel. residual 1e-9, x0 = 0, device CSR of the mixed assembly",
           "rows": fa.n_rows}
    out["ilu_fp64"] = _solve_once(gm, fa, lp, torch, dev, tstream, gm.PRECOND_ILU)
    out["ilu_fp32"] = _solve_once(gm, fa, lp, torch, dev, tstream, gm.PRECOND_ILU_FP32)
    if with_cpu:
        out["cpu_oracle_sample"] = solve_cpu_sample(gm, torch, dev, tstream)
    return out


def solve_cpu_sample(gm, torch, dev, tstream, lattice=30):
    """The solve on a bounded sample beside the oracle's restatement on one host core:
    the FP64-form system of the 163,618-tet mesh of the 30^3 lattice (189,000 unknowns;
    same material, setup and kind of state as the benchmark), solved by the library
    (FP64 factor) and by the oracle's ILU(1) + flexible GMRES on the host (factorisation
    included in both)."""
    try:
        import oracle
        syn = importlib.import_module("gales-multi-fluid_gb300.synthetic")
        mesh = syn.box_tet_delaunay(lattice, seed=1)
        mat, setup = syn.material_for(3, 0), syn.setup_for(3, 3)
        I, P = syn.state_for(mesh, 3, 0)
        fa = gm.FluidAssembly(mesh, mat, setup, device=dev.index or 0)
        try:
            rows = fa.n_rows
            lp = fa.linear_system(device=dev)
            fa.execute(torch.tensor(I, device=dev), torch.tensor(P, device=dev), 1e-3, lp, form=gm.FORM_FP64,
                       stream=tstream.cuda_stream)
            torch.cuda.synchronize(dev)
            gpu = _solve_once(gm, fa, lp, torch, dev, tstream, gm.PRECOND_ILU)
            vals, rhs = lp.vals.cpu().numpy(), lp.rhs.cpu().numpy()
        finally:
            fa.close()
        t0 = time.perf_counter()
        _, info = oracle.fgmres(lp.row_ptr, lp.col, vals, rhs, tol=1e-9, maxsubspace=200, maxrestarts=5, fill=1)
        cpu_ms = (time.perf_counter() - t0) * 1e3
        gpu_ms = gpu.get("ms")
        return {"workload": f"{mesh.n_elements} tets ({lattice}^3 lattice), {rows} unknowns, FP64-form system",
                "cpu_cores": 1, "cpu_ms": cpu_ms, "cpu_iterations": info["iterations"],
                "cpu_rel_res": info["rel_res"], "gpu_ms": gpu_ms, "gpu_iterations": gpu.get("iterations"),
                "gpu_rel_res": gpu.get("rel_res"), "cpu_over_gpu": (cpu_ms / gpu_ms) if gpu_ms else None}
    except Exception as e:  # reported, never fatal to the assembly line
        return {"error": f"{type(e).__name__}: {e}"}


def _solve_once(gm, fa, lp, torch, dev, tstream, precond):
    stream = tstream.cuda_stream
    try:
        t0 = time.perf_counter()
        sol = fa.linear_solver(gm.SolverParams(precond=precond))
        create_s = time.perf_counter() - t0
        x = torch.zeros(fa.n_rows, dtype=torch.float64, device=dev)
        runs = []
        for _ in range(2):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            sol.solve(lp.vals, lp.rhs, x, stream=stream)
            runs.append(time.perf_counter() - t0)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        sol.factorize(lp.vals, stream=stream)
        torch.cuda.synchronize(dev)
        factor_ms = (time.perf_counter() - t0) * 1e3
        v = torch.ones(fa.n_rows, dtype=torch.float64, device=dev)
        z = torch.zeros_like(v)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sol.apply(v, z, stream=stream)
        e0.record(tstream)
        for _ in range(5):
            sol.apply(v, z, stream=stream)
        e1.record(tstream)
        torch.cuda.synchronize(dev)
        lf, lb = sol.levels()
        ms = min(runs) * 1e3
        return {"ms": ms, "iterations": sol.num_it, "rel_res": sol.RRE,
                "converged": sol.converged, "factor_ms": factor_ms,
                "apply_ms": e0.elapsed_time(e1) / 5, "levels_fwd_bwd": [lf, lb],
                "ms_per_iteration": (ms - factor_ms) / max(1, sol.num_it), "create_s": create_s}
    except Exception as e:  # reported, never fatal to the assembly line
        return {"error": f"{type(e).__name__}: {e}"}


def magma_block(torch, dev, with_cpu, n=4_000_000):
    """Magma mixture properties (two magma_mix components with synthetic solubility
    tables, Ishii-Zuber gas correction) at n device-resident (p, T, Y) points: CUDA-event
    time of the evaluation (the call also reads back a 4-byte status); the oracle on a
    20,000-point sample on one host core beside it."""
    try:
        magma = importlib.import_module("gales-multi-fluid_gb300.magma")
        syn = importlib.import_module("gales-multi-fluid_gb300.synthetic")
        comps = syn.magma_pair()
        mat = magma.MagmaMaterial(comps)
        g = torch.Generator(device="cpu").manual_seed(0)
        p = (6.1e7 + 2.38e8 * torch.rand(n, generator=g, dtype=torch.float64)).to(dev)
        T = (1150.0 + 300.0 * torch.rand(n, generator=g, dtype=torch.float64)).to(dev)
        y = torch.rand(n, generator=g, dtype=torch.float64)
        Y = torch.stack([y, 1.0 - y], 1).contiguous().to(dev)
        for _ in range(2):
            mat.properties(p, T, Y)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k = 5
        e0.record()
        for _ in range(k):
            mat.properties(p, T, Y)
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / k
        out = {"workload": f"{n} points, 2 magmas (mix_of_mix), 2401-point pressure tables, Ishii-Zuber",
               "ms": ms, "points_per_s": n / (ms * 1e-3)}
        if with_cpu:
            import oracle
            m = 20000
            t0 = time.perf_counter()
            oracle.magma_properties(comps, p[:m].cpu().numpy(), T[:m].cpu().numpy(), Y[:m].cpu().numpy())
            out["cpu_oracle_points_per_s"] = m / (time.perf_counter() - t0)
            out["cpu_oracle_cores"] = 1
        return out
    except Exception as e:  # reported, never fatal to the assembly line
        return {"error": f"{type(e).__name__}: {e}"}


def vjp_block(gm, syn, torch, dev, n=32):
    """Adjoint workload: ~200k tets, 3 components.  Exact and frozen VJP against the
    forward residual (FP64 and mixed), and the memory a stored-point design would need."""
    mesh = syn.box_tet_delaunay(n, seed=3)
    mat = syn.material_for(3, 0)
    setup = syn.setup_for(3, 3)
    I, P = syn.state_for(mesh, 3, 0)
    fa = gm.FluidAssembly(mesh, mat, setup)
    Id, Pd = torch.tensor(I, device=dev), torch.tensor(P, device=dev)
    lam = torch.tensor(np.random.default_rng(1).normal(size=I.size), device=dev)
    lam /= lam.norm()
    b = torch.zeros_like(Id)
    g = torch.zeros_like(Id)
    th = torch.zeros(9, dtype=torch.float64, device=dev)

    def t(f, k=5):
        for _ in range(2):
            f()
        torch.cuda.synchronize(dev)
        ms = []
        for _ in range(k):
            f()
            ms.append(fa.device_ms())
        return float(np.median(ms))

    r64 = t(lambda: fa.residual(Id, Pd, 1e-3, b, form=gm.FORM_FP64))
    rmx = t(lambda: fa.residual(Id, Pd, 1e-3, b, form=gm.FORM_MIXED))
    # the exact VJP keeps its per-point reverse-mode tape in registers and, beyond them,
    # in per-thread local memory, which the driver reserves for every thread the device
    # can hold when the kernel first runs: that reservation is the recompute design's
    # real footprint
    torch.cuda.synchronize(dev)
    free0 = torch.cuda.mem_get_info(dev)[0]
    fa.vjp(Id, Pd, 1e-3, lam, gm.VJP_EXACT, g, th)
    torch.cuda.synchronize(dev)
    local_reserved = max(0, free0 - torch.cuda.mem_get_info(dev)[0])
    ex = t(lambda: fa.vjp(Id, Pd, 1e-3, lam, gm.VJP_EXACT, g, th))
    fr = t(lambda: fa.vjp(Id, Pd, 1e-3, lam, gm.VJP_FROZEN, g))
    nq = 4
    return {"workload": f"{mesh.n_elements} Delaunay tets ({n}^3 lattice), 3 components, lambda a seeded unit vector",
            "exact_ms": ex, "frozen_ms": fr, "residual_fp64_ms": r64, "residual_mixed_ms": rmx,
            "exact_over_residual_fp64": ex / r64, "exact_over_residual_mixed": ex / rmx,
            "memory": {"recompute_extra_bytes": int(local_reserved),
                       "store_points_bytes": int(mesh.n_elements * nq * 8 * 360),
                       "note": "recompute: the device-wide local-memory reservation of the exact VJP kernel "
                               "(its spilled per-thread tape, independent of the mesh size), measured as the "
                               "drop in free device memory at its first launch; store: ~360 doubles of forward "
                               "tape per point"}}


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
    ap.add_argument("--no-solve", action="store_true", help="skip the linear solve after the assembly")
    ap.add_argument("--lattice", type=int, default=LATTICE_N, help="lattice points per side (54 -> 1.0M tets)")
    ap.add_argument("--only", default="both", choices=["both", "mixed", "fp64"],
                    help="profiling aid: run only one form (no e2e, no CPU leg)")
    ap.add_argument("--workload", default="tet", choices=["tet", "hex"],
                    help="tet: 1.0M tets (default); hex: 4.0M hexahedra with a CUDA graph of 10 assemblies")
    ap.add_argument("--hex-dims", type=int, nargs=3, default=[160, 160, 156])
    ap.add_argument("--hex-chunk", type=int, default=0,
                    help="hex elements per interior chunk (0: as many as the record buffer holds)")
    ap.add_argument("--no-vjp", action="store_true", help="skip the adjoint block")
    ap.add_argument("--no-hex", action="store_true", help="skip the 4.0M-hex block")
    ap.add_argument("--no-newton", action="store_true", help="skip the Newton block")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "hex":
        return run_hex(args)

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
        kern, stages = [], []
        launches0 = fa.launch_count()
        e0.record(stream)
        for _ in range(k):
            step(form)
            kern.append(fa.phase_ms(1))
            stages.append((fa.phase_ms(3), fa.phase_ms(4)))
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = max_over_ranks(e0.elapsed_time(e1) / k, dist, dev)
        timed.stages = (statistics.median(x[0] for x in stages), statistics.median(x[1] for x in stages))
        return ms, statistics.median(kern), fa.launch_count() - launches0

    ms64, k64, _ = timed(gm.FORM_FP64, args.fp64_steps, 1)
    with ClockSampler(local) as clk:
        ms_mx, k_mx, launches = timed(gm.FORM_MIXED, args.steps, args.warmup)
    clocks = clk.summary()
    point_ms, matrix_ms = timed.stages

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
    # a host-buffer call returns when A and b are in host memory, so each step is timed
    # on its own as well as the whole run
    # six times the device-buffer step count (each step ~9 ms), so that one slow step
    # on the shared host link (single steps of 20-60 ms have been seen) weighs less in
    # the mean; every step is counted
    e2e_n = 6 * args.steps
    e2e_steps = []
    gc.collect()
    gc.disable()      # no collector pause of the Python host loop inside the timing
    t0 = time.perf_counter()
    for _ in range(e2e_n):
        ts = time.perf_counter()
        fa.execute(Ih, Ph, dt, lph, form=gm.FORM_MIXED, stream=sh)
        e2e_steps.append((time.perf_counter() - ts) * 1e3)
    torch.cuda.synchronize(dev)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_n, dist, dev)
    gc.enable()
    # the device-to-host copy of the CSR values alone (same pinned buffer and stream)
    d0, d1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        lph.vals.copy_(lp.vals, non_blocking=True)
        d0.record(stream)
        for _ in range(3):
            lph.vals.copy_(lp.vals, non_blocking=True)
        d1.record(stream)
    torch.cuda.synchronize(dev)
    d2h_ms = d0.elapsed_time(d1) / 3

    ne = mesh.n_elements
    value = whole_job_rate(ne, ms_mx, world)
    pk = peaks()
    hbm = pk.get("hbm_gbs")
    achieved = BYTES_PER_ELEM_TET * ne / (k_mx * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mx, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 element integrals + f64 EOS/tau/accumulation (mixed)",
        "data": "synthetic", "config": workload_config(mesh, args.lattice),
        "fp64": {"value": whole_job_rate(ne, ms64, world), "unit": "elements/s", "ms_per_step": ms64,
                 "interior_kernel_ms": k64},
        "mixed_over_fp64": ms64 / ms_mx,
        "mixed_rel_err_vs_fp64": {"matrix": err_A, "rhs": err_b,
                                  "reference": "the GPU FP64 form of this run, which the -m gpu tests check "
                                               "against the oracle on this mesh (<= 1e-12)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if hbm else None, "traffic": TRAFFIC_BYTES_PER_ELEM_TET * ne,
                     "traffic_source": "ncu DRAM bytes per element of the interior pass on 163,618 tets x elements",
                     "kernel": "interior pass (point_kernel + matrix_kernel, mixed form)", "kernel_ms": k_mx,
                     "bytes_per_element": BYTES_PER_ELEM_TET, "peak_source": "measured (MEASURED_PEAKS.json)"},
        "e2e": {"value": whole_job_rate(ne, e2e_s * 1e3, world), "unit": "elements/s",
                "h2d_bytes_per_step": 2 * fa.n_rows * 8, "d2h_bytes_per_step": (nnz + fa.n_rows) * 8,
                "ms_per_step": e2e_s * 1e3,
                "steps": e2e_n,
                "step_ms": {"median": statistics.median(e2e_steps), "min": min(e2e_steps),
                            "max": max(e2e_steps)},
                "over_device_buffers": (e2e_s * 1e3) / ms_mx,
                "d2h_values_alone_ms": d2h_ms, "d2h_gbs": nnz * 8 / (d2h_ms * 1e-3) / 1e9,
                "note": "a host-buffer call ends with the copy of the CSR values to the host; the rows are "
                        "copied while the pass runs, chunk by chunk, so the step is bound by the larger of "
                        "the assembly and the copy of all values (d2h_values_alone_ms)"},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "compute": compute_roofline(ne, point_ms, matrix_ms),
    }
    if rank == 0 and not args.no_vjp:
        syn = importlib.import_module("gales-multi-fluid_gb300.synthetic")
        line["vjp"] = vjp_block(gm, syn, torch, dev)
    if rank == 0:
        line["adaptive_dt"] = adaptive_dt_block(gm, fa, mesh, mat, setup, I, dt, torch, dev, not args.no_cpu)
    if rank == 0 and not args.no_solve:
        line["linear_solve"] = linear_solve_block(gm, fa, lp, torch, dev, stream, not args.no_cpu)
    if rank == 0:
        line["magma_properties"] = magma_block(torch, dev, not args.no_cpu)
    if rank == 0 and not args.no_newton:
        syn = importlib.import_module("gales-multi-fluid_gb300.synthetic")
        line["newton"] = newton_block(gm, syn, mesh, mat, torch, dev)
    if rank == 0 and not args.no_hex:
        # the hex workload after the tet workload's buffers are released
        del lph, Ih, Ph
        fa.close()
        lp = None
        torch.cuda.empty_cache()
        try:
            line["hex"] = hex_block(args, torch, dev)
        except Exception as e:  # reported, never fatal to the assembly line
            line["hex"] = {"error": f"{type(e).__name__}: {e}"}
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
