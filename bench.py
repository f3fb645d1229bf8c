"""Benchmark: matrix-free GMG Stokes solve, FP32-MG vs FP64-MG at a 1e-8 FP64 residual.

Workload (one step = one Stokes solve from a zero initial guess): 3D unit cube,
32^3 Q2-Q1 cells (823,875 velocity + 35,937 pressure DoFs, 6 levels), 8 smooth
sinkers (centres seeded SplitMix64 20261206), viscosity
1e-6 + (1-1e-6) prod_i(1 - exp(-d_i^2/(2 0.05^2))) (1e6 contrast), per-quadrature-point viscosity with the Q1 projection (ASPECT's default
averaging for GMG), free slip, FGMRES (restart 100) with the block-Schur
preconditioner and an FP32 V-cycle, FP64 outer residual, relative tolerance 1e-8.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
    python bench.py --profile-op a_cell_pass_fp32|stokes_cell_pass_fp64|stokes_vmult_fp64|mass_vmult_fp32|a_vmult_fp32
    python bench.py --sweep 32,64      (operator timings per size, no solve)
    python bench.py --configs solcx64,sphere16,adjoint32,shell3   (FP64-MG vs FP32-MG per workload)

(--profile-op runs one operation of the workload three times between
cudaProfilerStart/Stop, for `ncu --profile-from-start off` captures.)

`value` is DoFs solved per second with inputs resident in HBM (device-timed);
`e2e` is the same through the host-array C ABI (gb_gmg_solve) with the host<->device
copies inside the timed region. `--impl reference` times the CPU oracle (the
FP64-MG restatement of the reference algorithm) on the host cores.
N > 1 runs independent replicas (the solve does not shard; one GPU each).
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

METRIC = "Stokes solve time & operator GDoF/s: FP32-MG vs FP64-MG at 1e-8 FP64 residual"
WORKLOAD = "sinkers_32^3_Q2Q1_eta1e6_q1proj_fgmres_fp32mg_tol1e-8"
TOL = 1e-8
N_CELLS_1D = 32
# Algorithmic arithmetic per cell (the unit of the FP rooflines), counted by
# the sum-factorisation formula of the operator, not from any kernel's
# instructions (an FMA counts 2): A block = 3 components x 6 sweeps x 81 FMA x
# 2 (evaluate and integrate) x 2 + 27 points x 40 = 6,912; the Stokes operator
# adds the Q1 pressure by sum factorisation (3 sweeps of 2 -> 3 points each
# way, 2 x 114 FMA) and about 10 flop per point: 6,912 + 456 + 270 = 7,638.
ALG_FLOPS_A_CELL = 6912
ALG_FLOPS_STOKES_CELL = 7638
# dram__bytes_read.sum + dram__bytes_write.sum of one finest-level launch of the
# FP64 Stokes cell pass at 32^3 (ncu --metrics dram__bytes_read.sum,
# dram__bytes_write.sum of `bench.py --profile-op stokes_cell_pass_fp64`, two
# launches: 13,968,128 and 13,968,384 bytes read, 0 written -- the reads of u, p
# and eta; the per-cell contributions stay in L2)
STOKES_CELL_PASS_F64_DRAM_BYTES = 13968256


def measured_fp_peaks():
    """FP64 and FP32 FMA throughput of this GPU in TFLOP/s, measured live by the
    FMA-chain probe (aspect_gb300/csrc/peak_probe.cu, libgb_probe.so)."""
    import ctypes
    lib = ctypes.CDLL(os.path.join(ROOT, "aspect_gb300", "libgb_probe.so"))
    out = {}
    for key, fn in (("fp64", lib.gb_probe_fp64_fma_tflops), ("fp32", lib.gb_probe_fp32_fma_tflops)):
        v = ctypes.c_double()
        fn.argtypes = [ctypes.POINTER(ctypes.c_double)]
        best = 0.0
        for _ in range(3):
            if fn(ctypes.byref(v)) == 0:
                best = max(best, v.value)
        out[key] = best
    return out


def log(*a):
    print(f"[bench {time.strftime('%H:%M:%S')}]", *a, file=sys.stderr, flush=True)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if "Active" in s[3 + i]
                          and "Not" not in s[3 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def job_throughput(seconds_local: float, units_per_rank: float, device=None) -> tuple[float, float]:
    """Whole-job figures of N replicas: the timed seconds are the maximum over
    ranks (an all_reduce MAX when a process group is up, on `device`: a CUDA
    device under NCCL, the CPU under gloo) and the throughput is the units all
    ranks processed divided by that time. Returns (seconds, units per second)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    t = float(seconds_local)
    if world > 1:
        tt = torch.tensor([t], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    return t, world * units_per_rank / t


def build_problem():
    from aspect_gb300 import problems
    return problems.sinkers_3d(N_CELLS_1D)


def algorithmic_bytes(P, op: str, word: int) -> int:
    """Compulsory bytes of one operator application (src + dst vectors + viscosity
    table); DoF indices and constraints are not counted."""
    f = P.fine
    eta_words = f.n_cells * (27 if P.projection == 1 else 1)
    if op == "stokes":
        n = f.n_u + f.n_p
    elif op == "A":
        n = f.n_u
    else:
        n = f.n_p
    return 2 * n * word + eta_words * word


def cpu_solves(P, n_threads: int, mg_float: bool, n_solves: int):
    """Full converged solves of the workload on the host cores with the CPU
    restatement of the reference algorithm (oracle, fast mode: sum-factorised
    cell operators as in the reference's deal.II code, OpenMP over colour-ordered
    cells). Returns (seconds of each solve, outputs of the last)."""
    import oracle
    from oracle import Oracle
    oracle.set_fast(True)
    o = Oracle(P.levels, n_threads=n_threads)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    o.build_preconditioner(mg_float)
    times, info = [], None
    for _ in range(n_solves):
        t = time.perf_counter()
        _, info = o.solve(P.rhs, tol_rel=TOL)
        times.append(time.perf_counter() - t)
        if info["status"] != 0:
            raise RuntimeError(f"CPU solve did not converge: {info}")
    return times, info


def cpu_baseline(P, n_threads: int):
    """One full FP64-MG and one full FP32-MG solve on the host cores."""
    t64, i64 = cpu_solves(P, n_threads, False, 1)
    t32, i32 = cpu_solves(P, n_threads, True, 1)
    return {"fp64_mg": {"seconds": t64[0], "iterations": i64["cheap_iterations"] + i64["expensive_iterations"],
                        "mdofs": P.n_dofs / t64[0] / 1e6},
            "fp32_mg": {"seconds": t32[0], "iterations": i32["cheap_iterations"] + i32["expensive_iterations"],
                        "mdofs": P.n_dofs / t32[0] / 1e6}}


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's FP64-MG solve
    (GMGNumberType = double), all host cores, one full solve to 1e-8 per step;
    after the timed steps one FP32-MG solve (GMGNumberType = float)."""
    world, rank, _ = dist_init()
    if world > 1 and rank != 0:
        return
    P = build_problem()
    threads = os.cpu_count() or 1
    times, info = cpu_solves(P, threads, False, args.warmup + args.steps)
    timed = times[args.warmup:]
    its = info["cheap_iterations"] + info["expensive_iterations"]
    value = len(timed) * P.n_dofs / sum(timed) / 1e6
    t32, i32 = cpu_solves(P, threads, True, 1)
    sample = (f"full FP64-MG solves of the same 32^3 workload to 1e-8 ({its} GMRES iterations each), one per step; "
              f"CPU restatement of the reference algorithm, sum-factorised cell operators, OpenMP over "
              f"colour-ordered cells")
    line = {"metric": METRIC, "impl": "reference", "value": value, "unit": "MDoF/s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(timed) / len(timed) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD.replace("fgmres_fp32mg", "gmres_fp64mg"), "n_dofs": P.n_dofs,
                       "iterations": its},
            "cpu_baseline": {"value": value, "unit": "MDoF/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "MDoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "detail": {"seconds_per_solve": timed,
                       "fp32_mg": {"seconds": t32[0], "iterations": i32["cheap_iterations"] + i32["expensive_iterations"],
                                   "mdofs": P.n_dofs / t32[0] / 1e6}}}
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch
    from aspect_gb300 import gmg

    world, rank, local = dist_init()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    P = build_problem()
    f = P.fine
    n = P.n_dofs
    log("problem built", n)
    # set-up in the handler's phases: setup_dofs (once per mesh), assemble (set
    # the viscosity: once per nonlinear iteration in ASPECT) and
    # build_preconditioner (diagonals and eigenvalue estimates of the FP32
    # levels and the explicit coarse sub-cycles; the FP64 levels and the V-cycle
    # graphs follow on first use: also once per nonlinear iteration)
    t0 = time.perf_counter()
    g = gmg.StokesMatrixFreeGPU(3, len(P.levels))
    g.setup_dofs(P.levels)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    g.assemble(P.eta, P.projection, P.pressure_scaling)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    g.build_preconditioner()
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    setup = {"setup_dofs_s": t1 - t0, "assemble_s": t2 - t1, "build_preconditioner_s": t3 - t2}
    setup_s = t3 - t0
    log("setup done", setup)

    rhs_d = torch.from_numpy(P.rhs).to(dev)
    sol_d = torch.zeros(n, dtype=torch.float64, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > 129 MB L2
    params = dict(linear_solver_tolerance=TOL, mg_precision=gmg.FP32, krylov=gmg.GMRES)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        sol_d.zero_()
        o = g.solve_device(rhs_d.data_ptr(), sol_d.data_ptr(), **params)
        log("warmup solve", o)
    barrier()
    launches0 = g.kernel_launches()
    step_s, outs = [], []
    torch.cuda.profiler.start()  # ncu --profile-from-start off captures the timed solves only
    with ClockSampler(local) as clk:
        barrier()
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            sol_d.zero_()
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            out = g.solve_device(rhs_d.data_ptr(), sol_d.data_ptr(), **params)
            e1.record()
            torch.cuda.synchronize()
            step_s.append(e0.elapsed_time(e1) * 1e-3)
            outs.append(out)
        barrier()
        wall = time.perf_counter() - wall0
    torch.cuda.profiler.stop()
    launches = g.kernel_launches() - launches0
    log("timed solves", step_s)
    t_sum, value = job_throughput(sum(step_s), args.steps * n, dev)
    value /= 1e6
    mixed = outs[-1]

    # --- end to end through the host-array ABI (pinned host buffers)
    rhs_h = torch.from_numpy(P.rhs.copy()).pin_memory()
    sol_h = torch.zeros(n, dtype=torch.float64).pin_memory()
    import ctypes
    e2e_s = []
    for _ in range(max(1, min(args.steps, 3))):
        sol_h.zero_()
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t = time.perf_counter()
        prm = gmg.default_solve_params(**params)
        o = gmg.Outputs()
        g._chk(g.L.gb_gmg_solve(g.h, ctypes.c_void_p(rhs_h.data_ptr()), ctypes.c_void_p(sol_h.data_ptr()),
                                ctypes.byref(prm), ctypes.byref(o)))
        torch.cuda.synchronize()
        e2e_s.append(time.perf_counter() - t)
    e2e_value = world * n / statistics.median(e2e_s) / 1e6

    # --- FP64-MG comparison and the iterative-refinement variant (one timed solve each)
    def timed_solve(**kw):
        sol_d.zero_()
        g.solve_device(rhs_d.data_ptr(), sol_d.data_ptr(), **kw)  # warm
        sol_d.zero_()
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        o = g.solve_device(rhs_d.data_ptr(), sol_d.data_ptr(), **kw)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e-3, o, sol_d.clone()

    t64, o64, x64 = timed_solve(linear_solver_tolerance=TOL, mg_precision=gmg.FP64)
    log("fp64-mg solve", t64, o64)
    tir, oir, xir = timed_solve(linear_solver_tolerance=TOL, mg_precision=gmg.FP32, krylov=gmg.GMRES_IR)
    log("gmres-ir solve", tir, oir)
    tidr, oidr, xidr = timed_solve(linear_solver_tolerance=TOL, mg_precision=gmg.FP32, krylov=gmg.IDR, idr_s=2)
    log("idr(2) solve", tidr, oidr)
    tgs, ogs, xgs = timed_solve(**dict(params, orthogonalization=1))
    log("mixed solve, FP64 Gram-Schmidt passes", tgs, ogs)
    _, _, x32 = timed_solve(**params)
    rel = lambda a, b: float(torch.linalg.norm(a[: f.n_u] - b[: f.n_u]) / torch.linalg.norm(b[: f.n_u]))

    # --- operator timings (stokes_vmult etc.) and the roofline of the dominant kernel
    ops = {}
    for name, what, prec in [("stokes_vmult_fp64", gmg.TIME_STOKES_VMULT, gmg.FP64),
                             ("stokes_vmult_fp32", gmg.TIME_STOKES_VMULT, gmg.FP32),
                             ("A_vmult_fp32", gmg.TIME_A_VMULT, gmg.FP32),
                             ("A_vmult_fp64", gmg.TIME_A_VMULT, gmg.FP64),
                             ("mass_vmult_fp32", gmg.TIME_MASS_VMULT, gmg.FP32),
                             ("stokes_preconditioner_fp32", gmg.TIME_STOKES_PRECONDITIONER, gmg.FP32),
                             ("stokes_preconditioner_fp64", gmg.TIME_STOKES_PRECONDITIONER, gmg.FP64),
                             ("A_preconditioner_fp32", gmg.TIME_A_PRECONDITIONER, gmg.FP32),
                             ("S_preconditioner_fp32", gmg.TIME_S_PRECONDITIONER, gmg.FP32)]:
        flush.fill_(1.0)
        torch.cuda.synchronize()
        ops[name] = g.time_operation(what, prec, 20)
    gdofs = {"stokes_vmult_fp64": n / ops["stokes_vmult_fp64"] / 1e9,
             "stokes_vmult_fp32": n / ops["stokes_vmult_fp32"] / 1e9,
             "A_vmult_fp32": f.n_u / ops["A_vmult_fp32"] / 1e9,
             "A_vmult_fp64": f.n_u / ops["A_vmult_fp64"] / 1e9}
    # --- rooflines, each kernel timed alone on the finest level with CUDA events
    # on the library's stream, against peaks measured on this GPU: the FP64
    # Stokes cell pass (the FGMRES matrix-vector product; the largest share of
    # the solve's launch list) is bound by the FP64 pipe, the FP32 A-block
    # operator (every V-cycle level) by the FP32 pipe at this arithmetic
    # intensity (~35 flop per compulsory byte against a ridge near 12)
    fp = measured_fp_peaks()
    log("measured FMA peaks (TFLOP/s)", fp)
    peak, peak_kind = peaks()
    eta_words = f.n_cells * (27 if P.projection == 1 else 1)
    t_sc = g.time_operation(gmg.TIME_STOKES_CELL_PASS, gmg.FP64, 20)
    t_s64 = ops["stokes_vmult_fp64"]
    t_a32 = ops["A_vmult_fp32"]
    flops_sc = ALG_FLOPS_STOKES_CELL * f.n_cells
    flops_a = ALG_FLOPS_A_CELL * f.n_cells
    bytes_s64 = 8 * (2 * n + eta_words)      # compulsory: u, p in and out, eta
    bytes_a32 = 4 * (2 * f.n_u + eta_words)  # compulsory: u in and out, eta
    clocks = clk.summary()

    if rank != 0:
        return
    its_mixed = mixed["cheap_iterations"] + mixed["expensive_iterations"]
    its64 = o64["cheap_iterations"] + o64["expensive_iterations"]
    log("operators", ops)
    cpu = cpu_baseline(P, os.cpu_count() or 1)
    log("cpu baseline", cpu)
    line = {
        "metric": METRIC, "value": value, "unit": "MDoF/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_sum / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (V-cycle) / f64 (Krylov, Stokes residual)",
        "data": f"synthetic: 8 sinkers seeded SplitMix64({P.extra['seed']})",
        "config": {"workload": WORKLOAD, "cells": f.n_cells, "n_u": f.n_u, "n_p": f.n_p, "levels": len(P.levels),
                   "tolerance": TOL, "krylov": "FGMRES(100), FP64", "mg": "FP32 V-cycle, Chebyshev(4)",
                   "gram_schmidt": "classical, conditional second pass; float-pair products (~46 bits)",
                   "l2": "flushed between timed solves (256 MiB write)", "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": "MDoF/s", "h2d_bytes_per_step": 2 * n * 8, "d2h_bytes_per_step": n * 8,
                "solves": len(e2e_s), "seconds_per_solve": e2e_s},
        "gpu_launches": launches,
        "roofline": {"bound": "fp64", "kernel": "lattice_iso_kernel_f64<STOKES> (FP64 Stokes cell pass, 32^3 "
                                                 "finest level, 3 threads per cell)",
                     "achieved": flops_sc / t_sc / 1e12, "peak": fp["fp64"], "unit": "TFLOP/s",
                     "frac": flops_sc / t_sc / 1e12 / fp["fp64"],
                     "peak_kind": "measured (FP64 FMA-chain probe, libgb_probe.so, this run)",
                     "traffic": STOKES_CELL_PASS_F64_DRAM_BYTES, "algorithmic_flops_per_launch": flops_sc,
                     "flops_per_cell": ALG_FLOPS_STOKES_CELL, "seconds_per_launch": t_sc,
                     "hbm": {"operator": "FP64 Stokes vmult (cell pass + gathers)", "seconds": t_s64,
                             "algorithmic_bytes": bytes_s64, "achieved": bytes_s64 / t_s64 / 1e9, "peak": peak,
                             "unit": "GB/s", "frac": bytes_s64 / t_s64 / 1e9 / peak, "peak_kind": peak_kind}},
        "roofline_fp32_a_vmult": {
            "bound": "fp32", "kernel": "FP32 A-block vmult, 32^3 finest level (lattice cell pass + gather)",
            "achieved": flops_a / t_a32 / 1e12, "peak": fp["fp32"], "unit": "TFLOP/s",
            "frac": flops_a / t_a32 / 1e12 / fp["fp32"], "peak_kind": "measured (FP32 FMA-chain probe)",
            "seconds_per_application": t_a32, "flops_per_cell": ALG_FLOPS_A_CELL,
            "hbm": {"algorithmic_bytes": bytes_a32, "achieved": bytes_a32 / t_a32 / 1e9, "peak": peak,
                    "unit": "GB/s", "frac": bytes_a32 / t_a32 / 1e9 / peak, "peak_kind": peak_kind},
            "note": "all operands L2-resident at 32^3; the 64^3 / 128^3 sweep (bench.py --sweep) gives the "
                    "HBM-resident figures"},
        "cpu_baseline": {"value": cpu["fp64_mg"]["mdofs"], "unit": "MDoF/s", "cores": os.cpu_count(),
                         "kind": "port",
                         "sample": f"one full FP64-MG solve of the same 32^3 workload to 1e-8 "
                                   f"({cpu['fp64_mg']['iterations']} iterations, {cpu['fp64_mg']['seconds']:.2f} s), "
                                   f"CPU restatement of the reference algorithm (sum-factorised cell operators); "
                                   f"FP32-MG: {cpu['fp32_mg']['seconds']:.2f} s, {cpu['fp32_mg']['iterations']} "
                                   f"iterations",
                         "fp32_mg": cpu["fp32_mg"]},
        "clocks": clocks,
        "detail": {
            "setup_seconds": setup_s, "setup_phases": setup, "wall_seconds_timed": wall,
            "mixed": {"solve_s": t_sum / args.steps, "iterations": its_mixed,
                      "fp64_stokes_applications": mixed["fp64_stokes_applications"],
                      "final_residual": mixed["final_linear_residual"], "tolerance": mixed["solver_tolerance"]},
            "fp64_mg": {"solve_s": t64, "iterations": its64, "final_residual": o64["final_linear_residual"]},
            "speedup_mixed_vs_fp64_mg": t64 / (t_sum / args.steps),
            "gmres_ir": {"solve_s": tir, "iterations": oir["cheap_iterations"],
                         "fp64_stokes_applications": oir["fp64_stokes_applications"],
                         "speedup_vs_fp64_mg": t64 / tir},
            "idr2_fp32mg": {"solve_s": tidr, "iterations": oidr["cheap_iterations"] + oidr["expensive_iterations"],
                            "A_preconditioner_applications": oidr["A_preconditioner_applications"],
                            "fp64_stokes_applications": oidr["fp64_stokes_applications"],
                            "speedup_vs_fp64_mg": t64 / tidr},
            "mixed_fp64_gram_schmidt": {"solve_s": tgs, "iterations": ogs["cheap_iterations"],
                                        "velocity_rel_l2_vs_float_pair": rel(xgs, x32)},
            "velocity_rel_l2_vs_fp64_mg": {"mixed": rel(x32, x64), "gmres_ir": rel(xir, x64),
                                           "idr2": rel(xidr, x64)},
            "operator_seconds": ops, "operator_gdofs": gdofs,
            "solve_share_seconds": {"stokes_vmult_fp64": mixed["fp64_stokes_applications"] * t_s64},
        },
    }
    print(json.dumps(line), flush=True)


PROFILE_OPS = {"a_cell_pass_fp32": ("TIME_A_CELL_PASS", "FP32"), "a_vmult_fp32": ("TIME_A_VMULT", "FP32"),
               "stokes_cell_pass_fp64": ("TIME_STOKES_CELL_PASS", "FP64"),
               "stokes_vmult_fp64": ("TIME_STOKES_VMULT", "FP64"), "mass_vmult_fp32": ("TIME_MASS_VMULT", "FP32"),
               "s_preconditioner_fp32": ("TIME_S_PRECONDITIONER", "FP32"),
               "a_preconditioner_fp32": ("TIME_A_PRECONDITIONER", "FP32"),
               "build_preconditioner": (None, None), "solve_fp32": (None, None)}


def run_profile_op(name: str):
    """One operation of the workload, three times (a solve or the preconditioner
    set-up once) inside cudaProfilerStart/Stop, for ncu --profile-from-start off."""
    import torch
    from aspect_gb300 import gmg
    torch.cuda.init()
    P = build_problem()
    g = gmg.from_problem(P)
    if name == "build_preconditioner":
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        t0 = time.perf_counter()
        g.build_preconditioner()
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        torch.cuda.profiler.stop()
    elif name == "solve_fp32":
        g.solve(P.rhs, linear_solver_tolerance=TOL, mg_precision=gmg.FP32)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        _, out = g.solve(P.rhs, linear_solver_tolerance=TOL, mg_precision=gmg.FP32)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        sec = out["solve_seconds"]
    else:
        what, prec = getattr(gmg, PROFILE_OPS[name][0]), getattr(gmg, PROFILE_OPS[name][1])
        g.time_operation(what, prec, 3)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        sec = g.time_operation(what, prec, 3)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    print(json.dumps({"profile_op": name, "seconds_per_call": sec, "cells": P.fine.n_cells}), flush=True)


def run_sweep(sizes):
    """Operator timings of the sinker workload at several sizes (no solve). At 32^3
    every operand is L2-resident; from 64^3 on the FP32 A-block operator's vectors
    and viscosity exceed the 129 MB L2, so its HBM fraction means something. Bytes
    are the compulsory ones (vectors in and out, viscosity table); flops the
    algorithmic sum-factorisation counts. One JSON line per size."""
    import torch
    from aspect_gb300 import gmg, problems
    torch.cuda.init()
    peak, peak_kind = peaks()
    fp = measured_fp_peaks()
    for nc in sizes:
        t0 = time.perf_counter()
        P = problems.sinkers_3d(nc)
        t_problem = time.perf_counter() - t0
        g = gmg.from_problem(P, build=False)
        f = P.fine
        n = P.n_dofs
        eta_words = f.n_cells * (27 if P.projection == 1 else 1)
        t = {k: g.time_operation(getattr(gmg, w), getattr(gmg, pr), 20)
             for k, w, pr in [("A_vmult_fp32", "TIME_A_VMULT", "FP32"), ("A_cell_pass_fp32", "TIME_A_CELL_PASS", "FP32"),
                              ("stokes_vmult_fp64", "TIME_STOKES_VMULT", "FP64"),
                              ("stokes_cell_pass_fp64", "TIME_STOKES_CELL_PASS", "FP64"),
                              ("mass_vmult_fp32", "TIME_MASS_VMULT", "FP32")]}
        b = {"A_vmult_fp32": 4 * (2 * f.n_u + eta_words),
             "A_cell_pass_fp32": 4 * (f.n_u + eta_words),
             "stokes_vmult_fp64": 8 * (2 * n + eta_words),
             "stokes_cell_pass_fp64": 8 * (n + eta_words),
             "mass_vmult_fp32": 4 * (2 * f.n_p + eta_words)}
        fl = {"A_vmult_fp32": ("fp32", ALG_FLOPS_A_CELL), "A_cell_pass_fp32": ("fp32", ALG_FLOPS_A_CELL),
              "stokes_vmult_fp64": ("fp64", ALG_FLOPS_STOKES_CELL),
              "stokes_cell_pass_fp64": ("fp64", ALG_FLOPS_STOKES_CELL)}
        line = {"sweep": f"sinkers_{nc}^3", "cells": f.n_cells, "n_u": f.n_u, "n_p": f.n_p, "peak_gbs": peak,
                "peak_kind": peak_kind, "peak_tflops": fp, "host_problem_seconds": t_problem, "ops": {}}
        for k in t:
            gbs = b[k] / t[k] / 1e9
            row = {"seconds": t[k], "algorithmic_bytes": b[k], "gbs": gbs, "hbm_frac": gbs / peak,
                   "gdofs": (f.n_u if k.startswith("A") else (f.n_p if k.startswith("mass") else n)) / t[k] / 1e9}
            if k in fl:
                kind, per_cell = fl[k]
                tf = per_cell * f.n_cells / t[k] / 1e12
                row.update({f"{kind}_tflops": tf, f"{kind}_frac": tf / fp[kind]})
            line["ops"][k] = row
        print(json.dumps(line), flush=True)
        del g


def _solve_pair(P, options=None, project=None, oracle_residual=False):
    """FP64-MG and FP32-MG solves of one workload (each timed after a warm-up solve);
    oracle_residual: also the FP64 residual of both solutions, measured by the CPU
    oracle (the checker) on the same level meshes."""
    from aspect_gb300 import gmg
    t0 = time.perf_counter()
    g = gmg.from_problem(P, options)
    setup = time.perf_counter() - t0
    res = {}
    for key, prec in (("fp64_mg", gmg.FP64), ("fp32_mg", gmg.FP32)):
        g.solve(P.rhs, linear_solver_tolerance=TOL, mg_precision=prec)  # warm
        x, o = g.solve(P.rhs, linear_solver_tolerance=TOL, mg_precision=prec)
        res[key] = {"solve_s": o["solve_seconds"], "iterations": o["cheap_iterations"] + o["expensive_iterations"],
                    "status": o["status"], "tolerance": o["solver_tolerance"],
                    "final_residual": o["final_linear_residual"], "x": x}
    f = P.fine
    u64, u32 = res["fp64_mg"]["x"][: f.n_u], res["fp32_mg"]["x"][: f.n_u]
    if project is not None:
        u64, u32 = project(u64), project(u32)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    line = {"workload": P.name, "cells": f.n_cells, "n_u": f.n_u, "n_p": f.n_p, "setup_s": setup,
            "delta_iterations": res["fp32_mg"]["iterations"] - res["fp64_mg"]["iterations"],
            "speedup_fp32_mg": res["fp64_mg"]["solve_s"] / res["fp32_mg"]["solve_s"],
            "velocity_rel_l2_fp32_vs_fp64": rel(u32, u64),
            "pressure_rel_l2_fp32_vs_fp64": rel(res["fp32_mg"]["x"][f.n_u:], res["fp64_mg"]["x"][f.n_u:])}
    if oracle_residual:
        from oracle import Oracle
        t0 = time.perf_counter()
        o = Oracle(P.levels)
        o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
        for key in ("fp64_mg", "fp32_mg"):
            r = P.rhs - o.vmult(0, len(P.levels) - 1, res[key]["x"])
            res[key]["oracle_residual"] = float(np.linalg.norm(r))
        line["oracle_seconds"] = time.perf_counter() - t0
    for key in ("fp64_mg", "fp32_mg"):
        line[key] = {k: v for k, v in res[key].items() if k != "x"}
    return line


def _config_line(name):
    import torch
    from aspect_gb300 import adjoint, gmg, problems, shell
    if name == "solcx64":
        return _solve_pair(problems.solcx(6, density_sign=1.0))
    if name == "sphere16":
        return _solve_pair(problems.adaptive_sphere(4, 2))
    if name == "sinkers16q3":
        # velocity degree 3 (Q3-Q2, QGauss(4)) on the sinker workload at 16^3 cells
        # (the pressure space of the 32^3 Q2-Q1 workload); operator timings beside
        P = problems.sinkers_3d(16, degree=3)
        line = _solve_pair(P, oracle_residual=True)
        g = gmg.from_problem(P)
        ops = {"stokes_vmult_fp64": g.time_operation(gmg.TIME_STOKES_VMULT, gmg.FP64, 20),
               "stokes_vmult_fp32": g.time_operation(gmg.TIME_STOKES_VMULT, gmg.FP32, 20),
               "A_vmult_fp32": g.time_operation(gmg.TIME_A_VMULT, gmg.FP32, 20)}
        n = P.fine.n_u + P.fine.n_p
        line["operator_seconds"] = ops
        line["operator_gdofs"] = {k: (n if k.startswith("stokes") else P.fine.n_u) / v / 1e9 for k, v in ops.items()}
        return line
    if name in ("shell3", "shell3a"):
        # refinement 3, and for shell3a one adaptive level on the temperature gradient
        t0 = time.perf_counter()
        P = problems.spherical_shell(3, n_adaptive=1 if name == "shell3a" else 0)
        t_mesh = time.perf_counter() - t0
        q, _ = np.linalg.qr(shell.rotation_modes(P.fine).T)
        line = _solve_pair(P, {"coarse_solver": gmg.COARSE_DENSE_FP64}, lambda u: u - q @ (q.T @ u),
                           oracle_residual=name == "shell3a")
        line["host_mesh_seconds"] = t_mesh
        return line
    if name == "adjoint32":
        def factory(base):
            g = gmg.StokesMatrixFreeGPU(3, len(base.levels))
            g.setup_dofs(base.levels)
            return g
        ap, ev = adjoint.make_problem(32, factory, tol=1e-8)
        ev.gradient(ap.lneta)  # warm
        t0 = time.perf_counter()
        J, _, _, _ = ev.gradient(ap.lneta)
        torch.cuda.synchronize()
        return {"workload": "adjoint_gradient_32^3", "cells": len(ap.lneta), "J": J,
                "seconds_forward_adjoint_backward": time.perf_counter() - t0,
                "note": "viscosity tables and preconditioner rebuilt for the evaluation point, then forward "
                        "and adjoint FP32-MG/FP64 solves to 1e-8 and the backward kernel; host wall time"}
    raise ValueError(f"unknown workload {name}")


def run_configs(names):
    """FP64-MG against FP32-MG (FP64 FGMRES) solves to 1e-8 on the other
    workloads: 2D 64^2 SolCx-like (eta jump 1e6), 3D 16^3 + 2 adaptive levels
    around a sphere, the spherical shell at refinement 3 (FP64 dense coarse
    solve), and the adjoint gradient on 32^3 (forward + adjoint solve + backward
    kernel). One JSON line per workload, written as each finishes. Velocity
    differences on the shell are taken after removing the rigid rotations (its
    null space under free slip)."""
    import torch
    torch.cuda.init()
    for name in names:
        try:
            line = _config_line(name)
        except Exception as e:  # report it and go on with the next workload
            line = {"workload": name, "error": f"{type(e).__name__}: {e}"}
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--profile-op", default=None, choices=sorted(PROFILE_OPS))
    ap.add_argument("--sweep", default=None, help="comma-separated cells per direction, e.g. 32,64")
    ap.add_argument("--configs", default=None,
                    help="comma-separated: solcx64,sphere16,sinkers16q3,adjoint32,shell3,shell3a")
    args = ap.parse_args()
    if args.configs:
        run_configs(args.configs.split(","))
    elif args.sweep:
        run_sweep([int(v) for v in args.sweep.split(",")])
    elif args.profile_op:
        run_profile_op(args.profile_op)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
