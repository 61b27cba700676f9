#!/usr/bin/env python3
"""Benchmark of the GB300 workset assembly path on the 128^3 Q1 hex steady-thermal workload (C2).

A step is one Jacobian+residual assembly (assembleJacRes with fused zero-fill) over all 2,097,152
cells, inputs resident in HBM.  The L2 is flushed (256 MB write) before every timed step, outside the
CUDA events that time the step.  Printed as one JSON line on rank 0.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU restatement of the reference algorithm (the oracle; the reference
itself cannot be built without Trilinos) on the host cores with all threads, each step a bounded
sample of the same workload.  With N > 1 (torchrun) every rank runs an independent replica of the
workload (the problem has no exchange step in this form), so scaling is weak.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# the path's headline metric: Jacobian + residual assembly throughput, FP64 against mixed precision
METRIC = "Jac+res cells/s FP64 vs mixed (rel res\u22641e-10); DOF/s; serve p50/p99 ms"

WORKLOAD = ("C2: steady thermal, unit cube, 128^3 Q1 hex (2,097,152 cells, 8 nodes/cell, 2x2x2 Gauss), "
            "kappa=exp(0.5 g) per cell, f=1, u=0 on x=0 and x=1, one Jacobian+residual assembly per step")


def algorithmic_bytes(ncell, nnode, nnz, s_j, npe=8, dim=3):
    """Bytes one Q1 Jac+res assembly must move: J values, u and r, kappa and connectivity, coordinates."""
    return nnz * s_j + nnode * (8 + 8) + ncell * (8 + 4 * npe) + nnode * 8 * dim


def read_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the headline kernel,
# k_fact_hex<double,1,1,1,1>, on the 128^3 workload, from one ncu capture of
#     ncu --set full --clock-control none -k regex:k_fact_hex -s 2 -c 1 -o fact_hex_fp64 \
#         python bench.py --profile fp64 --steps 3 --warmup 2
# (k_kappa_scale, the other launch of the assembly call, moves 33.6 MB more)
# (this run does not measure it; the bench line says so next to the value)
C2_FP64_DRAM_BYTES_CAPTURED = 463_531_776


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0, t1):
        rows = []
        for ts, line in self.lines:
            if not (t0 <= ts <= t1):
                continue
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append(dict(sm=float(f[1]), smax=float(f[2]), power=float(f[3]) if f[3] not in ("[N/A]", "N/A") else 0.0,
                                 hw=f[5], hwt=f[6], swt=f[7], swp=f[8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        reasons = set()
        for r in rows:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"), ("swt", "sw_thermal_slowdown"),
                              ("swp", "sw_power_cap")):
                if r[key].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in rows), "sm_max_mhz": max(r["smax"] for r in rows),
                "power_w_max": max(r["power"] for r in rows), "reasons": sorted(reasons), "samples": len(rows)}


def cpu_baseline(n=128, slab=64, seed=2, threads=None, reps=5):
    """The oracle (C++ restatement of the reference algorithm, FP64 forward AD, OpenMP atomic scatter)
    timed on the host cores on the first `slab` z-layers of C2: the first slab*n*n cells of the mesh
    with their kappa (same cell size, same coefficient stream)."""
    from mrhyde_gb300.workloads import lognormal_kappa
    from oracle.oracle import OracleProblem, max_threads

    threads = threads or max_threads()
    kap = lognormal_kappa(n ** 3, seed, 0.5)[: slab * n * n]
    P = OracleProblem(dim=3, order=1, n=(n, n, slab), lo=(0, 0, 0), hi=(1.0, 1.0, slab / n), kind=0,
                      source=("const", 1.0, 0.0), kappa=kap, dirichlet_faces=3, workset_size=1024)
    u = np.random.default_rng(7).uniform(-1, 1, P.ndof)
    best = []
    P.assemble(u, nthreads=threads)  # warm-up
    for _ in range(reps):
        t = time.perf_counter()
        P.assemble(u, nthreads=threads)
        best.append(time.perf_counter() - t)
    dt = statistics.median(best)
    return dict(value=P.ncell / dt, unit="cells/s", cores=threads, kind="port",
                sample=f"first {slab} z-layers of C2 ({P.ncell} cells of 128^3, same kappa stream), "
                       f"Jac+res with 8-tangent forward AD, OpenMP atomic scatter, median of {reps} after 1 warm-up",
                seconds_per_sample=dt)


def run_reference(args, rank, world):
    if rank != 0:
        return
    n = 128
    step_slab = 4
    # K steps, each a bounded sample of the workload (first `step_slab` z-layers of C2)
    from mrhyde_gb300.workloads import lognormal_kappa
    from oracle.oracle import OracleProblem, max_threads

    threads = max_threads()
    kap = lognormal_kappa(n ** 3, 2, 0.5)[: step_slab * n * n]
    P = OracleProblem(dim=3, order=1, n=(n, n, step_slab), hi=(1.0, 1.0, step_slab / n), kind=0, source=("const", 1.0, 0.0),
                      kappa=kap, dirichlet_faces=3, workset_size=1024)
    u = np.random.default_rng(7).uniform(-1, 1, P.ndof)
    for _ in range(args.warmup):
        P.assemble(u, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        P.assemble(u, nthreads=threads)
    dt = time.perf_counter() - t0
    value = P.ncell * args.steps / dt
    out = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": WORKLOAD, "sample_cells_per_step": P.ncell,
                      "note": "reference (Trilinos/Kokkos) cannot be built here; timed: its algorithm restated in C++ (oracle/)"},
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": "port",
                            "sample": f"first {step_slab} z-layers of C2 per step ({P.ncell} cells)"},
           "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch

    import mrhyde_gb300
    from mrhyde_gb300 import AssemblyManager, Problem, SolverManager
    from mrhyde_gb300.workloads import c2

    torch.cuda.set_device(local_rank)
    mrhyde_gb300.load()
    dist = None
    if world > 1:
        import torch.distributed as dist

    cfg = c2(seed=2 + rank, n=args.n)
    P = Problem(**cfg)
    A = AssemblyManager(P)
    info = P.info
    u = torch.tensor(np.random.default_rng(7 + rank).uniform(0.0, 1.0, info.n_dofs), device="cuda")
    r = P.new_vector()
    J64 = P.new_matrix_values(fp32=False)
    J32 = P.new_matrix_values(fp32=True)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")  # 256 MB > 129 MB L2
    stream = torch.cuda.current_stream()

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(fn, steps):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        barrier()
        for k in range(steps):
            flush.fill_(k)
            ev[k][0].record(stream)
            fn()
            ev[k][1].record(stream)
        barrier()
        ms = [a.elapsed_time(b) for a, b in ev]
        tot = max_over_ranks(sum(ms), dist, "cuda")
        return tot, ms

    jac64 = lambda: A.assembleJacRes(u, r, J64, overwrite=True)
    jac32 = lambda: A.assembleJacRes(u, r, J32, fp32_jacobian=True, overwrite=True)
    res64 = lambda: A.assembleRes(u, r, overwrite=True)
    for _ in range(max(args.warmup, 3)):
        jac64(); jac32(); res64()
    torch.cuda.synchronize()

    sampler = ClockSampler(local_rank) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.6)
    t_clock0 = time.time()
    tot64, ms64 = timed(jac64, args.steps)
    # keep the same work running ~1.5 s so that the clock record has samples under load
    t_end = time.time() + 1.5
    while time.time() < t_end:
        for _ in range(50):
            jac64()
        torch.cuda.synchronize()
    t_clock1 = time.time()
    tot32, ms32 = timed(jac32, args.steps)
    totres, _ = timed(res64, args.steps)

    # e2e through the public API with host buffers: every step uploads u from pinned host memory, assembles,
    # and copies J and r back to pinned host memory.  Two buffer sets on two streams: step k+1's upload and
    # assembly run while step k's 474 MB copy-back (the bound: ~190 GB/s over the host link) is in flight.
    u_h = torch.empty(info.n_dofs, dtype=torch.float64, pin_memory=True)
    u_h.copy_(u.cpu())
    sets = []
    for k in range(2):
        sets.append({"ud": P.new_vector(), "r": P.new_vector(), "J": J64 if k == 0 else P.new_matrix_values(),
                     "J_h": torch.empty(info.nnz, dtype=torch.float64, pin_memory=True),
                     "r_h": torch.empty(info.n_dofs, dtype=torch.float64, pin_memory=True),
                     "s": torch.cuda.Stream()})

    def e2e_run(n):
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        t0.record(stream)
        for b in sets:
            b["s"].wait_event(t0)
        for k in range(n):
            b = sets[k % 2]
            with torch.cuda.stream(b["s"]):
                b["ud"].copy_(u_h, non_blocking=True)
                A.assembleJacRes(b["ud"], b["r"], b["J"], overwrite=True, stream=b["s"])
                b["J_h"].copy_(b["J"], non_blocking=True)
                b["r_h"].copy_(b["r"], non_blocking=True)
        for b in sets:
            e = torch.cuda.Event()
            e.record(b["s"])
            stream.wait_event(e)
        t1.record(stream)
        barrier()
        return max_over_ranks(t0.elapsed_time(t1), dist, "cuda")

    e2e_run(2)
    n_e2e = min(args.steps, 20)
    tot_e2e = e2e_run(n_e2e)
    torch.cuda.synchronize()
    if not torch.equal(sets[(n_e2e - 1) % 2]["J_h"], J64.cpu()):
        raise RuntimeError("e2e: the Jacobian copied back differs from the device result")
    if sampler:
        sampler.stop()

    cells = info.n_cells
    ms_step = tot64 / args.steps
    value = world * cells * args.steps / (tot64 * 1e-3)
    peaks, peak_kind = read_peaks()
    algo64 = algorithmic_bytes(cells, info.n_dofs, info.nnz, 8)
    algo32 = algorithmic_bytes(cells, info.n_dofs, info.nnz, 4)
    ach64 = algo64 / (ms_step * 1e-3) / 1e9
    traffic = C2_FP64_DRAM_BYTES_CAPTURED if args.n == 128 else None
    dp_ops = fp64_instructions(cfg)
    import ctypes

    from mrhyde_gb300 import _lib as LL

    r64, r32 = ctypes.c_double(0), ctypes.c_double(0)
    LL.check(LL.lib().mrg_measure_fma_rates(ctypes.byref(r64), ctypes.byref(r32), stream.cuda_stream), "fma rates")
    dp_peak = r64.value  # FP64 FMA instructions/s measured live on this GPU

    out = {
        "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": cells, "dofs": info.n_dofs, "nnz": info.nnz,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "flushed before every timed step (256 MB write, outside the step's CUDA events)",
                   "path": "factored row-gather (kappa_c * K_ref, one CSR row per thread, smem-staged 16B stores); "
                            "cubic cells: k_kappa_scale forms |K| kappa_c per cell, then every entry is the exact "
                            "64-bit fixed-point sum of its cells' scaled conductances rounded once (no FP64 "
                            "instruction), axis-neighbour entries +0, residual 21 FP64 FMAs per row"},
        "dof_per_s": world * info.n_dofs * args.steps / (tot64 * 1e-3),
        "mixed": {"value": world * cells * args.steps / (tot32 * 1e-3), "unit": "cells/s",
                  "ms_per_step": tot32 / args.steps, "dtype": "J f32 / residual f64",
                  "speedup_vs_fp64": tot64 / tot32},
        "residual_only": {"value": world * cells * args.steps / (totres * 1e-3), "unit": "cells/s",
                          "ms_per_step": totres / args.steps},
        "roofline": {"bound": "hbm", "achieved": ach64, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": ach64 / peaks["hbm_gbs"], "traffic": traffic,
                     "traffic_source": "ncu capture of one launch of this kernel on this workload (dram read + write "
                                       "bytes; a constant in bench.py, not measured by this run)",
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "duration": "CUDA events around the whole assembly call (k_kappa_scale + k_fact_hex)",
                     "algorithmic_bytes_per_launch": algo64,
                     "fp64_pipe": {"dp_instr_per_launch": dp_ops, "achieved_dp_instr_per_s": dp_ops / (ms_step * 1e-3),
                                   "peak_dp_instr_per_s": dp_peak, "frac": dp_ops / (ms_step * 1e-3) / dp_peak,
                                   "peak_source": "measured in this run (mrg_measure_fma_rates)",
                                   "fp32_fma_per_s": r32.value}},
        "e2e": {"value": world * cells * n_e2e / (tot_e2e * 1e-3), "unit": "cells/s",
                "h2d_bytes_per_step": info.n_dofs * 8, "d2h_bytes_per_step": info.nnz * 8 + info.n_dofs * 8,
                "schedule": "two buffer sets on two streams: step k+1's upload and assembly overlap step k's copy-back"},
        "gpu_launches": 2 * args.steps,  # k_kappa_scale + k_fact_hex per step
    }
    out["mixed"]["roofline_frac"] = algo32 / (tot32 / args.steps * 1e-3) / 1e9 / peaks["hbm_gbs"]
    if sampler:
        out["clocks"] = sampler.summary(t_clock0, t_clock1)

    # End-to-end solve: Newton (FP64 J + FP64 PCG) vs mixed (FP32 J + FP32 inner PCG, FP64 residual),
    # both to relative residual 1e-10, same initial guess; states the mixed result's error vs FP64.
    # Each preconditioner: Jacobi (the reference's SolverManager::PCG) and geometric multigrid.
    if not args.no_solve:
        sol = {}
        ref_u = None
        for prec in ("jacobi", "gmg"):
            part = {}
            for mode in ("fp64", "mixed"):
                # mixed: the FP32 inner solve's tolerance, measured per preconditioner (refinement contracts by
                # ~3e-5 a step whatever the inner tolerance): multigrid 1e-4 (4 steps, 12 iterations), Jacobi
                # 3e-5 (4 steps instead of 5 at 1e-4)
                lin_tol = 1e-11 if mode == "fp64" else (1e-4 if prec == "gmg" else 3e-5)
                S = SolverManager(P, nonlinear_tol=1e-10, max_nonlinear_iters=12, linear_tol=lin_tol,
                                  linear_maxiter=20000, mixed_precision=mode == "mixed", preconditioner=prec)
                uu = P.new_vector()
                S.nonlinearSolver(uu)  # warm (allocates workspace, captures graphs)
                uu.zero_()
                barrier()
                t = time.perf_counter()
                res = S.nonlinearSolver(uu, raise_on_noconv=False)
                barrier()
                dt = time.perf_counter() - t
                part[mode] = {"seconds": dt, "cells_per_s": world * cells / dt, "newton_iters": res.outer_iterations,
                              "pcg_iters": res.iterations, "rel_residual_inf": res.rel_residual}
                if ref_u is None:
                    ref_u = uu.clone()
                else:
                    part[mode]["max_rel_diff_vs_fp64_jacobi"] = float((uu - ref_u).abs().max() / ref_u.abs().max())
            part["mixed_speedup_e2e"] = part["fp64"]["seconds"] / part["mixed"]["seconds"]
            if prec == "jacobi":
                sol.update(part)
            else:
                sol["gmg"] = part
        SolverManager(P, preconditioner="jacobi")
        out["solve"] = sol

    if not args.no_extras:
        for name, fn in (("general", bench_general), ("general_quad", bench_general_quad), ("c3", bench_c3),
                         ("c4", bench_c4),
                         ("c5", lambda a: bench_c5(a, rank, world, dist))):
            try:
                out[name] = fn(args)
            except Exception as e:  # reported, never fatal for the headline line
                out[name] = {"error": f"{type(e).__name__}: {e}"}
            torch.cuda.synchronize()

    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            out["cpu_baseline"] = cpu_baseline()
        except Exception as e:  # reported, never fatal
            out["cpu_baseline"] = {"value": None, "error": str(e)}
    if rank == 0:
        out["targets"] = targets_summary(out)  # last key: survives a tail of the printed line
        print(json.dumps(out), flush=True)


def targets_summary(out):
    """The path's measurement targets in one compact object (values copied from the rest of the line)."""
    def g(d, *keys):
        for k in keys:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d

    def r3(x):
        return None if x is None else float(f"{x:.4g}")

    t = {"c2_fp64_jacres_ms": r3(out["ms_per_step"]), "c2_mixed_jacres_ms": r3(g(out, "mixed", "ms_per_step")),
         "c2_fp64_hbm_frac": r3(g(out, "roofline", "frac")),
         "c2_fp64_pipe_frac": r3(g(out, "roofline", "fp64_pipe", "frac")),
         "c2_e2e_cells_per_s": r3(g(out, "e2e", "value"))}
    sol = out.get("solve") or {}
    if sol:
        t["c2_solve_mixed_speedup_e2e"] = {"gmg": r3(g(sol, "gmg", "mixed_speedup_e2e")),
                                           "jacobi": r3(sol.get("mixed_speedup_e2e")),
                                           "gmg_fp64_s": r3(g(sol, "gmg", "fp64", "seconds")),
                                           "gmg_mixed_s": r3(g(sol, "gmg", "mixed", "seconds")),
                                           "mixed_max_rel_diff_vs_fp64": r3(g(sol, "gmg", "mixed", "max_rel_diff_vs_fp64_jacobi")),
                                           "mixed_rel_residual": r3(g(sol, "gmg", "mixed", "rel_residual_inf"))}
    c3 = out.get("c3") or {}
    if c3 and "error" not in c3:
        t["c3"] = {"jac_fp32_plus_res_ms": r3(c3.get("jac_fp32_plus_res_ms_tensor_cores")),
                   "jac_only_ms": r3(c3.get("jac_only_ms_tensor_cores")),
                   "hbm_frac": r3(g(c3, "roofline", "hbm_frac")),
                   "tensor_frac_issued": r3(g(c3, "roofline", "tensor_frac_issued")),
                   "newton_mixed_gmg_s": r3(g(c3, "newton_mixed_gmg", "seconds")),
                   "newton_rel_residual": r3(g(c3, "newton_mixed_gmg", "rel_residual_inf"))}
    gen = out.get("general") or {}
    if gen and "error" not in gen:
        t["general_noaffine"] = {"fp64_jacres_ms": r3(gen.get("fp64_jacres_ms")),
                                 "mixed_jacres_ms": r3(gen.get("mixed_jacres_ms")),
                                 "residual_ms": r3(gen.get("residual_ms")),
                                 "ad_kernels_fp64_jacres_ms": r3(gen.get("ad_kernels_fp64_jacres_ms")),
                                 "hbm_frac_fp64": r3(gen.get("hbm_frac_fp64"))}
    gq = out.get("general_quad") or {}
    if gq and "error" not in gq:
        t["general_noaffine_quad"] = {k: r3(gq.get(k)) for k in ("fp64_jacres_ms", "mixed_jacres_ms", "residual_ms",
                                                                 "ad_kernels_fp64_jacres_ms", "hbm_frac_fp64")}
    c4 = out.get("c4") or {}
    if c4 and "error" not in c4:
        t["c4"] = {"ms_per_batch": r3(c4.get("ms_per_batch")), "all_converged": c4.get("all_converged")}
    c5 = out.get("c5") or {}
    if c5 and "error" not in c5:
        t["c5"] = {m: {"p50_ms": r3(g(c5, m, "p50_ms")), "p99_ms": r3(g(c5, m, "p99_ms")),
                       "req_per_s": r3(g(c5, m, "req_per_s"))} for m in ("mixed", "fp64")}
        t["c5"]["batch_req_per_s"] = r3(g(c5, "batch_mixed", "req_per_s"))
        t["c5"]["at_80pct"] = {"p50_ms": r3(g(c5, "stream_at_80pct_batch", "p50_ms")),
                               "p99_ms": r3(g(c5, "stream_at_80pct_batch", "p99_ms")),
                               "p99_over_p50": r3(g(c5, "stream_at_80pct_batch", "p99_over_p50"))}
    cb = out.get("cpu_baseline") or {}
    if cb.get("value"):
        t["cpu_baseline_cells_per_s"] = r3(cb["value"])
    return t


def _ev_time(fn, reps):
    import torch

    s = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    a.record(s)
    for _ in range(reps):
        fn()
    b.record(s)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def bench_c3(args):
    """C3: -div((1+u^2) grad u) = 10 on 64^3 Q2 hexes, u0 ~ U(0, 0.1); Newton to 1e-10 (mixed: FP32
    Jacobian + FP32 inner PCG, FP64 residual), plus per-assembly timings."""
    import torch

    from mrhyde_gb300 import AssemblyManager, Problem, SolverManager
    from mrhyde_gb300.workloads import c3

    cfg, u0 = c3(seed=3, n=args.c3_n)
    P = Problem(**cfg)
    A = AssemblyManager(P)
    info = P.info
    u = torch.tensor(u0, device="cuda")
    r = P.new_vector()
    J32 = P.new_matrix_values(fp32=True)
    t_res = _ev_time(lambda: A.assembleRes(u, r, overwrite=True), 5)
    t_j32 = _ev_time(lambda: A.assembleJacRes(u, r, J32, fp32_jacobian=True, overwrite=True, tensor_cores=False), 3)
    t_jtc = _ev_time(lambda: A.assembleJacRes(u, r, J32, fp32_jacobian=True, overwrite=True, tensor_cores=True), 3)
    t_j32_only = _ev_time(lambda: A.assembleJac(u, J32, fp32_jacobian=True, overwrite=True, tensor_cores=False), 3)
    t_jtc_only = _ev_time(lambda: A.assembleJac(u, J32, fp32_jacobian=True, overwrite=True, tensor_cores=True), 3)
    out = {"workload": f"{args.c3_n}^3 Q2 hex, 27 nodes/cell, 3x3x3 Gauss, u=0 on x=0,1", "cells": info.n_cells,
           "dofs": info.n_dofs, "nnz": info.nnz,
           "residual_fp64_ms": t_res, "residual_cells_per_s": info.n_cells / (t_res * 1e-3),
           "jac_fp32_plus_res_ms_cuda_cores": t_j32, "jac_fp32_plus_res_ms_tensor_cores": t_jtc,
           "jac_fp32_cells_per_s_tensor_cores": info.n_cells / (t_jtc * 1e-3),
           "jac_only_ms_cuda_cores": t_j32_only, "jac_only_ms_tensor_cores": t_jtc_only,
           "contraction_tflops_tensor_cores": 2.0 * 27 * 27 * 108 * info.n_cells / (t_jtc_only * 1e-3) / 1e12}
    # Roofline of the Jacobian-only pass on the tensor cores: algorithmic bytes = the FP32 CSR values written
    # plus u read; algorithmic flops = 2*27*27*108 per cell (the B^T D B contraction); issued MMA flops =
    # 3 products (3xTF32) * 2 * 112 (K padded) * 768 (27 rows padded to 28, plus 12) per cell.  The TF32
    # dense rate is half the bf16 rate on this part: the denominator is half the measured bf16 GEMM rate.
    peaks, peak_kind = read_peaks()
    algo_bytes = info.nnz * 4 + info.n_dofs * 8
    issued = 3 * 2.0 * 112 * 768 * info.n_cells
    tf32_peak = 0.5 * peaks["bf16_tflops"] * 1e12
    out["roofline"] = {"pass": "Jacobian only (coefficients, tensor-core element matrices, CSR rows)",
                       "algorithmic_bytes": algo_bytes,
                       "hbm_achieved_gbs": algo_bytes / (t_jtc_only * 1e-3) / 1e9,
                       "hbm_frac": algo_bytes / (t_jtc_only * 1e-3) / 1e9 / peaks["hbm_gbs"],
                       "issued_tflops": issued / (t_jtc_only * 1e-3) / 1e12,
                       "tensor_frac_issued": issued / (t_jtc_only * 1e-3) / tf32_peak,
                       "peak_source": f"{peak_kind}: hbm_gbs; TF32 = bf16_tflops / 2"}
    del J32
    torch.cuda.empty_cache()
    # mixed Newton to 1e-10 with Jacobi BiCGStab (the reference's solver family) and with p-multigrid
    # BiCGStab; each timed on its second run (the first builds workspace, graphs and the hierarchy)
    for key, prec in (("newton_mixed", "jacobi"), ("newton_mixed_gmg", "gmg")):
        S = SolverManager(P, nonlinear_tol=1e-10, max_nonlinear_iters=25, linear_tol=1e-3, linear_maxiter=20000,
                          mixed_precision=True, preconditioner=prec)
        for rep in range(2):
            uu = torch.tensor(u0, device="cuda")
            torch.cuda.synchronize()
            t = time.perf_counter()
            res = S.nonlinearSolver(uu, raise_on_noconv=False)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t
        out[key] = {"seconds": dt, "newton_iters": res.outer_iterations, "krylov_iters": res.iterations,
                    "rel_residual_inf": res.rel_residual, "cells_per_s": info.n_cells / dt,
                    "dof_per_s": info.n_dofs / dt}
    SolverManager(P, preconditioner="jacobi")
    return out


def bench_general(args):
    """C2's coefficients, source and boundary data on non-affine hexahedra (interior vertices moved by up to
    0.2 h): the general per-cell path (geometry per cell, forward-AD tangents in registers, coloured
    scatter) -- what a mesh that is not a uniform box gets."""
    import torch

    from mrhyde_gb300 import AssemblyManager, Problem
    from mrhyde_gb300.workloads import c2_general

    n = args.general_n
    cfg = c2_general(seed=2, n=n)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    P = Problem(**cfg)  # creation computes and stores every cell's stiffness (the stored-geometry path)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    info = P.info
    A = AssemblyManager(P)
    u = torch.tensor(np.random.default_rng(7).uniform(0.0, 1.0, info.n_dofs), device="cuda")
    r = P.new_vector()
    J64 = P.new_matrix_values(fp32=False)
    t64 = _ev_time(lambda: A.assembleJacRes(u, r, J64, overwrite=True), 3)
    # the per-cell forward-AD kernels (geometry and AD tangents per cell, 8-colour scatter) on the same mesh
    tad = _ev_time(lambda: A.assembleJacRes(u, r, J64, overwrite=True, force_cell=True), 2)
    del J64
    J32 = P.new_matrix_values(fp32=True)
    t32 = _ev_time(lambda: A.assembleJacRes(u, r, J32, fp32_jacobian=True, overwrite=True), 3)
    del J32
    tres = _ev_time(lambda: A.assembleRes(u, r, overwrite=True), 3)
    torch.cuda.empty_cache()
    peaks, peak_kind = read_peaks()
    algo = algorithmic_bytes(info.n_cells, info.n_dofs, info.nnz, 8)
    return {"workload": f"{n}^3 Q1 hex, interior vertices perturbed by up to 0.2 h (non-affine), C2 coefficients",
            "path": info.path, "cells": info.n_cells, "dofs": info.n_dofs, "nnz": info.nnz,
            "fp64_jacres_ms": t64, "fp64_cells_per_s": info.n_cells / (t64 * 1e-3),
            "mixed_jacres_ms": t32, "mixed_cells_per_s": info.n_cells / (t32 * 1e-3),
            "residual_ms": tres, "residual_cells_per_s": info.n_cells / (tres * 1e-3),
            "ad_kernels_fp64_jacres_ms": tad, "setup_s": setup_s,
            "hbm_frac_fp64": algo / (t64 * 1e-3) / 1e9 / peaks["hbm_gbs"], "algorithmic_bytes": algo}


def bench_general_quad(args):
    """C1's coefficients, source and boundary data on n^2 non-affine quadrilaterals (interior vertices moved
    by up to 0.2 h): the stored-geometry path in 2-D, beside the per-cell forward-AD kernels."""
    import torch

    from mrhyde_gb300 import AssemblyManager, Problem
    from mrhyde_gb300.workloads import c1_general

    n = args.general_quad_n
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    P = Problem(**c1_general(seed=1, n=n))
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    info = P.info
    A = AssemblyManager(P)
    u = torch.tensor(np.random.default_rng(7).uniform(0.0, 1.0, info.n_dofs), device="cuda")
    r = P.new_vector()
    J64 = P.new_matrix_values(fp32=False)
    t64 = _ev_time(lambda: A.assembleJacRes(u, r, J64, overwrite=True), 3)
    tad = _ev_time(lambda: A.assembleJacRes(u, r, J64, overwrite=True, force_cell=True), 2)
    del J64
    J32 = P.new_matrix_values(fp32=True)
    t32 = _ev_time(lambda: A.assembleJacRes(u, r, J32, fp32_jacobian=True, overwrite=True), 3)
    del J32
    tres = _ev_time(lambda: A.assembleRes(u, r, overwrite=True), 3)
    torch.cuda.empty_cache()
    peaks, _ = read_peaks()
    algo = algorithmic_bytes(info.n_cells, info.n_dofs, info.nnz, 8, npe=4, dim=2)
    return {"workload": f"{n}^2 Q1 quadrilaterals, interior vertices perturbed by up to 0.2 h (non-affine), "
                        "C1 coefficients", "path": info.path, "cells": info.n_cells, "dofs": info.n_dofs,
            "nnz": info.nnz, "fp64_jacres_ms": t64, "fp64_cells_per_s": info.n_cells / (t64 * 1e-3),
            "mixed_jacres_ms": t32, "residual_ms": tres, "ad_kernels_fp64_jacres_ms": tad, "setup_s": setup_s,
            "hbm_frac_fp64": algo / (t64 * 1e-3) / 1e9 / peaks["hbm_gbs"], "algorithmic_bytes": algo}


def bench_c4(args):
    """C4: 4096 local steady-thermal problems (per-axis cells U{4..16}), one persistent launch."""
    import torch

    from mrhyde_gb300.subgrid import SubgridBatch
    from mrhyde_gb300.workloads import c4_problem, c4_sizes

    sizes = c4_sizes(4096, seed=4)
    probs = [c4_problem(sizes, k, seed=4) for k in range(len(sizes))]
    B = SubgridBatch(sizes, [p["kappa"] for p in probs], [p["dirichlet"][1] for p in probs], source=1.0)
    cfg = B.autotune()
    st = B.solve()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s = torch.cuda.current_stream()
    reps = 3
    a.record(s)
    for _ in range(reps):
        B.solve(stats=False)
    b.record(s)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    st = B.solve()
    info = B.info
    return {"problems": int(len(sizes)), "cells": int(info.n_cells), "dofs": int(info.n_nodes), "nnz": int(info.nnz),
            "ms_per_batch": ms, "cells_per_s": info.n_cells / (ms * 1e-3), "dof_per_s": info.n_nodes / (ms * 1e-3),
            "problems_per_s": len(sizes) / (ms * 1e-3), "config": {"threads": cfg[0], "ctas_per_sm": cfg[1]},
            "max_rel_residual": float(st[:, 2].max()), "mean_outer": float(st[:, 0].mean()),
            "mean_inner": float(st[:, 1].mean()), "all_converged": bool((st[:, 3] == 0).all())}


def max_over_ranks(x: float, dist=None, device="cpu") -> float:
    """The largest value of x over all ranks (x itself on one process)."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def fp64_instructions(cfg):
    """FP64 instructions of one FP64 Jac+res assembly of the factored Q1 path on a box with Dirichlet rows on
    the x = 0 and x = 1 faces.  Box cells: a DMUL (K(off) * S(off)) and a DFMA (residual) per entry of a free
    row.  Cubic cells: the axis-neighbour entries take none (K = +0) and the others one DFMA each (the
    entries are exact sums of scaled conductances, formed on the integer pipes), plus one DMUL per cell in
    k_kappa_scale.  The kappa sums are exact fixed-point sums on the integer pipes (no FP64 instruction)."""
    import numpy as np

    n = [c + 1 for c in cfg["n"]]
    h = [(b - a) / c for a, b, c in zip(cfg["lo"], cfg["hi"], cfg["n"])]
    nb = [(np.arange(m) > 0).astype(np.int64) + (np.arange(m) < m - 1) for m in n]  # neighbours per axis
    bx, by, bz = nb[0][1:-1][None, None, :], nb[1][None, :, None], nb[2][:, None, None]  # free rows: 0 < ix < nx
    entries = int(((1 + bx) * (1 + by) * (1 + bz)).sum())
    if h[0] == h[1] == h[2]:
        entries -= int((bx + by + bz).sum())
        return entries + int(np.prod(cfg["n"]))
    return 2 * entries


def serve_replicated(reqs, slots, realtime, rank=0, world=1, dist=None):
    """Serves this replica's share of `reqs`; on N replicas returns the whole-job summary (every rank)."""
    from mrhyde_gb300 import serving

    srv = serving.Server(hbm_budget_bytes=80 * 10**9, slots=slots)
    srv.warmup()
    mine = serving.shard(reqs, rank, world) if world > 1 else reqs
    summ = srv.run(mine, realtime=realtime)
    summ["peak_active"] = srv.peak_active
    if world == 1 or dist is None:
        return summ
    parts = [None] * world
    dist.all_gather_object(parts, ([r for r in srv.results], srv.wall))
    whole = serving.merge(parts)
    whole["peak_active"] = summ["peak_active"]
    whole["replicas"] = world
    return whole


def bench_c5(args, rank=0, world=1, dist=None):
    """C5: Poisson stream (200 req/s) of thermal and nonlinear-diffusion solves on Q1 cubes with edge
    log-uniform in [16, 96], admitted under an 80 GB budget; p50/p99 latency and DOF/s, mixed vs FP64;
    plus the batch throughput (all requests at t=0) and a stream at 80 % of it.  On N GPUs the stream is
    spread round-robin over N independent replicas and the figures are whole-job."""
    from mrhyde_gb300 import serving

    out = {}
    for mode in ("mixed", "fp64"):
        reqs = serving.poisson_stream(rate=200.0, count=args.c5_count, mixed=(mode == "mixed"), seed=5)
        out[mode] = serve_replicated(reqs, args.c5_slots, True, rank, world, dist)
    reqs = serving.poisson_stream(rate=200.0, count=args.c5_count, mixed=True, seed=5)
    batch = serve_replicated(reqs, args.c5_slots, False, rank, world, dist)
    out["batch_mixed"] = batch
    rate80 = 0.8 * batch["req_per_s"]
    reqs = serving.poisson_stream(rate=rate80, count=args.c5_count, mixed=True, seed=6)
    s80 = serve_replicated(reqs, args.c5_slots, True, rank, world, dist)
    s80["rate"] = rate80
    s80["p99_over_p50"] = s80["p99_ms"] / s80["p50_ms"]
    out["stream_at_80pct_batch"] = s80
    out["config"] = {"arrivals": "Poisson 200/s", "edge": "log-uniform [16,96]", "nonlinear_fraction": 0.5,
                     "kappa": "lognormal sigma=1 per cell (device generator, per-request seed)",
                     "budget_bytes": 80 * 10**9, "slots": args.c5_slots, "requests": args.c5_count}
    return out


def run_profile(args, local_rank):
    """Runs one kernel family only (W untimed + K launches) on C2, for ncu captures of that kernel."""
    import torch

    import mrhyde_gb300
    from mrhyde_gb300 import AssemblyManager, Problem, SolverManager
    from mrhyde_gb300.workloads import c2

    torch.cuda.set_device(local_rank)
    mrhyde_gb300.load()
    if args.profile == "c2newton":  # C2 mixed Newton with multigrid CG (the bench's solve leg): warm-up, then solve(s)
        from mrhyde_gb300 import Problem, SolverManager
        from mrhyde_gb300.workloads import c2

        P = Problem(**c2(n=args.n))
        S = SolverManager(P, nonlinear_tol=1e-10, max_nonlinear_iters=12, linear_tol=1e-4, linear_maxiter=20000,
                          mixed_precision=True, preconditioner="gmg")
        for _ in range(args.warmup + args.steps):
            uu = P.new_vector()
            t = time.perf_counter()
            res = S.nonlinearSolver(uu, raise_on_noconv=False)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t
        print(json.dumps({"profile": "c2newton", "steps": args.steps, "seconds_last": dt,
                          "newton_iters": res.outer_iterations, "krylov_iters": res.iterations}))
        return
    if args.profile == "c3gmg":  # C3 mixed Newton with p-multigrid BiCGStab: warm-up solve(s), then the solve(s)
        from mrhyde_gb300 import Problem, SolverManager
        from mrhyde_gb300.workloads import c3

        cfg, u0 = c3(seed=3, n=args.c3_n)
        P = Problem(**cfg)
        S = SolverManager(P, nonlinear_tol=1e-10, max_nonlinear_iters=25, linear_tol=1e-3, linear_maxiter=20000,
                          mixed_precision=True, preconditioner="gmg")
        for _ in range(args.warmup + args.steps):
            uu = torch.tensor(u0, device="cuda")
            res = S.nonlinearSolver(uu, raise_on_noconv=False)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "c3gmg", "steps": args.steps, "newton_iters": res.outer_iterations,
                          "krylov_iters": res.iterations, "rel_residual_inf": res.rel_residual}))
        return
    if args.profile == "c4":  # the batched subgrid solve, default configuration (no autotuning)
        from mrhyde_gb300.subgrid import SubgridBatch
        from mrhyde_gb300.workloads import c4_problem, c4_sizes

        sizes = c4_sizes(4096, seed=4)
        probs = [c4_problem(sizes, k, seed=4) for k in range(len(sizes))]
        B = SubgridBatch(sizes, [p["kappa"] for p in probs], [p["dirichlet"][1] for p in probs], source=1.0)
        for _ in range(args.warmup + args.steps):
            B.solve(stats=False)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "c4", "steps": args.steps, "ok": True}))
        return
    if args.profile in ("cell64", "cell32", "cellad64"):  # non-affine hexahedra, C2 coefficients; cellad64
        # forces the per-cell forward-AD kernels, the others take the default (stored-geometry) path
        from mrhyde_gb300.workloads import c2_general

        P = Problem(**c2_general(seed=2, n=args.general_n))
        A = AssemblyManager(P)
        u = torch.tensor(np.random.default_rng(7).uniform(0.0, 1.0, P.info.n_dofs), device="cuda")
        r, J = P.new_vector(), P.new_matrix_values(fp32=args.profile == "cell32")
        for _ in range(args.warmup + args.steps):
            A.assembleJacRes(u, r, J, fp32_jacobian=args.profile == "cell32", overwrite=True,
                             force_cell=args.profile == "cellad64")
        torch.cuda.synchronize()
        print(json.dumps({"profile": args.profile, "n": args.general_n, "steps": args.steps, "ok": True}))
        return
    if args.profile == "q1nl64":  # Q1 1+u^2 FP64 Jacobian + residual on 96^3 box cells (a nonlinear serving request)
        from mrhyde_gb300 import _lib as LL

        n = 96
        P = Problem(dim=3, order=1, n=(n, n, n), kind="diffusion_1pu2", source=("const", 10.0, 0.0), kappa=1.0,
                    dirichlet_faces=LL.MRG_FACE_XLO | LL.MRG_FACE_XHI)
        A = AssemblyManager(P)
        u = torch.tensor(np.random.default_rng(3).uniform(0.0, 0.3, P.info.n_dofs), device="cuda")
        r, J = P.new_vector(), P.new_matrix_values()
        for _ in range(args.warmup + args.steps):
            A.assembleJacRes(u, r, J, overwrite=True)
        torch.cuda.synchronize()
        print(json.dumps({"profile": args.profile, "n": n, "steps": args.steps, "ok": True}))
        return
    if args.profile in ("quad64", "quad32"):  # non-affine quadrilaterals, C1 coefficients, stored-geometry path
        from mrhyde_gb300.workloads import c1_general

        P = Problem(**c1_general(seed=1, n=args.general_quad_n))
        A = AssemblyManager(P)
        u = torch.tensor(np.random.default_rng(7).uniform(0.0, 1.0, P.info.n_dofs), device="cuda")
        r, J = P.new_vector(), P.new_matrix_values(fp32=args.profile == "quad32")
        for _ in range(args.warmup + args.steps):
            A.assembleJacRes(u, r, J, fp32_jacobian=args.profile == "quad32", overwrite=True)
        torch.cuda.synchronize()
        print(json.dumps({"profile": args.profile, "n": args.general_quad_n, "steps": args.steps, "ok": True}))
        return
    if args.profile == "q2tcj":  # the Q2 FP32 Jacobian alone on the tensor cores (coefficients, contraction, rows)
        from mrhyde_gb300.workloads import c3

        cfg, u0 = c3(seed=3, n=args.c3_n)
        P = Problem(**cfg)
        A = AssemblyManager(P)
        u = torch.tensor(u0, device="cuda")
        J = P.new_matrix_values(fp32=True)
        for _ in range(args.warmup + args.steps):
            A.assembleJac(u, J, fp32_jacobian=True, overwrite=True, tensor_cores=True)
        torch.cuda.synchronize()
        print(json.dumps({"profile": args.profile, "n": args.c3_n, "steps": args.steps, "ok": True}))
        return
    if args.profile in ("q2tc", "q2cc"):
        from mrhyde_gb300.workloads import c3

        cfg, u0 = c3(seed=3, n=args.c3_n)
        P = Problem(**cfg)
        A = AssemblyManager(P)
        u = torch.tensor(u0, device="cuda")
        r, J = P.new_vector(), P.new_matrix_values(fp32=True)
        for _ in range(args.warmup + args.steps):
            A.assembleJacRes(u, r, J, fp32_jacobian=True, overwrite=True, tensor_cores=(args.profile == "q2tc"))
        torch.cuda.synchronize()
        print(json.dumps({"profile": args.profile, "n": args.c3_n, "steps": args.steps, "ok": True}))
        return
    P = Problem(**c2(seed=2, n=args.n))
    A, S = AssemblyManager(P), SolverManager(P)
    u = torch.tensor(np.random.default_rng(7).uniform(0.0, 1.0, P.info.n_dofs), device="cuda")
    r = P.new_vector()
    fp32 = args.profile in ("mixed", "pcg32")
    J = P.new_matrix_values(fp32=fp32)
    if args.profile in ("fp64", "mixed", "residual"):
        step = {"fp64": lambda: A.assembleJacRes(u, r, J, overwrite=True),
                "mixed": lambda: A.assembleJacRes(u, r, J, fp32_jacobian=True, overwrite=True),
                "residual": lambda: A.assembleRes(u, r, overwrite=True)}[args.profile]
        for _ in range(args.warmup + args.steps):
            step()
    elif args.profile in ("gmg64", "gmg32"):  # one multigrid-CG solve of the C2 system to 1e-10
        J = P.new_matrix_values(fp32=args.profile == "gmg32")
        A.assembleJacRes(u, r, J, fp32_jacobian=args.profile == "gmg32", overwrite=True)
        S = SolverManager(P, preconditioner="gmg")
        for _ in range(max(args.warmup, 1) + args.steps):
            x = P.new_vector()
            S.PCG(J, r, x, tol=1e-10 if args.profile == "gmg64" else 1e-5, maxiter=100, raise_on_noconv=False)
    else:  # pcg64 / pcg32: K iterations of the PCG on the C2 Jacobian
        A.assembleJacRes(u, r, J, fp32_jacobian=fp32, overwrite=True)
        x = P.new_vector()
        S.PCG(J, r, x, tol=0.0, maxiter=args.steps, raise_on_noconv=False)
    torch.cuda.synchronize()
    print(json.dumps({"profile": args.profile, "n": args.n, "steps": args.steps, "ok": True}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the C3/C4/C5 measurements")
    ap.add_argument("--c3-n", type=int, default=64)
    ap.add_argument("--general-n", type=int, default=128, help="cells per axis of the non-affine mesh leg")
    ap.add_argument("--general-quad-n", type=int, default=2048,
                    help="cells per axis of the non-affine quadrilateral leg")
    ap.add_argument("--c5-count", type=int, default=400)
    ap.add_argument("--c5-slots", type=int, default=12)
    ap.add_argument("--profile", default=None, choices=["fp64", "mixed", "residual", "pcg64", "pcg32", "q2tc", "q2cc", "gmg64", "gmg32", "c2newton", "c3gmg", "c4", "quad64", "quad32", "q1nl64",
                             "cell64", "cell32", "cellad64", "q2tcj"],
                    help="run one kernel family only (for ncu captures); prints no bench line")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.profile:
        run_profile(args, local_rank)
        return
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
