#!/usr/bin/env python
"""Benchmark of the pressure-correction hot path on one GB300.

Workload: the 256^3 jittered-hex pressure Poisson solve (16,777,216 cells, interior
vertices jittered U(-0.2h, 0.2h), unit diffusivity, Dirichlet p = 0 on the x = 0 wall,
zero-gradient elsewhere, RHS U(-1,1) * cell volume from a fixed seed), assembled with
the laplacian kernel and solved to the reference's stop test, L1-relative residual
< 1e-8.  One step = one solve from a zero start through the C ABI (matrix load into the
solver's sliced-ELL copy, the whole Krylov loop, the final FP64 residual check).

Metric: time to 1e-8 relative residual (seconds, lower is better).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun each rank solves its own copy of the system on its own GPU (replicas;
the path does not shard across GPUs in this build) and the slowest rank is reported.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import platform
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time-to-1e-8 rel. residual: learned+mixed FCG vs plain FP64 PCG, same GB300"
SEED = 2024
JITTER = 0.2
TOL = 1e-8
NSW = 20000
# DPCG sweeps to 1e-8 on the N = 256 system of this file (seed 2024).  The reference arm
# times a bounded sample of sweeps and scales by this count: the oracle runs the same
# algorithm, whose sweep count is a property of the system, not of the hardware.
DPCG_SWEEPS = {256: 1729, 128: 875}  # measured on GB300 (FP64 DPCG of this build)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def spmv_bytes(n, nnz):
    return 12 * nnz + 4 * (n + 1) + 16 * n


def dpcg_iter_bytes(n, nnz):
    return 12 * nnz + 4 * (n + 1) + 104 * n


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        rows = [r.split(", ") for r in out.strip().splitlines() if r.count(",") >= 6]
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def reduce_max(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def build_system(N):
    import freecappuccino_gb300 as fcg

    t0 = time.perf_counter()
    m = fcg.hex_mesh(N, jitter=JITTER, seed=SEED, keep_topology=True)
    t_mesh = time.perf_counter() - t0
    mu = np.full(m.numCells, -1.0)
    phi = np.zeros(m.numTotal)
    su = fcg.uniform(SEED, 0, m.numCells) * m.vol
    return m, mu, phi, su, t_mesh


def cpu_baseline(m, mu, phi, su, sweeps_needed, sample_sweeps):
    """The oracle (serial restatement of dpcg.f90) on this host: a bounded sample of
    sweeps on the full-size system, scaled to the sweep count of a full solve."""
    from oracle import oracle

    om = oracle.Mesh(**m.oracle_kwargs())
    csr = oracle.create_csr(m.numCells, m.owner, m.neighbour)
    a, su2 = oracle.laplacian(om, csr, mu, phi, su)
    t0 = time.perf_counter()
    r = oracle.dpcg(csr, a, su2, np.zeros(m.numCells), 0.0, sample_sweeps)
    dt = time.perf_counter() - t0
    per_sweep = dt / max(r.iters, 1)
    return {"value": per_sweep * sweeps_needed, "unit": "s", "cores": 1, "kind": "port",
            "sample": f"{r.iters} DPCG sweeps of the full {m.numCells}-cell system on 1 host "
                      f"thread ({dt:.2f} s, {per_sweep * 1e3:.1f} ms/sweep, {platform.machine()}), "
                      f"scaled to {sweeps_needed} sweeps to 1e-8"}


def run_reference(args, ws, rank):
    """--impl reference: the reference's CPU path (the oracle port: no Fortran compiler
    here) on the host cores, same workload, bounded sample per step."""
    if rank != 0:
        return
    from oracle import oracle
    import freecappuccino_gb300 as fcg

    oracle.build()
    N = args.N
    t0 = time.perf_counter()
    # Mesh files (points/faces) from the generator; geometry, CSR and assembly by the oracle.
    m = fcg.hex_mesh(N, jitter=JITTER, seed=SEED, keep_topology=True)
    g = oracle.geometry(m.points[:, 0], m.points[:, 1], m.points[:, 2], m.numCells,
                        m.numInnerFaces, m.face_ptr, m.face_nodes, m.owner, m.neighbour)
    kw = m.oracle_kwargs()
    kw.update(g)
    om = oracle.Mesh(**kw)
    csr = oracle.create_csr(m.numCells, m.owner, m.neighbour)
    mu = np.full(m.numCells, -1.0)
    su = fcg.uniform(SEED, 0, m.numCells) * g["vol"]
    a, su = oracle.laplacian(om, csr, mu, np.zeros(m.numTotal), su)
    setup = time.perf_counter() - t0
    sweeps_needed = DPCG_SWEEPS.get(N) or args.ref_sweeps
    S = args.ref_sample
    times = []
    for i in range(args.warmup + args.steps):
        t1 = time.perf_counter()
        r = oracle.dpcg(csr, a, su, np.zeros(m.numCells), 0.0, S)
        dt = time.perf_counter() - t1
        if i >= args.warmup:
            times.append(dt / r.iters * sweeps_needed)
    v = statistics.mean(times)
    line = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic: seeded jittered hex mesh and U(-1,1)*vol right-hand side",
            "config": {"workload": f"pressure Poisson {N}^3 jittered hex ({m.numCells} cells), "
                                   "plain FP64 DPCG (dpcg.f90) to L1-relative 1e-8",
                       "N": N, "cells": m.numCells, "nnz": int(csr.nnz), "setup_s": setup},
            "cpu_baseline": {"value": v, "unit": "s", "cores": 1, "kind": "port",
                             "sample": f"{S} DPCG sweeps per step on 1 host thread (the reference "
                                       f"is serial), scaled to {sweeps_needed} sweeps"},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fcg", choices=["fcg", "reference"])
    ap.add_argument("--N", type=int, default=256)
    ap.add_argument("--cpu-sample", type=int, default=10, help="oracle sweeps timed for cpu_baseline")
    ap.add_argument("--ref-sample", type=int, default=10, help="oracle sweeps per reference step")
    ap.add_argument("--ref-sweeps", type=int, default=1200,
                    help="sweep count used by the reference arm when none is recorded")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--solver", default="dpcg_mixed",
                    choices=["dpcg_mixed", "dpcg", "iccg", "bicgstab"])
    ap.add_argument("--no-graph", action="store_true",
                    help="host-driven sweep loop instead of the CUDA-graph WHILE loop")
    args = ap.parse_args()
    if args.no_graph:
        os.environ["FCG_NO_GRAPH"] = "1"

    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return

    import torch

    import freecappuccino_gb300 as fcg
    from freecappuccino_gb300 import _lib

    torch.cuda.set_device(local)
    lib = _lib.load()
    N = args.N
    m, mu, phi, su, t_mesh = build_system(N)
    t0 = time.perf_counter()
    ctx = fcg.Context(m, device=local)
    t_bind = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    n, nnz = m.numCells, m.nnz
    dev = torch.device("cuda", local)
    with torch.cuda.stream(stream):
        mu_d = torch.from_numpy(mu).to(dev)
        phi_d = torch.from_numpy(phi).to(dev)
        su_d = torch.from_numpy(su).to(dev)
        a_d, su_d = ctx.laplacian(mu_d, phi_d, su_d)
        fi0 = torch.zeros(n, dtype=torch.float64, device=dev)
    stream.synchronize()

    method = args.solver

    def run(name):
        return getattr(ctx, name)(a_d, su_d, fi0, TOL, NSW, want_res=False)

    for _ in range(args.warmup):
        run(method)
    sampler = ClockSampler(local)
    sampler.start()
    barrier(ws)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    reports = []
    for e0, e1 in evs:
        e0.record(stream)
        reports.append(run(method))
        e1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    clocks = sampler.stop()
    step_s = [e0.elapsed_time(e1) * 1e-3 for e0, e1 in evs]
    t_solve = reduce_max(ws, statistics.mean(step_s))
    last = reports[-1]
    iters = last.iters
    per_solve_launches = {"dpcg": lambda it: 3 + 3 * it, "dpcg_mixed": lambda it: 6 + 5 * it}
    launches = sum(per_solve_launches.get(method, lambda it: 3 + 3 * it)(r.iters) for r in reports)
    x_method = last.fi.clone()

    # Per-kernel device time of the method's sweep, CUDA events around each launch.
    prof = ctx.profile_sweeps(20)
    peak, peak_kind = peaks()
    if method == "dpcg_mixed":
        dom = "k_mx_spmv"
        dom_bytes = 8 * nnz + 4 * (n + 1) + 8 * n  # FP32 values + int32 columns, FP32 x/y
        sweep_bytes = dom_bytes + 36 * n           # + FP32 vector passes of one sweep
        dom_desc = "k_mx_spmv (FP32 sliced-ELL SpMV of the scaled matrix + p.Ap, 256^3)"
    else:
        dom = "k_cg_spmv"
        dom_bytes = spmv_bytes(n, nnz)
        sweep_bytes = dpcg_iter_bytes(n, nnz)
        dom_desc = "k_cg_spmv (FP64 sliced-ELL SpMV + p.Ap, 256^3)"
    t_dom = prof[dom] * 1e-3
    achieved = dom_bytes / t_dom / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        traffic = json.load(open(tp)).get(dom, {}).get(f"bytes_per_launch_{N}")
    roof = {"kernel": dom_desc, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": dom_bytes, "launch_ms": t_dom * 1e3,
            "sweep_kernels_ms": prof}
    sweep_gbs = sweep_bytes / (t_solve / max(iters, 1)) / 1e9

    # Plain FP64 DPCG on the same system: the method the headline is compared with.
    fp64 = None
    if method != "dpcg":
        run("dpcg")
        t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0e.record(stream)
        r64 = run("dpcg")
        t1e.record(stream)
        torch.cuda.synchronize()
        t64 = reduce_max(ws, t0e.elapsed_time(t1e) * 1e-3)
        err = float((x_method - r64.fi).abs().max() / r64.fi.abs().max())
        fp64 = {"dpcg_fp64_s": t64, "dpcg_fp64_sweeps": r64.iters, "speedup_vs_fp64": t64 / t_solve,
                "max_rel_diff_vs_fp64_solution": err,
                "fp64_sweep_GBps": dpcg_iter_bytes(n, nnz) / (t64 / r64.iters) / 1e9}

    # Standalone FP64 SpMV (one event pair per launch: host gaps are not counted).
    x = torch.rand(n, dtype=torch.float64, device=dev)
    y = torch.empty_like(x)
    ctx.spmv(None, x, y)
    pairs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
             for _ in range(20)]
    for s0, s1 in pairs:
        s0.record(stream)
        ctx.spmv(None, x, y)
        s1.record(stream)
    torch.cuda.synchronize()
    t_spmv = statistics.median(s0.elapsed_time(s1) for s0, s1 in pairs) * 1e-3
    spmv64 = {"kernel": "k_spmv (FP64)", "launch_ms": t_spmv * 1e3,
              "achieved_GBps": spmv_bytes(n, nnz) / t_spmv / 1e9,
              "frac": spmv_bytes(n, nnz) / t_spmv / 1e9 / peak}

    # End to end through the C ABI with pinned host buffers: copies inside the timed region.
    e2e_s = []
    if args.e2e_steps > 0:
        a_h = a_d.cpu().pin_memory()
        su_h = su_d.cpu().pin_memory()
        fi_h = torch.zeros(n, dtype=torch.float64).pin_memory()
    for _ in range(args.e2e_steps):
        fi_h.zero_()
        resor = C.c_double()
        rep = _lib.SolveReport()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        entry = lib.fcg_dpcg_mixed if method == "dpcg_mixed" else lib.fcg_dpcg
        rc = entry(ctx.h, a_h.data_ptr(), su_h.data_ptr(), fi_h.data_ptr(), None, TOL, NSW,
                   C.byref(resor), C.byref(rep))
        e1.record(stream)
        torch.cuda.synchronize()
        assert rc == 0, rc
        e2e_s.append(e0.elapsed_time(e1) * 1e-3)
    e2e = None
    if e2e_s:
        e2e = {"value": reduce_max(ws, statistics.mean(e2e_s)), "unit": "s",
               "h2d_bytes_per_step": 8 * nnz + 16 * n, "d2h_bytes_per_step": 8 * n}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(m, mu, phi, su, iters, args.cpu_sample)

    if rank == 0:
        line = {"metric": METRIC, "value": t_solve, "unit": "s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_solve * 1e3, "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 sweeps, f64 residual/updates" if method == "dpcg_mixed" else "f64",
                "data": "synthetic: seeded jittered hex mesh and U(-1,1)*vol right-hand side",
                "config": {"workload": f"pressure Poisson {N}^3 jittered hex ({n} cells, nnz {nnz}), "
                                       "solved to L1-relative 1e-8 (true FP64 residual)",
                           "method": method, "N": N, "cells": n, "nnz": nnz,
                           "jitter": JITTER, "tolerance": TOL, "sweeps": iters,
                           "l2": "inputs larger than L2 (matrix 1.4 GB, vectors 134 MB each)",
                           "parallelism": f"replicas x{ws}"},
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
                "gpu_launches": launches,
                "extra": {"fp64_comparison": fp64, "spmv_fp64": spmv64,
                          "sweep_GBps_algorithmic": sweep_gbs, "sweep_frac": sweep_gbs / peak,
                          "l2_rel_final": last.l2_rel, "resl_over_res0": last.resl / last.res0,
                          "mesh_setup_s": t_mesh, "bind_s": t_bind, "step_s": step_s}}
        print(json.dumps(line), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
