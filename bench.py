#!/usr/bin/env python
"""Benchmark: time to a 1e-6 true relative residual on the 96³
dielectric-sphere scatterer (40 spheres, ε = 12.25, 10-cell PML, λ = 16,
x-polarised current sheet at z = 15), mixed precision versus FP64 on the same
GB300, plus the HBM roofline of the operator kernel.

A step is one complete mixed-precision BiCGStab(4) solve (complex64 operator and
Krylov vectors, FP64 reductions and reliable FP64 residual replacement) with
b resident in HBM.  The same workload is also solved once in plain complex128
(the FP64 comparison), end to end through the C ABI with host buffers
(``e2e``), and — on a bounded sample — by an OpenMP complex128 CSR BiCGStab(4)
of the assembled A on all host cores (``cpu_baseline``), the same algorithm.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun with N > 1 every rank solves its own replica (the path does
not shard: replicas only); the reported time is the maximum over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time to 1e-6 rel. residual, mixed vs FP64 on same GB300; matvec HBM GB/s"
WORKLOAD = "96^3 dielectric-sphere scatterer: 40 spheres r~U[3,8] eps=12.25, 10-cell PML, lambda=16, x-pol sheet z=15"
METHOD, ELL = "bicgstabl", 4   # BiCGStab(4) in both precisions
# The mixed solve stops at a 5e-7 true residual with reliable updates every
# 100-fold residual drop: at a 1e-6 stop its field error against an accurate
# FP64 solution was 0.7-1.9e-5 (error/residual ratios of 11-31 on this
# system, depending on where in a residual drop the stop falls), at 5e-7 it
# stays near 5e-6.  The timed mixed solve therefore reaches a stricter
# residual than the FP64 one it is compared with.
MIXED_TOL, MIXED_DELTA = 5e-7, 0.01


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _pg_init(ws, backend):
    import torch.distributed as dist
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(value, ws, device=None):
    """Max of a float over all ranks (identity when ws == 1)."""
    if ws == 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
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
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


_CPU = {}


def _cpu_system():
    """The oracle's assembled complex128 CSR A and b for this workload (built
    once), held for the OpenMP CSR BiCGStab(4) of oracle/csr_bicgstab.c on all
    host cores."""
    if not _CPU:
        import __graft_entry__ as ge
        from oracle import fdfd_oracle as O
        from oracle.build_oracle import build as build_oracle
        from oracle.csr_native import NativeCSR
        build_oracle()
        pkg = ge.load_package()
        mdl, om = pkg.workloads.config2()
        g = O.uniform_grid(mdl.grid.N)
        objs = [O.Sphere(o.shape.c, o.shape.r, o.eps) for o in mdl.objects]
        t0 = time.perf_counter()
        S = O.System(g, om, mdl.Npml, objs)
        S.add_planesrc(2, 15.0, (1, 0, 0))
        b = S.b()
        M = NativeCSR(S.A, threads=os.cpu_count() or 1)
        _CPU.update(b=b, M=M, t_asm=time.perf_counter() - t0)
    return _CPU


def _cpu_model():
    """The host CPU's model name (lscpu), else the machine type."""
    import platform
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return platform.processor() or platform.machine()


def cpu_sample(seconds=8.0):
    """Time per operator application of the CPU baseline's FP64 BiCGStab(4)
    over a bounded sample (about `seconds` of work, at least 3 cycles)."""
    c = _cpu_system()
    M, b = c["M"], c["b"]
    t0 = time.perf_counter()
    _, mv, _ = M.bicgstabl(b, ell=4, tol=1e-300, maxmv=8)
    t_est = (time.perf_counter() - t0) / max(mv, 1)
    mvs = int(min(20000, max(24, seconds / max(t_est, 1e-6))))
    t0 = time.perf_counter()
    _, mv, _ = M.bicgstabl(b, ell=4, tol=1e-300, maxmv=mvs)
    t_mv = (time.perf_counter() - t0) / max(mv, 1)
    return {"t_mv": t_mv, "matvecs": mv, "t_assemble": c["t_asm"], "nnz": M.nnz, "threads": M.threads}


def cpu_full_solve():
    """One complete FP64 BiCGStab(4) solve of the workload to a relative
    residual of 1e-6 by the CPU baseline (OpenMP complex128 CSR on all host
    threads), timed by the wall clock; returns (seconds, applications, true
    relative residual)."""
    c = _cpu_system()
    M, b = c["M"], c["b"]
    t0 = time.perf_counter()
    x, mv, _ = M.bicgstabl(b, ell=4, tol=1e-6, maxmv=2000000)
    t = time.perf_counter() - t0
    rel = float(np.linalg.norm(b - M.matvec(x)) / np.linalg.norm(b))
    return t, mv, rel


def run_reference(args):
    """The CPU arm: W + K bounded samples (about 2 s each) of the CPU
    baseline's per-application time, then ONE complete solve of the same
    system to 1e-6 timed by the wall clock — the reported value (a full solve
    takes several minutes on the host cores, so it is not repeated K times)."""
    ws, rank, local = _dist()
    if rank != 0:
        return 0
    samples = []
    r = None
    for s in range(args.warmup + args.steps):
        r = cpu_sample(seconds=2.0)
        if s >= args.warmup:
            samples.append(r["t_mv"])
    t_mv = statistics.median(samples)
    t_full, mv_full, rel_full = cpu_full_solve()
    sample = (f"one complete FP64 BiCGStab(4) solve to 1e-6 ({mv_full} operator applications, true relres "
              f"{rel_full:.2e}) of the same 96^3 system by the CPU baseline (complex128 CSR, {r['nnz']} nnz, OpenMP "
              f"on {r['threads']} host threads of {os.cpu_count()}, {_cpu_model()}; oracle/csr_bicgstab.c), wall "
              f"clock; plus {args.steps} bounded samples of {r['matvecs']} applications: median "
              f"{t_mv*1e3:.2f} ms per application")
    line = {"metric": METRIC, "value": t_full, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_full * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": WORKLOAD, "precision": "fp64", "solver": "BiCGStab(4)", "tol": 1e-6},
            "cpu_baseline": {"value": t_full, "unit": "s", "cores": r["threads"], "kind": "port", "sample": sample},
            "e2e": {"value": t_full, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "cpu_matvecs": mv_full, "cpu_relres": rel_full, "cpu_ms_per_application": t_mv * 1e3}
    print(json.dumps(line))
    return 0


def operator_320(pkg, dev, hbm_peak, reps=10):
    """The complex64 and complex128 operator on the 320³ workload (400
    spheres r ~ U[4, 16], ε ∈ {1, 2.25, 12.25}, 12-cell PML, λ = 24): CUDA
    events on the library's stream around single launches, L2 flushed by a
    256 MiB read before each (inputs 0.8 / 1.6 GB, far above L2)."""
    import torch
    mdl, om, _ = pkg.workloads.config5()
    A = pkg.create_A(mdl, om)
    _, eo, _ = A.get_eps()
    n_off = int(np.count_nonzero(np.any(eo != 0, axis=-1)))
    del eo
    stream = torch.cuda.ExternalStream(A.stream, device=dev)
    flush = torch.ones(64 << 20, dtype=torch.float32, device=dev)
    out = {"workload": "320^3, 400 spheres r~U[4,16] eps in {1,2.25,12.25}, 12-cell PML, lambda=24",
           "cells": A.ncell, "off_diagonal_corners": n_off}
    for prec, dt, per_cell, per_off in (("c64", torch.float32, 60, 12), ("c128", torch.float64, 120, 24)):
        xin = torch.randn(A.n, 2, device=dev, dtype=dt)
        yout = torch.empty_like(xin)
        ts = []
        with torch.cuda.stream(stream):
            for r in range(reps + 2):
                flush.sum()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                A.matvec_dev(xin.data_ptr(), yout.data_ptr(), prec)
                e1.record(stream)
                e1.synchronize()
                if r >= 2:
                    ts.append(e0.elapsed_time(e1) / 1e3)
        t = statistics.mean(ts)
        alg = A.ncell * per_cell + n_off * per_off
        out[prec] = {"us": t * 1e6, "alg_bytes": alg, "achieved_gbs": alg / t / 1e9,
                     "frac": alg / t / 1e9 / hbm_peak, "cells_per_s": A.ncell / t}
        del xin, yout
    A.close()
    torch.cuda.empty_cache()
    return out


def run_ours(args):
    import torch
    ws, rank, local = _dist()
    if ws > 1:
        torch.cuda.set_device(local)
        _pg_init(ws, "nccl")
    import __graft_entry__ as ge
    pkg = ge.load_package()
    wl = pkg.workloads
    dev = torch.device("cuda", local)
    mdl, om = wl.config2(seed=1000 + rank)
    A = pkg.create_A(mdl, om, device=local)
    b = pkg.create_b(mdl, om)
    n = A.n
    stream = torch.cuda.ExternalStream(A.stream, device=dev)
    b_dev = torch.from_numpy(b.view(np.float64).reshape(n, 2)).to(dev)
    x_dev = torch.zeros_like(b_dev)
    tol = 1e-6
    for _ in range(args.warmup):
        A.solve_dev(b_dev.data_ptr(), x_dev.data_ptr(), tol=MIXED_TOL, precision="mixed", method=METHOD, ell=ELL,
                    delta=MIXED_DELTA)
    torch.cuda.synchronize(dev)
    _barrier(ws)
    clk = ClockSampler(local)
    clk.start()
    times, stats = [], []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    for _ in range(args.steps):
        ev0.record(stream)
        st = A.solve_dev(b_dev.data_ptr(), x_dev.data_ptr(), tol=MIXED_TOL, precision="mixed", method=METHOD, ell=ELL,
                         delta=MIXED_DELTA)
        ev1.record(stream)
        ev1.synchronize()
        times.append(ev0.elapsed_time(ev1) / 1e3)
        stats.append(st)
    torch.cuda.synchronize(dev)
    _barrier(ws)
    clocks = clk.stop()
    t_mixed = max_over_ranks(statistics.mean(times), ws, dev)
    x_mixed = x_dev.cpu().numpy().view(np.complex128).reshape(-1).copy()

    # FP64 comparison on the same GPU (one solve)
    x64_dev = torch.zeros_like(b_dev)
    ev0.record(stream)
    st64 = A.solve_dev(b_dev.data_ptr(), x64_dev.data_ptr(), tol=tol, precision="fp64", method=METHOD,
                       ell=ELL)
    ev1.record(stream)
    ev1.synchronize()
    t_fp64 = max_over_ranks(ev0.elapsed_time(ev1) / 1e3, ws, dev)
    x_fp64 = x64_dev.cpu().numpy().view(np.complex128).reshape(-1)
    # field error against an accurate FP64 solution (continued from the FP64
    # solve to a 1e-9 residual; untimed): at 1e-6 both solves still carry
    # errors of that order times the conditioning, so they are not compared
    # with each other
    A.solve_dev(b_dev.data_ptr(), x64_dev.data_ptr(), tol=1e-9, precision="fp64", method=METHOD, ell=ELL,
                x0_given=True)
    x_ref = x64_dev.cpu().numpy().view(np.complex128).reshape(-1)
    ferr = float(np.linalg.norm(x_mixed - x_ref) / np.linalg.norm(x_ref))
    ferr64 = float(np.linalg.norm(x_fp64 - x_ref) / np.linalg.norm(x_ref))

    # operator kernel roofline: complex64 A·x launches on inputs > L2, L2 flushed before each
    ed, eo, _ = A.get_eps()
    n_off = int(np.count_nonzero(np.any(eo != 0, axis=-1)))
    alg64 = A.ncell * 60 + n_off * 12
    alg128 = A.ncell * 120 + n_off * 24
    xin = torch.randn(n, 2, device=dev, dtype=torch.float32)
    yout = torch.empty_like(xin)
    xin64 = torch.randn(n, 2, device=dev, dtype=torch.float64)
    yout64 = torch.empty_like(xin64)
    # L2 flush by READING 256 MiB (> 129 MB L2): evicts the operands and
    # leaves only clean lines, so the timed launch is not charged for the
    # write-back of a flush buffer
    flush = torch.ones(64 << 20, dtype=torch.float32, device=dev)
    def timed(prec, xx, yy, reps):
        ts = []
        with torch.cuda.stream(stream):
            for r in range(reps + 2):
                flush.sum()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                A.matvec_dev(xx.data_ptr(), yy.data_ptr(), prec)
                e1.record(stream)
                e1.synchronize()
                if r >= 2:
                    ts.append(e0.elapsed_time(e1) / 1e3)
        return statistics.mean(ts)
    t_mv = timed("c64", xin, yout, 20)
    t_mv128 = timed("c128", xin64, yout64, 5)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg64 / t_mv / 1e9

    # the 320³ operator (400 spheres, the workload the ≥ 0.70-of-HBM target
    # is stated on): complex64 and complex128 A x launches timed the same way
    op320 = None
    if not args.no_320 and rank == 0:
        op320 = operator_320(pkg, dev, hbm_peak)

    # end to end through the C ABI with pinned host buffers (copies inside)
    bh = torch.from_numpy(b.view(np.float64).reshape(n, 2).copy()).pin_memory()
    xh = torch.zeros_like(bh).pin_memory()
    e2e_t = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        xs, _st = A.solve(bh.numpy().view(np.complex128).reshape(-1), tol=MIXED_TOL, precision="mixed", method=METHOD,
                          ell=ELL, delta=MIXED_DELTA)
        e2e_t.append(time.perf_counter() - t0)
    e2e = max_over_ranks(statistics.mean(e2e_t), ws, dev)

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            r = cpu_sample(seconds=10.0)
            proj = r["t_mv"] * st64["matvecs"]
            cpu = {"value": proj, "unit": "s", "cores": r["threads"], "kind": "port",
                   "sample": (f"{r['matvecs']} operator applications of FP64 BiCGStab(4) on the CPU baseline "
                              f"(complex128 CSR, {r['nnz']} nnz, OpenMP on {r['threads']} host threads of "
                              f"{os.cpu_count()}, {_cpu_model()}) on the same "
                              f"system: {r['t_mv']*1e3:.2f} ms per application, projected to the {st64['matvecs']} "
                              f"applications the FP64 GPU solve needed")}
        line = {
            "metric": METRIC, "value": t_mixed, "unit": "s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_mixed * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64 (double-float FP32 reductions, FP64 residual replacement)",
            "data": "synthetic (seeded spheres, seed 1000+rank)",
            "config": {"workload": WORKLOAD, "cells": A.ncell, "unknowns": n, "solver": "BiCGStab(4)",
                       "tol": tol, "mixed_stop": MIXED_TOL, "mixed_delta": MIXED_DELTA, "l2": "solve working set > L2 (12 c64 + 3 c128 vectors = 0.38 GB); L2 "
                                         "flushed by a 256 MiB read before each roofline launch",
                       "parallelism": "replicas" if ws > 1 else "1 GPU"},
            "fp64_time_s": t_fp64, "mixed_speedup_vs_fp64": t_fp64 / t_mixed,
            "iterations": stats[-1]["iterations"], "fp64_iterations": st64["iterations"],
            "matvecs": stats[-1]["matvecs"], "fp64_matvecs": st64["matvecs"],
            "refinements": stats[-1]["refinements"], "relres": stats[-1]["relres"],
            "fp64_relres": st64["relres"], "field_err_vs_fp64_1e-9": ferr, "fp64_field_err_vs_fp64_1e-9": ferr64,
            "matvec_c64_us": t_mv * 1e6, "matvec_c128_us": t_mv128 * 1e6,
            "cells_per_s_c64": A.ncell / t_mv,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": None,
                         "kernel": "k_apply_v2<float, EPI_STORE> (y = A x, complex64)",
                         "alg_bytes_per_launch": alg64,
                         "traffic_note": "ncu dram bytes per launch are kept in profiles/, not read by this script",
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s"},
            "operator_320": op320,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": 16 * n},
            "clocks": clocks,
            "gpu_launches": int(sum(s["launches"] for s in stats)),
        }
        print(json.dumps(line))
    A.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_profile(args):
    """Small, self-terminating runs for ncu: `matvec` applies the complex64
    operator `--reps` times on a sphere model of size `--grid`; `solve` runs
    the bench workload's mixed solve capped at `--maxit` iterations."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    dev = torch.device("cuda", 0)
    if args.profile == "matvec":
        N = tuple(int(v) for v in args.grid.split(","))
        g = pkg.uniform_grid(N)
        om = 2 * np.pi / 16
        mdl = pkg.ModelFull(g)
        pkg.set_ωpml(mdl, om)
        pkg.set_Npml(mdl, ((10,) * 3, (10,) * 3))
        rng = np.random.default_rng(7)
        if args.spheres == "c5":
            # the 320³ workload's sphere statistics, count scaled to the grid volume
            nsph = max(1, int(round(400 * np.prod(N) / 320 ** 3)))
            sph = pkg.workloads._spheres(rng, N, 12, nsph, 4.0, 16.0, [1.0, 2.25, 12.25])
        else:
            sph = pkg.workloads._spheres(rng, N, 10, 40, 3.0, 8.0, [12.25])
        for c, r, e in sph:
            pkg.add_obj(mdl, "dielectric", pkg.Sphere(c, r), ε=e)
        A = pkg.create_A(mdl, om)
        prec = args.precision
        dt = torch.float32 if prec == "c64" else torch.float64
        x = torch.randn(A.n, 2, device=dev, dtype=dt)
        y = torch.empty_like(x)
        A.sync()
        # an NVTX range around the timed applications, so that a profiler can
        # skip the autotuner's launches (ncu --nvtx --nvtx-include "matvec/")
        torch.cuda.nvtx.range_push("matvec")
        for _ in range(args.reps):
            A.matvec_dev(x.data_ptr(), y.data_ptr(), prec)
        A.sync()
        torch.cuda.nvtx.range_pop()
        print(f"profile matvec {N} {prec} x{args.reps} done")
    else:
        mdl, om = pkg.workloads.config2()
        A = pkg.create_A(mdl, om)
        b = pkg.create_b(mdl, om)
        bd = torch.from_numpy(b.view(np.float64).reshape(-1, 2)).to(dev)
        xd = torch.zeros_like(bd)
        try:
            st = A.solve_dev(bd.data_ptr(), xd.data_ptr(), tol=1e-6, precision="mixed", maxit=args.maxit,
                             check_every=10)
        except pkg.FDFDError as e:
            st = getattr(e, "stats", None) or str(e)
        print(f"profile solve maxit={args.maxit}: {st}")
    A.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-320", action="store_true", help="skip the 320^3 operator timing")
    ap.add_argument("--profile", choices=["matvec", "solve"], help="short run for ncu (no bench line)")
    ap.add_argument("--grid", default="256,256,128")
    ap.add_argument("--precision", default="c64", choices=["c64", "c128"])
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--spheres", default="c2", choices=["c2", "c5"],
                    help="profile matvec: sphere statistics of the 96^3 (c2) or the 320^3 (c5) workload")
    ap.add_argument("--maxit", type=int, default=100)
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
