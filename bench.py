#!/usr/bin/env python
"""Benchmark: MGCG time to a 1e-10 relative residual at N = 4097^2, mixed
precision vs FP64, and the operator apply's HBM bandwidth.

One "step" is one complete MGCG solve of the N = 4097 manufactured problem
(u = sin(pi x) cos(pi y), SBP-SAT, V-cycle to 65^2, Jacobi 3+3) from x0 = 0
to ||b - A x|| <= 1e-10 ||b||, with b resident in HBM.  `value` is the
mixed-precision time per solve (ms, lower is better); the FP64 time, the
end-to-end time through the C ABI with host buffers, the apply roofline and
a CPU baseline (the reference's sparse CPU path restated in C, OpenMP, on
this machine's host cores) are reported beside it.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
For N > 1 launch under torch.distributed.run: every rank solves its own
replica (the path does not shard; no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MGCG time to 1e-10 rel. residual at N=4097²: mixed vs FP64; apply GB/s vs HBM"
# DRAM bytes (read + write) of one sbp_apply_f64 launch at N = 4097, measured
# with ncu (dram__bytes_read.sum + dram__bytes_write.sum).
APPLY_F64_TRAFFIC = 222.6e6
WORKLOAD = ("plain/mixed matrix-free MGCG, N=4097 (16.8M unknowns), u=sin(pi x)cos(pi y), "
            "V-cycle to 65^2, weighted Jacobi 2/3 3+3, SBP-compatible restriction, "
            "bilinear prolongation, FP64 direct coarse solve, tol 1e-10")


def workload(n: int) -> str:
    """The workload string for grid n (the headline configuration is N = 4097)."""
    if n == 4097:
        return WORKLOAD
    return WORKLOAD.replace("N=4097 (16.8M unknowns)", f"N={n} ({n * n / 1e6:.1f}M unknowns)")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--grid", "--n", dest="n", type=int, default=4097,
                   help="points per side (use --grid under torch.distributed.run)")
    p.add_argument("--apply-iters", type=int, default=50)
    p.add_argument("--cpu-baseline", type=int, default=1, help="time the CPU baseline leg")
    p.add_argument("--dtype", choices=["f64", "f32"], default="f64",
                   help="operand type of --mode apply")
    p.add_argument("--mode", choices=["full", "apply", "solve-fp64", "solve-mixed", "vcycle",
                                      "high-order", "variable", "adjoint",
                                      "batch", "spmv"],
                   default="full", help="profiling modes run one part only and print a "
                   "short line (not the benchmark line)")
    return p.parse_args()


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# distributed helpers (replicas only)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self, want: int):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            backend = os.environ.get("SBP_BENCH_BACKEND", "nccl")
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg is not None:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if self.pg is None:
            return v
        import torch
        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg is not None:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# clock sampling during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int = 0):
        self.proc = None
        self.path = None
        self.dev = device_index

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.dev)], stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.25)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for k, name in enumerate(names):
                    if parts[5 + k].lower().startswith("active"):
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the reference's sparse CPU path restated in C (OpenMP)
# ---------------------------------------------------------------------------
def cpu_mgcg_timing(n: int, b_host, steps: int, warmup: int, threads: int | None = None):
    from oracle import cpu_path
    import numpy as np
    threads = threads or os.cpu_count() or 1
    cpu_path.set_threads(threads)
    t0 = time.perf_counter()
    m = cpu_path.CpuMG(n, smoother="jacobi", restriction="galerkin", coarse_n=65)
    setup = time.perf_counter() - t0
    abstol = 1e-10 * float(np.linalg.norm(b_host))
    times, iters = [], None
    for k in range(warmup + steps):
        x0 = np.zeros_like(b_host)
        t = time.perf_counter()
        x, it, norms = m.mgcg(b_host, x0, abstol)
        dt = time.perf_counter() - t
        if k >= warmup:
            times.append(dt)
        iters = it
    m.close()
    return {"ms_per_solve": 1e3 * statistics.median(times), "threads": threads, "iters": iters,
            "setup_s": setup, "solves": len(times)}


# ---------------------------------------------------------------------------
def run_reference(args, d: Dist):
    if d.rank != 0:
        return
    import numpy as np
    from sc_2022_gb300 import problems
    n = args.n
    # host-side problem (no GPU work on this arm)
    f, g, _ = problems.manufactured(n, "baseline")
    b = _host_rhs(n, f, g)
    r = cpu_mgcg_timing(n, b, args.steps, args.warmup)
    val = r["ms_per_solve"]
    cores = r["threads"]
    line = {
        "impl": "reference", "metric": METRIC, "value": round(val, 3), "unit": "ms",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(val, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (manufactured solution)",
        "config": {"workload": workload(n) + " [CPU: C restatement of the reference's sparse "
                   "CSR path, same V-cycle]", "n": n, "parallelism": "replicas"},
        "cpu_baseline": {"value": round(val, 3), "unit": "ms", "cores": cores, "kind": "port",
                         "sample": f"{r['solves']} full FP64 MGCG solves at N={n} "
                                   f"({r['iters']} iterations each), setup excluded"},
        "e2e": {"value": round(val, 3), "unit": "ms", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "detail": {"iters": r["iters"], "setup_s": round(r["setup_s"], 2)},
    }
    print(json.dumps(line), flush=True)


def _host_rhs(n, f, g):
    """b on the host with the same per-point formula as the GPU kernel."""
    import numpy as np
    h = 1.0 / (n - 1)
    w = np.ones(n)
    w[0] = w[-1] = 0.5
    cD = (-11.5, -2.0, 0.5)
    B = (h * h) * (w[:, None] * w[None, :]) * f
    for jj in range(min(3, n)):
        B[jj, :] += w * cD[jj] * g["W"]
    for jj in range(max(0, n - 3), n):
        B[jj, :] += w * cD[n - 1 - jj] * g["E"]
    B[:, 0] += h * w * (-1.0) * g["S"]
    B[:, n - 1] += h * w * (-1.0) * g["N"]
    return np.ascontiguousarray((-B).ravel())


def run_ours(args, d: Dist):
    import ctypes as C

    import numpy as np
    import torch

    import sc_2022_gb300 as sbp
    from sc_2022_gb300 import _lib, problems

    torch.cuda.set_device(d.local)
    dev = torch.device("cuda", d.local)
    n = args.n
    f, g, U = problems.manufactured(n, "baseline")
    b = problems.assemble_rhs(f, g, device=dev).reshape(-1)
    bnorm = b.norm().item()
    s64 = sbp.Solver(n, sbp.default_options(_lib.SBP_PREC_FP64))
    s32 = sbp.Solver(n, sbp.default_options(_lib.SBP_PREC_MIXED))
    x = torch.zeros_like(b)
    stream = torch.cuda.current_stream()
    lib = sbp.load_library()

    def solve(s):
        x.zero_()
        return s.mgcg(b, x, reltol=1e-10)

    def timed(fn, steps):
        d.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = None
        for _ in range(steps):
            out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        d.barrier()
        return e0.elapsed_time(e1) / steps, out

    for _ in range(args.warmup):
        solve(s32)
        solve(s64)
    sampler = ClockSampler(d.local)
    sampler.start()
    ms32, r32 = timed(lambda: solve(s32), args.steps)
    launches32 = s32.last_launches
    x32 = x.clone()
    ms64, r64 = timed(lambda: solve(s64), args.steps)
    x64 = x.clone()
    # end to end through the C ABI with host buffers: H2D of b, solve, D2H of x
    b_host = torch.empty(b.shape, dtype=torch.float64, pin_memory=True)
    b_host.copy_(b)
    x_host = torch.empty_like(b_host, pin_memory=True)
    b_dev = torch.empty_like(b)

    def e2e():
        b_dev.copy_(b_host, non_blocking=True)
        x.zero_()
        r = s32.mgcg(b_dev, x, reltol=1e-10)
        x_host.copy_(x, non_blocking=True)
        return r

    for _ in range(2):
        e2e()
    ms_e2e, _ = timed(e2e, args.steps)
    # operator apply roofline (two inputs alternated: 4 x 134 MB > L2)
    gen = torch.Generator(device=dev).manual_seed(0)
    us = [torch.randn(n * n, generator=gen, device=dev, dtype=torch.float64) for _ in range(2)]
    outs = [torch.empty_like(us[0]) for _ in range(2)]
    sp = C.c_void_p(stream.cuda_stream)

    def apply_pair():
        for k in range(2):
            rc = lib.sbp_apply_f64(C.c_void_p(us[k].data_ptr()), C.c_void_p(outs[k].data_ptr()),
                                   n, -1, sp)
            assert rc == 0

    for _ in range(3):
        apply_pair()
    ms_apply2, _ = timed(apply_pair, args.apply_iters)
    # the FP32 apply of the mixed V-cycle's operator (4 x 67 MB inputs/outputs)
    us32 = [u.float() for u in us]
    outs32 = [torch.empty_like(us32[0]) for _ in range(2)]

    def apply_pair32():
        for k in range(2):
            rc = lib.sbp_apply_f32(C.c_void_p(us32[k].data_ptr()),
                                   C.c_void_p(outs32[k].data_ptr()), n, -1, sp)
            assert rc == 0

    for _ in range(3):
        apply_pair32()
    ms_apply32_2, _ = timed(apply_pair32, args.apply_iters)
    clocks = sampler.stop()
    ms_apply = ms_apply2 / 2.0
    ms_apply32 = d.max(ms_apply32_2 / 2.0)

    ms32 = d.max(ms32)
    ms64 = d.max(ms64)
    ms_e2e = d.max(ms_e2e)
    ms_apply = d.max(ms_apply)

    # accuracy of the timed solves
    def true_rel(xv):
        out = C.c_double()
        rc = lib.sbp_residual_norm_f64(C.c_void_p(xv.data_ptr()), C.c_void_p(b.data_ptr()), n, 1,
                                       C.byref(out), sp)
        assert rc == 0
        return out.value / bnorm

    rel32, rel64 = true_rel(x32), true_rel(x64)
    err_vs_fp64 = ((x32 - x64).norm() / x64.norm()).item()

    peak, peak_kind = measured_peaks()
    apply_bytes = 16.0 * n * n
    achieved = apply_bytes / (ms_apply * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": round(ms32, 4), "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms32, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (manufactured solution u=sin(pi x)cos(pi y), b resident in HBM)",
        "config": {"workload": workload(n), "n": n, "unknowns": n * n,
                   "parallelism": "replicas" if args.gpus > 1 else "single GPU",
                   "l2": f"inputs {'larger' if 8 * n * n > 129e6 else 'smaller'} than L2 "
                         f"(b, x, r, p, Ap: {8 * n * n / 1e6:.0f} MB each)"},
        "fp64_ms_per_solve": round(ms64, 4),
        "mixed_speedup_vs_fp64": round(ms64 / ms32, 3),
        "solves_per_s_all_gpus": round(args.gpus * 1e3 / ms32, 2),
        "e2e": {"value": round(ms_e2e, 4), "unit": "ms", "h2d_bytes_per_step": 8 * n * n,
                "d2h_bytes_per_step": 8 * n * n, "path": "sbp_mgcg_solve (mixed) with pinned "
                "host b/x copied in and out every step"},
        "roofline": {"kernel": "k_apply<double> (operator apply, FP64)", "bound": "hbm",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": apply_bytes,
                     # DRAM read + write of one launch at N = 4097 from a single ncu
                     # capture (profiles/apply_f64_n4097.md); part of the output stays in L2
                     "traffic": APPLY_F64_TRAFFIC if n == 4097 else None,
                     "ms_per_launch": round(ms_apply, 5)},
        "apply_f32": {"kernel": "sbp_apply_f32 (operator apply, FP32)", "achieved_gbs":
                      round(8.0 * n * n / (ms_apply32 * 1e-3) / 1e9, 1),
                      "frac": round(8.0 * n * n / (ms_apply32 * 1e-3) / 1e9 / peak, 4),
                      "algorithmic_bytes_per_launch": 8.0 * n * n,
                      "ms_per_launch": round(ms_apply32, 5)},
        "clocks": clocks,
        "gpu_launches": int(launches32 * args.steps),
        "detail": {"iters_mixed": r32.iters, "iters_fp64": r64.iters,
                   "true_rel_residual_mixed": rel32, "true_rel_residual_fp64": rel64,
                   "mixed_vs_fp64_solution_rel_diff": err_vs_fp64,
                   "launches_per_solve": launches32,
                   "device_bytes": s32.device_bytes + s64.device_bytes},
    }
    if d.rank == 0 and args.cpu_baseline:
        bh = b.detach().cpu().numpy()
        r = cpu_mgcg_timing(n, bh, steps=1, warmup=0)
        r1 = cpu_mgcg_timing(n, bh, steps=1, warmup=0, threads=1)
        line["cpu_baseline"] = {
            "value": round(r["ms_per_solve"], 2), "unit": "ms", "cores": r["threads"],
            "kind": "port", "sample": f"1 full FP64 MGCG solve at N={n} ({r['iters']} iterations) "
                                      "with the C restatement of the reference's sparse CPU path "
                                      "(CSR SpMV, same V-cycle), setup excluded",
            "value_1_core": round(r1["ms_per_solve"], 2)}
    if d.rank == 0:
        print(json.dumps(line), flush=True)
    s32.close()
    s64.close()


def run_part(args):
    """Profiling helper: one part of the benchmark on a single GPU."""
    import ctypes as C

    import torch

    import sc_2022_gb300 as sbp
    from sc_2022_gb300 import _lib, problems
    n = args.n
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    lib = sbp.load_library()
    if args.mode == "apply":
        gen = torch.Generator(device=dev).manual_seed(0)
        dt = torch.float64 if args.dtype == "f64" else torch.float32
        fn = lib.sbp_apply_f64 if args.dtype == "f64" else lib.sbp_apply_f32
        us = [torch.randn(n * n, generator=gen, device=dev, dtype=dt) for _ in range(2)]
        outs = [torch.empty_like(us[0]) for _ in range(2)]
        for k in range(args.warmup + args.steps):
            rc = fn(C.c_void_p(us[k % 2].data_ptr()), C.c_void_p(outs[k % 2].data_ptr()), n, -1, sp)
            assert rc == 0
        torch.cuda.synchronize()
        print(json.dumps({"mode": "apply", "dtype": args.dtype, "n": n,
                          "launches": args.warmup + args.steps}))
        return
    if args.mode == "spmv":
        # the reference's matrix-free vs assembled-SpMV comparison at --n:
        # FP64 y = A x with this project's CSR SpMV and with the matrix-free apply
        from sc_2022_gb300 import csr
        A = csr.CsrOperator(n, device=dev)
        gen = torch.Generator(device=dev).manual_seed(0)
        xs = [torch.randn(n * n, generator=gen, device=dev, dtype=torch.float64) for _ in range(2)]
        ys = [torch.empty_like(xs[0]) for _ in range(2)]
        out = {"mode": "spmv", "n": n, "nnz": A.nnz}

        def run_spmv(k):
            A.matvec(xs[k % 2], ys[k % 2])

        def run_mf(k):
            assert lib.sbp_apply_f64(C.c_void_p(xs[k % 2].data_ptr()),
                                     C.c_void_p(ys[k % 2].data_ptr()), n, 1, sp) == 0

        for name, fn, nbytes in (("spmv", run_spmv, A.device_bytes + 16 * n * n),
                                 ("matrix_free", run_mf, 16 * n * n)):
            for k in range(args.warmup):
                fn(k)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for k in range(args.steps):
                fn(k)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            out[name + "_us"] = round(1e3 * ms, 2)
            out[name + "_gbs"] = round(nbytes / (ms * 1e-3) / 1e9, 1)
        out["matrix_free_speedup"] = round(out["spmv_us"] / out["matrix_free_us"], 3)
        print(json.dumps(out))
        return
    if args.mode == "batch":
        # 256 problems, N log-uniform over {65..1025}, bump/trig data, FP64
        # MGCG to 1e-10: batched vs one solve at a time
        import time
        ns, bs = problems.batch_problems(256, seed=4, device=dev)
        opts = sbp.default_options()
        B = sbp.BatchSolver(ns, opts)
        xs = [torch.zeros_like(b) for b in bs]
        budgets = B.autotune(bs, xs)
        solvers = {m: sbp.Solver(m, opts) for m in sorted(set(ns))}

        def batched():
            for x in xs:
                x.zero_()
            return B.mgcg(bs, xs, reltol=1e-10, maxiter=200)

        def sequential():
            out = []
            for m, b, x in zip(ns, bs, xs):
                x.zero_()
                out.append(solvers[m].mgcg(b, x, reltol=1e-10, maxiter=200))
            return out

        res = {}
        for name, fn in (("batched", batched), ("sequential", sequential)):
            for _ in range(args.warmup):
                fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                r = fn()
            torch.cuda.synchronize()
            res[name + "_ms"] = round(1e3 * (time.perf_counter() - t0) / args.steps, 3)
            res[name + "_iters"] = sum(x.iters for x in r)
        res.update({"mode": "batch", "problems": len(ns),
                    "sizes": {str(m): ns.count(m) for m in sorted(set(ns))},
                    "speedup": round(res["sequential_ms"] / res["batched_ms"], 3),
                    "launches_batched": B.last_launches, "cta_budgets": budgets})
        print(json.dumps(res))
        return
    if args.mode == "high-order":
        # p = 4 and p = 6 operators at --n: the FP64 apply (16 B per point
        # moved) and MGCG to 1e-10 from zero on a seeded random right-hand side
        out = {"mode": "high-order", "n": n}
        gen = torch.Generator(device=dev).manual_seed(0)
        us = [torch.randn(n * n, generator=gen, device=dev, dtype=torch.float64) for _ in range(2)]
        outs = [torch.empty_like(us[0]) for _ in range(2)]
        hbm, hbm_src = measured_peaks()
        out["hbm_peak_gbs"] = hbm
        out["hbm_peak_source"] = hbm_src
        for p in (4, 6):
            for k in range(args.warmup):
                sbp.matrix_free_A_high_order_GPU(us[k % 2], outs[k % 2], p=p)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for k in range(args.steps):
                sbp.matrix_free_A_high_order_GPU(us[k % 2], outs[k % 2], p=p)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            gbs = 16.0 * n * n / (ms * 1e-3) / 1e9
            out[f"p{p}_apply_us"] = round(1e3 * ms, 2)
            out[f"p{p}_apply_gbs"] = round(gbs, 1)
            out[f"p{p}_apply_frac_of_hbm"] = round(gbs / hbm, 3)
            for tag, prec in (("fp64", _lib.SBP_PREC_FP64), ("mixed", _lib.SBP_PREC_MIXED)):
                s = sbp.HighOrderSolver(n, p, sbp.default_options(prec))
                x = torch.zeros_like(us[0])
                for _ in range(args.warmup):
                    x.zero_()
                    s.mgcg(us[0], x, reltol=1e-10, maxiter=200)
                torch.cuda.synchronize()
                e0.record()
                for _ in range(args.steps):
                    x.zero_()
                    r = s.mgcg(us[0], x, reltol=1e-10, maxiter=200)
                e1.record()
                torch.cuda.synchronize()
                out[f"p{p}_mgcg_{tag}_ms"] = round(e0.elapsed_time(e1) / args.steps, 3)
                out[f"p{p}_mgcg_{tag}_iters"] = r.iters
                out[f"p{p}_mgcg_{tag}_converged"] = r.converged
                s.close()
        print(json.dumps(out))
        return
    if args.mode == "variable":
        # div(c grad u) at --n with the seeded layered coefficient (c from 1
        # to 10 across y = 1/2): the FP64 apply from nodal c (u, c read, out
        # written: 24 B per point) and MGCG to 1e-10 from zero
        out = {"mode": "variable", "n": n, "coefficient": "layered 1..10"}
        x1 = torch.linspace(0.0, 1.0, n, device=dev, dtype=torch.float64)
        coef = (1.0 + 4.5 * (1.0 + torch.tanh((x1 - 0.5) * (n - 1) / 2.0)))[:, None].expand(
            n, n).contiguous().reshape(-1)
        gen = torch.Generator(device=dev).manual_seed(0)
        us = [torch.randn(n * n, generator=gen, device=dev, dtype=torch.float64) for _ in range(2)]
        outs = [torch.empty_like(us[0]) for _ in range(2)]
        hbm, hbm_src = measured_peaks()
        for k in range(args.warmup):
            sbp.matrix_free_A_variable_GPU(us[k % 2], coef, outs[k % 2])
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for k in range(args.steps):
            sbp.matrix_free_A_variable_GPU(us[k % 2], coef, outs[k % 2])
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        gbs = 24.0 * n * n / (ms * 1e-3) / 1e9
        out.update({"apply_us": round(1e3 * ms, 2), "apply_gbs": round(gbs, 1),
                    "apply_frac_of_hbm": round(gbs / hbm, 3), "hbm_peak_source": hbm_src})
        for tag, prec in (("fp64", _lib.SBP_PREC_FP64), ("mixed", _lib.SBP_PREC_MIXED)):
            s = sbp.VariableCoefficientSolver(n, coef, sbp.default_options(prec))
            x = torch.zeros_like(us[0])
            for _ in range(args.warmup):
                x.zero_()
                s.mgcg(us[0], x, reltol=1e-10, maxiter=200)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(args.steps):
                x.zero_()
                r = s.mgcg(us[0], x, reltol=1e-10, maxiter=200)
            e1.record()
            torch.cuda.synchronize()
            out[f"mgcg_{tag}_ms"] = round(e0.elapsed_time(e1) / args.steps, 3)
            out[f"mgcg_{tag}_iters"] = r.iters
            out[f"mgcg_{tag}_converged"] = r.converged
            out["levels"] = s.levels
            s.close()
        print(json.dumps(out))
        return
    if args.mode == "adjoint":
        # the gradient of L = sum_k 1/2 (u_k - t_k)' H~ (u_k - t_k) with respect
        # to the sources f_k and the boundary data g_k, for a batch of 16 bump
        # problems at --grid, through torch autograd: forward MGCG solves, the
        # H-misfit, then the adjoint MGCG solves and the transposed right-hand
        # side map, all to 1e-10
        import time

        import numpy as np

        from sc_2022_gb300 import adjoint as adj
        B = 16
        fs, gs = [], {side: [] for side in "WESN"}
        for k in range(B):
            f, g = problems.bump_problem(n, 5000 + k)
            fs.append(np.asarray(f).reshape(n, n))
            for side in "WESN":
                gs[side].append(np.asarray(g[side]))
        f0 = torch.tensor(np.stack(fs), dtype=torch.float64, device=dev)
        g0 = [torch.tensor(np.stack(gs[side]), dtype=torch.float64, device=dev)
              for side in "WESN"]
        targets = 1e-3 * torch.randn((B, n, n), dtype=torch.float64, device=dev,
                                     generator=torch.Generator(device=dev).manual_seed(3))
        out = {"mode": "adjoint", "n": n, "batch": B, "reltol": 1e-10}
        grads = {}
        for tag, prec in (("fp64", _lib.SBP_PREC_FP64), ("mixed", _lib.SBP_PREC_MIXED)):
            s = sbp.Solver(n, sbp.default_options(prec))

            def gradient():
                f = f0.clone().requires_grad_(True)
                g = [t.clone().requires_grad_(True) for t in g0]
                u = adj.PoissonSolve.apply(f, *g, s, 1e-10)
                loss = adj.HMisfit.apply(u, targets)
                loss.backward()
                return loss, f.grad

            for _ in range(args.warmup):
                gradient()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                loss, df = gradient()
            torch.cuda.synchronize()
            out[f"{tag}_ms_per_gradient"] = round(1e3 * (time.perf_counter() - t0) / args.steps, 2)
            out[f"{tag}_loss"] = float(loss.detach())
            grads[tag] = df.detach().clone()
            s.close()
        out["mixed_vs_fp64_df_rel_diff"] = float((grads["mixed"] - grads["fp64"]).norm() /
                                                 grads["fp64"].norm())
        print(json.dumps(out))
        return
    if args.mode == "vcycle":
        # time one V-cycle (mixed and FP64) for the default hierarchy at --n
        out = {"mode": "vcycle", "n": n}
        gen = torch.Generator(device=dev).manual_seed(0)
        b = torch.randn(n * n, generator=gen, device=dev, dtype=torch.float64)
        v = torch.empty_like(b)
        for name, prec in (("mixed", _lib.SBP_PREC_MIXED), ("fp64", _lib.SBP_PREC_FP64)):
            s = sbp.Solver(n, sbp.default_options(prec))
            for _ in range(args.warmup):
                s.vcycle(b, v)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                s.vcycle(b, v)
            e1.record()
            torch.cuda.synchronize()
            out[name + "_us"] = round(1e3 * e0.elapsed_time(e1) / args.steps, 2)
            out["levels"] = s.levels
            s.close()
        print(json.dumps(out))
        return
    prec = _lib.SBP_PREC_MIXED if args.mode == "solve-mixed" else _lib.SBP_PREC_FP64
    f, g, _ = problems.manufactured(n, "baseline")
    b = problems.assemble_rhs(f, g, device=dev).reshape(-1)
    s = sbp.Solver(n, sbp.default_options(prec))
    x = torch.zeros_like(b)
    for _ in range(args.warmup + args.steps):
        x.zero_()
        r = s.mgcg(b, x, reltol=1e-10)
    torch.cuda.synchronize()
    print(json.dumps({"mode": args.mode, "n": n, "iters": r.iters, "converged": r.converged,
                      "launches_per_solve": s.last_launches}))


def main():
    args = parse_args()
    if args.mode != "full":
        run_part(args)
        return
    d = Dist(args.gpus)
    try:
        if args.impl == "reference":
            run_reference(args, d)
        else:
            run_ours(args, d)
    finally:
        d.close()


if __name__ == "__main__":
    main()
