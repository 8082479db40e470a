#!/usr/bin/env python
"""Benchmark: MGCG time to a 1e-10 relative residual at N = 4097^2, mixed
precision vs FP64, and the operator apply's HBM bandwidth.

One "step" is one complete MGCG solve of the N = 4097 manufactured problem
(u = sin(pi x) cos(pi y), SBP-SAT, V-cycle to 65^2, Jacobi 3+3) from x0 = 0
to ||b - A x|| <= 1e-10 ||b||, with b resident in HBM.  `value` is the
mixed-precision time per solve (ms, lower is better).  Beside it the line
carries the FP64 time, the end-to-end time through the C ABI with host
buffers, the per-kernel times of the solve and the roofline of its dominant
kernel, the operator applies against HBM (and the FP64 apply against the
measured FP64 rate), the solution's distance from the C oracle's solve of
the same problem, plain FP64 CG at the same size, a CPU baseline (the
reference's sparse CPU path restated in C, OpenMP, on this machine's host
cores), and one timing of each further configuration (N = 8193 mixed, the
256-problem batch, the N = 2049 x 16 adjoint gradient, the p = 4 / 6 and
variable-coefficient solvers, assembled SpMV against the matrix-free apply).

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
import traceback

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MGCG time to 1e-10 rel. residual at N=4097²: mixed vs FP64; apply GB/s vs HBM"
WORKLOAD = ("plain/mixed matrix-free MGCG, N=4097 (16.8M unknowns), u=sin(pi x)cos(pi y), "
            "V-cycle to 65^2, weighted Jacobi 2/3 3+3, SBP-compatible restriction, "
            "bilinear prolongation, FP64 direct coarse solve, tol 1e-10")

# Algorithmic bytes per fine-grid point of the solver kernels that run on the
# finest level once per iteration (unique arrays read + written once).
KERNEL_BYTES_PER_POINT = {
    "k_dir_wave": 20,         # the same over the interior rectangle (KERNEL_POINTS)
    "CgDirF32Job": 20,        # z, p_old (f32) read; p (f32), Ap written
    "CgDirJob<double, double": 32,   # z, p_old read; p, Ap written
    "k_cg_update<": 48,       # x, r, Ap, p (f32) read; x, r, r_lo (f32) written
}
# Points one launch covers, where not the whole n x n grid: the direction
# wave does rows [65, n - 64) x columns [33, n - 32), the staged tiles the rest.
KERNEL_POINTS = {
    "k_dir_wave": lambda n: (n - 129) * (n - 65),
}


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
    p.add_argument("--extras", type=int, default=1,
                   help="time the further configurations after the headline (1 GPU only)")
    p.add_argument("--dtype", choices=["f64", "f32"], default="f64",
                   help="operand type of --mode apply")
    p.add_argument("--mode", choices=["full", "apply", "solve-fp64", "solve-mixed", "vcycle",
                                      "cg", "n8193", "high-order", "variable", "adjoint",
                                      "batch", "spmv", "profile"],
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
    """Median time of `steps` FP64 MGCG solves (after `warmup`) with the C
    restatement; also returns the last solution (the oracle's x)."""
    from oracle import cpu_path
    import numpy as np
    threads = threads or os.cpu_count() or 1
    cpu_path.set_threads(threads)
    t0 = time.perf_counter()
    m = cpu_path.CpuMG(n, smoother="jacobi", restriction="galerkin", coarse_n=65)
    setup = time.perf_counter() - t0
    abstol = 1e-10 * float(np.linalg.norm(b_host))
    times, iters, x = [], None, None
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
            "setup_s": setup, "solves": len(times), "warmup": warmup, "x": x}


def cpu_sample_text(r, n, extra=""):
    return (f"median of {r['solves']} full FP64 MGCG solves at N={n} ({r['iters']} iterations "
            f"each) after {r['warmup']} warm-up, with the C restatement of the reference's sparse "
            f"CPU path (CSR SpMV, same V-cycle), setup excluded{extra}")


# ---------------------------------------------------------------------------
def run_reference(args, d: Dist):
    if d.rank != 0:
        return
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
        "config": config_block(args, n),
        "cpu_baseline": {"value": round(val, 3), "unit": "ms", "cores": cores, "kind": "port",
                         "sample": cpu_sample_text(r, n, "; the reference itself is Julia, "
                                                   "which this machine cannot run")},
        "e2e": {"value": round(val, 3), "unit": "ms", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "detail": {"iters": r["iters"], "setup_s": round(r["setup_s"], 2)},
    }
    print(json.dumps(line), flush=True)


def config_block(args, n):
    return {"workload": workload(n), "n": n, "unknowns": n * n,
            "parallelism": "replicas" if args.gpus > 1 else "single GPU",
            "l2": f"inputs {'larger' if 8 * n * n > 129e6 else 'smaller'} than L2 "
                  f"(b, x, r, p, Ap: {8 * n * n / 1e6:.0f} MB each)"}


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


# ---------------------------------------------------------------------------
# timing helpers
# ---------------------------------------------------------------------------
def event_time(fn, steps, warmup=0, stream=None):
    """ms per call of fn over `steps` calls, CUDA events on the stream."""
    import torch
    stream = stream or torch.cuda.current_stream()
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    out = None
    for _ in range(steps):
        out = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, out


def true_rel_residual(lib, x, b, n, sign=1):
    import ctypes as C
    import torch
    out = C.c_double()
    rc = lib.sbp_residual_norm_f64(C.c_void_p(x.data_ptr()), C.c_void_p(b.data_ptr()), n, sign,
                                   C.byref(out),
                                   C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, rc
    return out.value / b.norm().item()


def short_name(k: str) -> str:
    """Kernel name without the namespace and template noise."""
    k = k.replace("sbp::", "").replace("void ", "")
    return k.split("(")[0] if not k.startswith("k_persist") else k.split(">(")[0] + ">"


def apply_timing(n, dtype, iters, dev, sign=-1):
    """ms per launch of sbp_apply_f64 / _f32 over two alternated inputs
    (4 arrays larger than L2 at N = 4097)."""
    import ctypes as C
    import torch
    import sc_2022_gb300 as sbp
    lib = sbp.load_library()
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    gen = torch.Generator(device=dev).manual_seed(0)
    dt = torch.float64 if dtype == "f64" else torch.float32
    fn = lib.sbp_apply_f64 if dtype == "f64" else lib.sbp_apply_f32
    us = [torch.randn(n * n, generator=gen, device=dev, dtype=torch.float64).to(dt)
          for _ in range(2)]
    outs = [torch.empty_like(us[0]) for _ in range(2)]

    def pair():
        for k in range(2):
            rc = fn(C.c_void_p(us[k].data_ptr()), C.c_void_p(outs[k].data_ptr()), n, sign, sp)
            assert rc == 0, rc

    ms2, _ = event_time(pair, iters, warmup=3, stream=stream)
    return ms2 / 2.0


# ---------------------------------------------------------------------------
# further configurations (one timing each; also the --mode parts)
# ---------------------------------------------------------------------------
def part_cg(n, dev, steps=1):
    """Plain FP64 matrix-free CG on A x = b (CG_CPU semantics) from zero to
    1e-10 relative residual, manufactured problem."""
    import sc_2022_gb300 as sbp
    import torch
    from sc_2022_gb300 import problems
    lib = sbp.load_library()
    f, g, _ = problems.manufactured(n, "baseline")
    b = problems.assemble_rhs(f, g, device=dev).reshape(-1)
    s = sbp.Solver(n)
    x = torch.zeros_like(b)
    s.cg(b, x, sign=1, reltol=1e-10, maxiter=20)   # captures the iteration graphs

    def solve():
        x.zero_()
        return s.cg(b, x, sign=1, reltol=1e-10, maxiter=200000)

    ms, r = event_time(solve, steps)
    out = {"n": n, "iters": r.iters, "converged": r.converged, "ms_per_solve": round(ms, 2),
           "us_per_iteration": round(1e3 * ms / max(r.iters, 1), 2),
           "true_rel_residual": true_rel_residual(lib, x, b, n), "reltol": 1e-10,
           "launches_per_solve": s.last_launches}
    s.close()
    return out


def part_n8193(dev, warmup=1, steps=3):
    """Config 3: N = 8193 bump/trig problem, mixed and FP64 MGCG to 1e-10."""
    import sc_2022_gb300 as sbp
    import torch
    from sc_2022_gb300 import _lib, problems
    lib = sbp.load_library()
    n = 8193
    f, g = problems.bump_problem(n, seed=3)
    b = problems.assemble_rhs(f, g, device=dev).reshape(-1)
    del f
    out = {"n": n, "problem": "8 Gaussian bumps + 6-mode trig boundary data, seed 3"}
    xs = {}
    for tag, prec in (("mixed", _lib.SBP_PREC_MIXED), ("fp64", _lib.SBP_PREC_FP64)):
        s = sbp.Solver(n, sbp.default_options(prec))
        x = torch.zeros_like(b)

        def solve():
            x.zero_()
            return s.mgcg(b, x, reltol=1e-10)

        ms, r = event_time(solve, steps, warmup=warmup)
        out[f"{tag}_ms"] = round(ms, 3)
        out[f"{tag}_iters"] = r.iters
        out[f"{tag}_true_rel_residual"] = true_rel_residual(lib, x, b, n)
        xs[tag] = x
        s.close()
    out["mixed_speedup_vs_fp64"] = round(out["fp64_ms"] / out["mixed_ms"], 3)
    out["mixed_vs_fp64_solution_rel_diff"] = ((xs["mixed"] - xs["fp64"]).norm() /
                                              xs["fp64"].norm()).item()
    return out


def part_batch(dev, warmup=1, steps=2):
    """Config 4: 256 problems, N log-uniform over {65..1025}, bump/trig data,
    FP64 MGCG to 1e-10: batched vs one solve at a time."""
    import sc_2022_gb300 as sbp
    import torch
    from sc_2022_gb300 import problems
    ns, bs = problems.batch_problems(256, seed=4, device=dev)
    opts = sbp.default_options()
    B = sbp.BatchSolver(ns, opts)
    xs = [torch.zeros_like(b) for b in bs]
    t0 = time.perf_counter()
    budgets = B.autotune(bs, xs)
    tune_s = time.perf_counter() - t0
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
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            r = fn()
        torch.cuda.synchronize()
        res[name + "_ms"] = round(1e3 * (time.perf_counter() - t0) / steps, 3)
        res[name + "_iters"] = sum(x.iters for x in r)
        res[name + "_all_converged"] = all(x.converged for x in r)
    res.update({"problems": len(ns), "sizes": {str(m): ns.count(m) for m in sorted(set(ns))},
                "speedup": round(res["sequential_ms"] / res["batched_ms"], 3),
                "launches_batched": B.last_launches, "autotune": budgets,
                "autotune_s": round(tune_s, 2), "timing": "host wall clock around synchronised "
                "solves (the batch spans several streams)"})
    B.close()
    for s in solvers.values():
        s.close()
    return res


def part_adjoint(n, dev, warmup=1, steps=2):
    """Config 5: gradient of L = sum_k 1/2 (u_k - t_k)' H~ (u_k - t_k) with
    respect to the 16 sources and boundary data through torch autograd:
    forward MGCG solves, the H-misfit, the adjoint MGCG solves and the
    transposed right-hand-side map, all to 1e-10."""
    import numpy as np
    import sc_2022_gb300 as sbp
    import torch
    from sc_2022_gb300 import _lib, problems
    from sc_2022_gb300 import adjoint as adj
    B = 16
    fs, gs = [], {side: [] for side in "WESN"}
    for k in range(B):
        f, g = problems.bump_problem(n, 5000 + k)
        fs.append(np.asarray(f).reshape(n, n))
        for side in "WESN":
            gs[side].append(np.asarray(g[side]))
    f0 = torch.tensor(np.stack(fs), dtype=torch.float64, device=dev)
    g0 = [torch.tensor(np.stack(gs[side]), dtype=torch.float64, device=dev) for side in "WESN"]
    targets = 1e-3 * torch.randn((B, n, n), dtype=torch.float64, device=dev,
                                 generator=torch.Generator(device=dev).manual_seed(3))
    out = {"n": n, "batch": B, "reltol": 1e-10}
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

        for _ in range(warmup):
            gradient()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            loss, df = gradient()
        torch.cuda.synchronize()
        out[f"{tag}_ms_per_gradient"] = round(1e3 * (time.perf_counter() - t0) / steps, 2)
        out[f"{tag}_loss"] = float(loss.detach())
        grads[tag] = df.detach().clone()
        s.close()
    out["mixed_vs_fp64_df_rel_diff"] = float((grads["mixed"] - grads["fp64"]).norm() /
                                             grads["fp64"].norm())
    return out


def part_high_order(n, dev, warmup=1, steps=3):
    """p = 4 and p = 6 operators: the FP64 apply (16 B per point moved) and
    MGCG to 1e-10 from zero on a seeded random right-hand side."""
    import sc_2022_gb300 as sbp
    import torch
    from sc_2022_gb300 import _lib
    out = {"n": n}
    gen = torch.Generator(device=dev).manual_seed(0)
    us = [torch.randn(n * n, generator=gen, device=dev, dtype=torch.float64) for _ in range(2)]
    outs = [torch.empty_like(us[0]) for _ in range(2)]
    hbm, _ = measured_peaks()
    for p in (4, 6):
        k = [0]

        def app():
            sbp.matrix_free_A_high_order_GPU(us[k[0] % 2], outs[k[0] % 2], p=p)
            k[0] += 1

        ms, _ = event_time(app, 10 * steps, warmup=warmup)
        out[f"p{p}_apply_us"] = round(1e3 * ms, 2)
        out[f"p{p}_apply_frac_of_hbm"] = round(16.0 * n * n / (ms * 1e-3) / 1e9 / hbm, 3)
        for tag, prec in (("fp64", _lib.SBP_PREC_FP64), ("mixed", _lib.SBP_PREC_MIXED)):
            s = sbp.HighOrderSolver(n, p, sbp.default_options(prec))
            x = torch.zeros_like(us[0])

            def solve():
                x.zero_()
                return s.mgcg(us[0], x, reltol=1e-10, maxiter=200)

            ms, r = event_time(solve, steps, warmup=warmup)
            out[f"p{p}_mgcg_{tag}_ms"] = round(ms, 3)
            out[f"p{p}_mgcg_{tag}_iters"] = r.iters
            out[f"p{p}_mgcg_{tag}_converged"] = r.converged
            s.close()
    return out


def part_variable(n, dev, warmup=1, steps=3):
    """div(c grad u) with the seeded layered coefficient (c from 1 to 10
    across y = 1/2): the FP64 apply from nodal c (u, c read, out written:
    24 B per point) and MGCG to 1e-10 from zero."""
    import sc_2022_gb300 as sbp
    import torch
    from sc_2022_gb300 import _lib
    out = {"n": n, "coefficient": "layered 1..10"}
    x1 = torch.linspace(0.0, 1.0, n, device=dev, dtype=torch.float64)
    coef = (1.0 + 4.5 * (1.0 + torch.tanh((x1 - 0.5) * (n - 1) / 2.0)))[:, None].expand(
        n, n).contiguous().reshape(-1)
    gen = torch.Generator(device=dev).manual_seed(0)
    us = [torch.randn(n * n, generator=gen, device=dev, dtype=torch.float64) for _ in range(2)]
    outs = [torch.empty_like(us[0]) for _ in range(2)]
    hbm, _ = measured_peaks()
    k = [0]

    def app():
        sbp.matrix_free_A_variable_GPU(us[k[0] % 2], coef, outs[k[0] % 2])
        k[0] += 1

    ms, _ = event_time(app, 10 * steps, warmup=warmup)
    out.update({"apply_us": round(1e3 * ms, 2),
                "apply_frac_of_hbm": round(24.0 * n * n / (ms * 1e-3) / 1e9 / hbm, 3)})
    for tag, prec in (("fp64", _lib.SBP_PREC_FP64), ("mixed", _lib.SBP_PREC_MIXED)):
        s = sbp.VariableCoefficientSolver(n, coef, sbp.default_options(prec))
        x = torch.zeros_like(us[0])

        def solve():
            x.zero_()
            return s.mgcg(us[0], x, reltol=1e-10, maxiter=200)

        ms, r = event_time(solve, steps, warmup=warmup)
        out[f"mgcg_{tag}_ms"] = round(ms, 3)
        out[f"mgcg_{tag}_iters"] = r.iters
        out[f"mgcg_{tag}_converged"] = r.converged
        out["levels"] = s.levels
        s.close()
    return out


def part_spmv(n, dev, warmup=3, steps=20):
    """The reference's matrix-free vs assembled-SpMV comparison at n: FP64
    y = A x with this project's CSR SpMV and with the matrix-free apply."""
    import ctypes as C
    import sc_2022_gb300 as sbp
    import torch
    from sc_2022_gb300 import csr
    lib = sbp.load_library()
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    A = csr.CsrOperator(n, device=dev)
    gen = torch.Generator(device=dev).manual_seed(0)
    xs = [torch.randn(n * n, generator=gen, device=dev, dtype=torch.float64) for _ in range(2)]
    ys = [torch.empty_like(xs[0]) for _ in range(2)]
    out = {"n": n, "nnz": A.nnz}
    k = [0]

    def run_spmv():
        A.matvec(xs[k[0] % 2], ys[k[0] % 2])
        k[0] += 1

    def run_mf():
        assert lib.sbp_apply_f64(C.c_void_p(xs[k[0] % 2].data_ptr()),
                                 C.c_void_p(ys[k[0] % 2].data_ptr()), n, 1, sp) == 0
        k[0] += 1

    for name, fn, nbytes in (("spmv", run_spmv, A.device_bytes + 16 * n * n),
                             ("matrix_free", run_mf, 16 * n * n)):
        ms, _ = event_time(fn, steps, warmup=warmup)
        out[name + "_us"] = round(1e3 * ms, 2)
        out[name + "_gbs"] = round(nbytes / (ms * 1e-3) / 1e9, 1)
    out["matrix_free_speedup"] = round(out["spmv_us"] / out["matrix_free_us"], 3)
    del A
    return out


def part_profile(s, b, x, n):
    """Per-kernel times of one mixed solve (uncaptured, CUDA events around
    every launch) and the roofline of the dominant kernel."""
    res, rows = s.profile(b, x, kind="mgcg", reltol=1e-10)
    tot = sum(r["total_ms"] for r in rows)
    kernels = [{"kernel": short_name(r["kernel"]), "launches": r["launches"],
                "us_per_launch": round(1e3 * r["ms_per_launch"], 2),
                "share": round(r["total_ms"] / tot, 4)} for r in rows[:10]]
    top = rows[0]
    bpp = None
    for key, v in KERNEL_BYTES_PER_POINT.items():
        if key in top["kernel"]:
            bpp = v
            break
    points = n * n
    for key, fn in KERNEL_POINTS.items():
        if key in top["kernel"]:
            points = fn(n)
    top = dict(top, points=points)
    return res, rows, kernels, top, bpp, tot


def fp64_rate(lib):
    import ctypes as C
    import torch
    g = C.c_double()
    rc = lib.sbp_fp64_fma_rate(C.byref(g), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return g.value if rc == 0 else None


# ---------------------------------------------------------------------------
def run_ours(args, d: Dist):
    import numpy as np
    import torch

    import sc_2022_gb300 as sbp
    from sc_2022_gb300 import _lib, problems

    torch.cuda.set_device(d.local)
    dev = torch.device("cuda", d.local)
    n = args.n
    f, g, U = problems.manufactured(n, "baseline")
    b = problems.assemble_rhs(f, g, device=dev).reshape(-1)
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
    # operator applies (two inputs alternated: 4 x 134 MB > L2 for FP64)
    ms_apply = d.max(apply_timing(n, "f64", args.apply_iters, dev))
    ms_apply32 = d.max(apply_timing(n, "f32", args.apply_iters, dev))
    clocks = sampler.stop()
    ms32 = d.max(ms32)
    ms64 = d.max(ms64)
    ms_e2e = d.max(ms_e2e)

    # per-kernel times of one mixed solve and the dominant kernel's roofline
    xp = torch.zeros_like(b)
    rp, prof_rows, kernels, top, bpp, prof_total = part_profile(s32, b, xp, n)
    del xp

    rel32, rel64 = true_rel_residual(lib, x32, b, n), true_rel_residual(lib, x64, b, n)
    err_vs_fp64 = ((x32 - x64).norm() / x64.norm()).item()

    peak, peak_kind = measured_peaks()
    gfma = fp64_rate(lib)
    apply_bytes = 16.0 * n * n
    achieved64 = apply_bytes / (ms_apply * 1e-3) / 1e9
    achieved32 = 8.0 * n * n / (ms_apply32 * 1e-3) / 1e9
    top_ms = top["ms_per_launch"]
    roof = {"kernel": short_name(top["kernel"]), "bound": "hbm", "peak": peak, "unit": "GB/s",
            "peak_kind": peak_kind, "traffic": None,
            "ms_per_launch": round(top_ms, 5), "launches_per_solve": top["launches"],
            "share_of_solve": round(top["total_ms"] / prof_total, 4),
            "timing": "CUDA events around each launch of one mixed solve launched without "
                      "graphs (sbp_solver_profile), on the launching stream"}
    if bpp is not None:
        achieved = bpp * top["points"] / (top_ms * 1e-3) / 1e9
        roof.update({"achieved": round(achieved, 1), "frac": round(achieved / peak, 4),
                     "algorithmic_bytes_per_launch": bpp * top["points"],
                     "bytes_per_point": bpp, "points_per_launch": top["points"]})
    line = {
        "metric": METRIC, "value": round(ms32, 4), "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms32, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (manufactured solution u=sin(pi x)cos(pi y), b resident in HBM)",
        "config": config_block(args, n),
        "fp64_ms_per_solve": round(ms64, 4),
        "mixed_speedup_vs_fp64": round(ms64 / ms32, 3),
        "solves_per_s_all_gpus": round(args.gpus * 1e3 / ms32, 2),
        "e2e": {"value": round(ms_e2e, 4), "unit": "ms", "h2d_bytes_per_step": 8 * n * n,
                "d2h_bytes_per_step": 8 * n * n, "path": "sbp_mgcg_solve (mixed) with pinned "
                "host b/x copied in and out every step"},
        "roofline": roof,
        "solve_kernels": kernels,
        "apply_f32": {"kernel": "sbp_apply_f32 (operator apply, FP32, caller layout)",
                      "achieved_gbs": round(achieved32, 1), "frac": round(achieved32 / peak, 4),
                      "peak": peak, "algorithmic_bytes_per_launch": 8.0 * n * n,
                      "ms_per_launch": round(ms_apply32, 5)},
        "apply_f64": {"kernel": "sbp_apply_f64 (operator apply, FP64, caller layout)",
                      "achieved_gbs": round(achieved64, 1), "frac": round(achieved64 / peak, 4),
                      "peak": peak, "algorithmic_bytes_per_launch": apply_bytes,
                      "ms_per_launch": round(ms_apply, 5),
                      "fp64_pipe": None if not gfma else {
                          "ops_per_point": 4,
                          "achieved_gops": round(4.0 * n * n / (ms_apply * 1e-3) / 1e9, 1),
                          "peak_gops": round(gfma, 1),
                          "frac": round(4.0 * n * n / (ms_apply * 1e-3) / 1e9 / gfma, 4),
                          "peak_kind": "measured (sbp_fp64_fma_rate, this run)",
                          "note": "4 = the stencil's minimum FP64 operations per point (3 adds, "
                                  "1 FMA); half the warps form the sum exactly on the integer "
                                  "pipe instead, so the FP64-equivalent rate can exceed the "
                                  "FP64 pipe's own"}},
        "clocks": clocks,
        "gpu_launches": int(launches32 * args.steps),
        "detail": {"iters_mixed": r32.iters, "iters_fp64": r64.iters,
                   "true_rel_residual_mixed": rel32, "true_rel_residual_fp64": rel64,
                   "mixed_vs_fp64_solution_rel_diff": err_vs_fp64,
                   "launches_per_solve": launches32,
                   "profiled_solve_iters": rp.iters,
                   "profiled_solve_kernel_ms": round(prof_total, 3),
                   "device_bytes": s32.device_bytes + s64.device_bytes},
    }
    s32.close()
    s64.close()
    if d.rank == 0 and args.cpu_baseline:
        bh = b.detach().cpu().numpy()
        r = cpu_mgcg_timing(n, bh, steps=3, warmup=1)
        xo = r.pop("x")
        # the oracle pin: the GPU solutions against the C oracle's FP64 solve
        line["detail"]["oracle_iters"] = r["iters"]
        on = float(np.linalg.norm(xo))
        line["detail"]["fp64_vs_oracle_rel"] = float(
            np.linalg.norm(x64.cpu().numpy() - xo) / on)
        line["detail"]["mixed_vs_oracle_rel"] = float(
            np.linalg.norm(x32.cpu().numpy() - xo) / on)
        r1 = cpu_mgcg_timing(n, bh, steps=1, warmup=0, threads=1)
        r1.pop("x")
        line["cpu_baseline"] = {
            "value": round(r["ms_per_solve"], 2), "unit": "ms", "cores": r["threads"],
            "kind": "port", "sample": cpu_sample_text(r, n),
            "value_1_core": round(r1["ms_per_solve"], 2)}
    if d.rank == 0 and args.extras and d.world == 1:
        extras = {}
        for name, fn in (("cg_fp64", lambda: part_cg(n, dev)),
                         ("n8193", lambda: part_n8193(dev)),
                         ("batch256", lambda: part_batch(dev)),
                         ("adjoint_2049x16", lambda: part_adjoint(2049, dev)),
                         ("high_order", lambda: part_high_order(n, dev)),
                         ("variable", lambda: part_variable(n, dev)),
                         ("spmv", lambda: part_spmv(n, dev))):
            t0 = time.perf_counter()
            try:
                extras[name] = fn()
            except Exception as exc:   # one failing extra must not lose the line
                extras[name] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
                traceback.print_exc(file=sys.stderr)
            extras[name]["wall_s"] = round(time.perf_counter() - t0, 1)
            torch.cuda.empty_cache()
        line["cg_fp64"] = extras.pop("cg_fp64")
        line["configs"] = extras
    if d.rank == 0:
        print(json.dumps(line), flush=True)


def run_part(args):
    """Profiling helper: one part of the benchmark on a single GPU."""
    import torch

    import sc_2022_gb300 as sbp
    from sc_2022_gb300 import _lib, problems
    n = args.n
    dev = torch.device("cuda", 0)
    lib = sbp.load_library()
    if args.mode == "apply":
        import ctypes as C
        sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        gen = torch.Generator(device=dev).manual_seed(0)
        dt = torch.float64 if args.dtype == "f64" else torch.float32
        fn = lib.sbp_apply_f64 if args.dtype == "f64" else lib.sbp_apply_f32
        us = [torch.randn(n * n, generator=gen, device=dev, dtype=torch.float64).to(dt)
              for _ in range(2)]
        outs = [torch.empty_like(us[0]) for _ in range(2)]
        for k in range(args.warmup + args.steps):
            rc = fn(C.c_void_p(us[k % 2].data_ptr()), C.c_void_p(outs[k % 2].data_ptr()), n, -1, sp)
            assert rc == 0
        torch.cuda.synchronize()
        print(json.dumps({"mode": "apply", "dtype": args.dtype, "n": n,
                          "launches": args.warmup + args.steps,
                          "us_per_launch_timed": round(
                              1e3 * apply_timing(n, args.dtype, max(args.steps, 1), dev), 2)}))
        return
    if args.mode == "cg":
        print(json.dumps({"mode": "cg", **part_cg(n, dev, steps=max(args.steps, 1))}))
        return
    if args.mode == "n8193":
        print(json.dumps({"mode": "n8193", **part_n8193(dev, args.warmup, max(args.steps, 1))}))
        return
    if args.mode == "spmv":
        print(json.dumps({"mode": "spmv", **part_spmv(n, dev, args.warmup, max(args.steps, 1))}))
        return
    if args.mode == "batch":
        print(json.dumps({"mode": "batch", **part_batch(dev, args.warmup, max(args.steps, 1))}))
        return
    if args.mode == "high-order":
        print(json.dumps({"mode": "high-order",
                          **part_high_order(n, dev, args.warmup, max(args.steps, 1))}))
        return
    if args.mode == "variable":
        print(json.dumps({"mode": "variable",
                          **part_variable(n, dev, args.warmup, max(args.steps, 1))}))
        return
    if args.mode == "adjoint":
        print(json.dumps({"mode": "adjoint",
                          **part_adjoint(n, dev, args.warmup, max(args.steps, 1))}))
        return
    if args.mode == "profile":
        f, g, _ = problems.manufactured(n, "baseline")
        b = problems.assemble_rhs(f, g, device=dev).reshape(-1)
        out = {"mode": "profile", "n": n}
        for tag, prec in (("mixed", _lib.SBP_PREC_MIXED), ("fp64", _lib.SBP_PREC_FP64)):
            s = sbp.Solver(n, sbp.default_options(prec))
            x = torch.zeros_like(b)
            s.mgcg(b, x, reltol=1e-10)
            x.zero_()
            res, rows, kernels, top, bpp, tot = part_profile(s, b, x, n)
            out[tag] = {"iters": res.iters, "kernel_ms": round(tot, 3), "kernels": kernels}
            s.close()
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
            ms, _ = event_time(lambda: s.vcycle(b, v), max(args.steps, 1), warmup=args.warmup)
            out[name + "_us"] = round(1e3 * ms, 2)
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
